// iqs_gb300/qureg.hpp -- header-only iqs::QubitRegister<Type> over libiqsg (include/iqsg.h).
//
// Drop-in for the gate-application path of intel-qs' class of the same name
// (include/qureg.hpp:127-417): same namespace, class template, method names and argument
// types (program-qubit indices as unsigned, TM2x2 / TM4x4 matrices by const reference,
// angles as BaseType). The state lives in GPU memory. This header keeps the program-qubit ->
// position Permutation and the GateCounter on the host and forwards every operation to one
// C-ABI call. Where the reference asserts, these methods throw std::invalid_argument; CUDA
// failures throw std::runtime_error.
//
// Differences a caller can observe: operator[] returns a proxy that reads or writes one
// amplitude in device memory (a copy per access), and RawState() returns the device address.
#pragma once

#include <algorithm>
#include <cstdio>
#include <cmath>
#include <complex>
#include <cstring>
#include <memory>
#include <numeric>
#include <ostream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../iqsg.h"
#include "tinymatrix.hpp"
#include "utils.hpp"
#include "mpi_env.hpp"
#include "permutation.hpp"
#include "noise.hpp"

using ComplexSP = std::complex<float>;
using ComplexDP = std::complex<double>;

namespace iqs {

inline void check_status(int st) {
  if (st == IQSG_OK) return;
  if (st == IQSG_EINVAL) throw std::invalid_argument(iqsg_last_error());
  throw std::runtime_error(iqsg_last_error());
}

template <class Type> struct extract_value_type;
template <> struct extract_value_type<ComplexDP> { using value_type = double; };
template <> struct extract_value_type<ComplexSP> { using value_type = float; };


template <class Type = ComplexDP>
class QubitRegister {
 public:
  using value_type = Type;
  using BaseType = typename extract_value_type<Type>::value_type;

  // Reads / writes one amplitude of device memory (operator[] of the reference).
  class Amplitude {
   public:
    Amplitude(QubitRegister* r, std::size_t i) : r_(r), i_(i) {}
    operator Type() const { return r_->read(i_); }
    Amplitude& operator=(const Type& v) { r_->write(i_, v); return *this; }
    Amplitude& operator=(const Amplitude& o) { return *this = Type(o); }
    Type real_imag() const { return Type(*this); }
    BaseType real() const { return Type(*this).real(); }
    BaseType imag() const { return Type(*this).imag(); }
    // Arithmetic as on the Type& the reference returns (std::complex's operators are templates
    // and do not see the conversion): each read or write is one amplitude copy.
    Amplitude& operator+=(const Type& v) { return *this = Type(*this) + v; }
    Amplitude& operator-=(const Type& v) { return *this = Type(*this) - v; }
    Amplitude& operator*=(const Type& v) { return *this = Type(*this) * v; }
    Amplitude& operator/=(const Type& v) { return *this = Type(*this) / v; }
    Amplitude& operator*=(BaseType v) { return *this = Type(*this) * v; }
    Amplitude& operator/=(BaseType v) { return *this = Type(*this) / v; }
    Type operator-() const { return -Type(*this); }
    Type operator+() const { return Type(*this); }
    friend Type operator+(const Amplitude& a, const Type& b) { return Type(a) + b; }
    friend Type operator+(const Type& a, const Amplitude& b) { return a + Type(b); }
    friend Type operator+(const Amplitude& a, const Amplitude& b) { return Type(a) + Type(b); }
    friend Type operator-(const Amplitude& a, const Type& b) { return Type(a) - b; }
    friend Type operator-(const Type& a, const Amplitude& b) { return a - Type(b); }
    friend Type operator-(const Amplitude& a, const Amplitude& b) { return Type(a) - Type(b); }
    friend Type operator*(const Amplitude& a, const Type& b) { return Type(a) * b; }
    friend Type operator*(const Type& a, const Amplitude& b) { return a * Type(b); }
    friend Type operator*(const Amplitude& a, const Amplitude& b) { return Type(a) * Type(b); }
    friend Type operator*(const Amplitude& a, BaseType b) { return Type(a) * b; }
    friend Type operator*(BaseType a, const Amplitude& b) { return a * Type(b); }
    friend Type operator/(const Amplitude& a, const Type& b) { return Type(a) / b; }
    friend Type operator/(const Amplitude& a, BaseType b) { return Type(a) / b; }
    friend bool operator==(const Amplitude& a, const Type& b) { return Type(a) == b; }
    friend bool operator!=(const Amplitude& a, const Type& b) { return Type(a) != b; }
    friend std::ostream& operator<<(std::ostream& os, const Amplitude& a) { return os << Type(a); }
    friend BaseType abs(const Amplitude& a) { return std::abs(Type(a)); }
    friend BaseType norm(const Amplitude& a) { return std::norm(Type(a)); }
    friend Type conj(const Amplitude& a) { return std::conj(Type(a)); }

   private:
    QubitRegister* r_;
    std::size_t i_;
  };

  QubitRegister() : QubitRegister(1, "base", 0) {}
  QubitRegister(std::size_t num_qubits, std::string style = "", std::size_t base_index = 0,
                std::size_t /*tmp_spacesize*/ = 0)
      : num_qubits(num_qubits), n_((unsigned)num_qubits), perm_(num_qubits) {
    check_status(iqsg_create(n_, kPrec, nullptr, &h_));
    Initialize(style, base_index);
  }
  // Imported state: the device memory at state is used in place and not freed.
  QubitRegister(std::size_t num_qubits, Type* device_state, std::size_t /*tmp_spacesize*/ = 0)
      : num_qubits(num_qubits), imported_state(true), n_((unsigned)num_qubits), perm_(num_qubits) {
    check_status(iqsg_create_from_device(n_, kPrec, device_state, nullptr, &h_));
  }
  QubitRegister(const QubitRegister& in) : num_qubits(in.num_qubits), n_(in.n_), perm_(in.perm_), fusion_(false) {
    const_cast<QubitRegister&>(in).ApplyFusedGates();
    check_status(iqsg_clone(in.h_, &h_));
  }
  QubitRegister& operator=(const QubitRegister&) = delete;
  ~QubitRegister() {
    delete gate_counter;
    iqsg_destroy(h_);
  }

  // Public members of the reference's class (include/qureg.hpp:382-393) that callers and
  // subclasses use: the size, the program-qubit map, the gate counter (null unless statistics
  // are enabled) and whether the state memory belongs to the caller.
  std::size_t num_qubits = 0;
  Permutation* qubit_permutation = &perm_;
  GateCounter* gate_counter = nullptr;
  bool imported_state = false;

  // ---- information and access ----
  std::size_t NumQubits() const { return n_; }
  std::size_t LocalSize() const { return std::size_t(1) << n_; }
  std::size_t GlobalSize() const { return std::size_t(1) << n_; }
  std::size_t size() const { return GlobalSize(); }
  Type* RawState() {
    ApplyFusedGates();
    void* p = nullptr;
    check_status(iqsg_info(h_, nullptr, nullptr, &p));
    return static_cast<Type*>(p);
  }
  Amplitude operator[](std::size_t index) { return Amplitude(this, index); }
  Type GetGlobalAmplitude(std::size_t index) { return read(perm_.program2data_(check_index(index))); }
  void SetGlobalAmplitude(std::size_t index, Type value) { write(perm_.program2data_(check_index(index)), value); }
  void SetMath(int math) { ApplyFusedGates(); check_status(iqsg_set_math(h_, math)); }
  iqsg_state* handle() { return h_; }
  Permutation* qubit_permutation_ptr() { return &perm_; }
  const std::vector<std::size_t>& QubitMap() const { return perm_.map; }

  void Initialize(const std::string& style, std::size_t base_index) {
    fwindow_.clear();
    if (style == "base") {
      check_status(iqsg_init_basis(h_, perm_.program2data_(check_index(base_index))));
    } else if (style == "++++") {
      check_status(iqsg_fill(h_, (BaseType)(1. / std::sqrt((double)GlobalSize())), 0.0));
    } else if (style.empty()) {
      check_status(iqsg_fill(h_, 0.0, 0.0));
    } else if (style == "rand") {
      // src/qureg_init.cpp:256-333: uniform real and imaginary parts in [-1, 1) from the "pool"
      // stream (base_index 0) or the "local" one (base_index = number of states = 1), normalised.
      if (!rng_ptr_) throw std::invalid_argument("Initialize(\"rand\"): SetRngPtr first");
      if (base_index > 1) throw std::invalid_argument("Initialize(\"rand\"): base_index must be 0 or 1");
      check_status(iqsg_init_random(h_, rng_ptr_->handle(), base_index == 0 ? 0 : 2));
      Normalize();
    } else {
      throw std::invalid_argument("Initialize: style must be \"base\", \"++++\", \"rand\" or \"\"");
    }
  }

  // ---- random number generator (include/qureg.hpp:375-379) ----
  RandomNumberGenerator<BaseType>* GetRngPtr() { return rng_ptr_; }
  void ResetRngPtr() { rng_ptr_ = nullptr; }
  void SetRngPtr(RandomNumberGenerator<BaseType>* rng_ptr) { rng_ptr_ = rng_ptr; }
  void SetSeedRngPtr(std::size_t seed) {
    if (!rng_ptr_) throw std::invalid_argument("SetSeedRngPtr: no RandomNumberGenerator set");
    rng_ptr_->SetSeedStreamPtrs(seed);
  }

  // ---- noise (src/qureg_noisysimul.cpp, src/qureg_apply_channel.cpp) ----
  BaseType GetT1() { return T_1_; }
  BaseType GetT2() { return T_2_; }
  BaseType GetTphi() { return T_phi_; }
  void SetNoiseTimescales(BaseType T1, BaseType T2) {
    if (!(T2 >= T1 / 2.)) throw std::invalid_argument("SetNoiseTimescales: T2 must be at least T1/2");
    T_1_ = T1;
    T_2_ = T2;
    T_phi_ = 1. / (1. / T2 - 1. / (2. * T1));
  }
  // Pauli-twirl noise for `duration` (three Gaussian angles from the "state" stream, one gate).
  void ApplyNoiseGate(const unsigned qubit, const BaseType duration) {
    if (!rng_ptr_) throw std::invalid_argument("ApplyNoiseGate: SetRngPtr first");
    if (duration == 0) return;
    double m[8];
    check_status(iqsg_noise_gate_draw(rng_ptr_->handle(), kPrec, T_1_, T_2_, duration, m));
    QubitRegister::Apply1QubitGate(qubit, mat2(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7]));
  }
  // One eigenvector of chi, drawn from the "state" stream, applied as a gate; a negative
  // eigenvalue flips the overall sign.
  void ApplyChannel(const unsigned qubit, CM4x4<Type>& chi) {
    double g[8];
    channel_draw(4, chi, g);
    QubitRegister::Apply1QubitGate(qubit, mat2(g[0], g[1], g[2], g[3], g[4], g[5], g[6], g[7]));
  }
  void ApplyChannel(const unsigned qubit1, const unsigned qubit2, CM16x16<Type>& chi) {
    double g[32];
    channel_draw(16, chi, g);
    TM4x4<Type> m;
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) m(r, c) = Type((BaseType)g[2 * (4 * r + c)], (BaseType)g[2 * (4 * r + c) + 1]);
    QubitRegister::Apply2QubitGate(qubit1, qubit2, m);
  }
  BaseType GetOverallSignOfChannels() { return overall_sign_of_channels; }
  void InitializationWithSameAmplitudeEverywhere(Type a) {
    ApplyFusedGates();
    check_status(iqsg_fill(h_, a.real(), a.imag()));
  }

  // ---- statistics ----
  void EnableStatistics() {
    delete gate_counter;
    gate_counter = new GateCounter((int)n_);
  }
  void DisableStatistics() {
    delete gate_counter;
    gate_counter = nullptr;
  }
  void ResetStatistics() {
    DisableStatistics();
    EnableStatistics();
  }
  // The gate counter's breakdown (the reference also prints its timer, which is not kept here).
  void GetStatistics() {
    if (!gate_counter) throw std::invalid_argument("GetStatistics: statistics are not enabled");
    gate_counter->Breakdown();
  }
  GateCounter* GetGateCounter() { return gate_counter; }

  // ---- fusion ----
  void TurnOnFusion(unsigned log2llc = 20) { fusion_ = true; log2llc_ = log2llc; }
  void TurnOffFusion() { ApplyFusedGates(); fusion_ = false; }
  bool IsFusionEnabled() { return fusion_; }
  void ApplyFusedGates() {
    if (fwindow_.empty()) return;
    std::vector<iqsg_op> ops;
    ops.swap(fwindow_);
    check_status(iqsg_apply_ops(h_, ops.data(), (unsigned)ops.size(), nullptr));
  }
  void TurnOnSpecialize() {}
  void TurnOffSpecialize() {}
  void TurnOnSpecializeV2() {}
  void TurnOffSpecializeV2() {}

  // ---- generic gates ----
  void Apply1QubitGate(unsigned qubit, const TM2x2<Type>& m) {
    const unsigned p = pos(qubit);
    if (gate_counter) gate_counter->OneQubitIncrement((int)qubit);
    iqsg_op op = make(IQSG_OP_1Q, p, 0, m8(m).data(), 8);
    if (fusion_) return queue(op);
    check_status(iqsg_apply_1q(h_, p, op.m));
  }
  void ApplyControlled1QubitGate(unsigned control, unsigned target, const TM2x2<Type>& m) {
    const unsigned pc = pos(control), pt = pos(target);
    if (control == target) throw std::invalid_argument("ApplyControlled1QubitGate: control == target");
    if (gate_counter) gate_counter->TwoQubitIncrement((int)control, (int)target);
    iqsg_op op = make(IQSG_OP_CTRL, pt, 0, m8(m).data(), 8);
    op.nctrl = 1;
    op.ctrl[0] = pc;
    if (fusion_) return queue(op);
    check_status(iqsg_apply_controlled_1q(h_, pc, pt, op.m));
  }
  void Apply2QubitGate(unsigned qubit_high, unsigned qubit_low, const TM4x4<Type>& m) {
    const unsigned ph = pos(qubit_high), pl = pos(qubit_low);
    if (qubit_high == qubit_low) throw std::invalid_argument("Apply2QubitGate: qubits coincide");
    double d[32];
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) { d[2 * (4 * r + c)] = (double)m(r, c).real(); d[2 * (4 * r + c) + 1] = (double)m(r, c).imag(); }
    iqsg_op op = make(IQSG_OP_2Q, ph, pl, d, 32);
    if (fusion_) queue(op);
    else check_status(iqsg_apply_2q(h_, ph, pl, op.m));
    if (gate_counter) gate_counter->TwoQubitIncrement((int)qubit_high, (int)qubit_low);
  }
  void ApplyDiag(unsigned qubit_1, unsigned qubit_2, const TM4x4<Type>& m) {
    const unsigned p1 = pos(qubit_1), p2 = pos(qubit_2);
    if (qubit_1 == qubit_2) throw std::invalid_argument("ApplyDiag: qubits coincide");
    if (gate_counter) gate_counter->TwoQubitIncrement((int)qubit_1, (int)qubit_2);
    double d[8];
    for (int k = 0; k < 4; ++k) { d[2 * k] = (double)m(k, k).real(); d[2 * k + 1] = (double)m(k, k).imag(); }
    iqsg_op op = make(IQSG_OP_DIAG2, p1, p2, d, 8);
    if (fusion_) return queue(op);
    check_status(iqsg_apply_diag_2q(h_, p1, p2, op.m));
  }

  // The same diagonal as ApplyDiag, not counted as a gate (src/qureg_applydiag.cpp:17-51).
  void ApplyDiagSimp(unsigned qubit_1, unsigned qubit_2, const TM4x4<Type>& m) {
    GateCounter* keep = gate_counter;
    gate_counter = nullptr;
    try {
      ApplyDiag(qubit_1, qubit_2, m);
    } catch (...) {
      gate_counter = keep;
      throw;
    }
    gate_counter = keep;
  }

  // ---- named one-qubit gates (src/qureg_apply1qubitgate.cpp:277-501) ----
  void ApplyRotationX(unsigned q, BaseType t) {
    TM2x2<Type> m;
    m(0, 1) = m(1, 0) = Type(0, -std::sin(t / 2.));
    m(0, 0) = m(1, 1) = Type(std::cos(t / 2.), 0);
    Apply1QubitGate(q, m);
  }
  void ApplyRotationY(unsigned q, BaseType t) {
    TM2x2<Type> m;
    m(0, 1) = Type(-std::sin(t / 2.), 0.);
    m(1, 0) = Type(std::sin(t / 2.), 0.);
    m(0, 0) = m(1, 1) = Type(std::cos(t / 2.), 0);
    Apply1QubitGate(q, m);
  }
  void ApplyRotationZ(unsigned q, BaseType t) {
    TM2x2<Type> m;
    m(0, 0) = Type(std::cos(t / 2.), -std::sin(t / 2.));
    m(1, 1) = Type(std::cos(t / 2.), std::sin(t / 2.));
    Apply1QubitGate(q, m);
  }
  void ApplyPauliX(unsigned q) { Apply1QubitGate(q, mat2(0, 0, 1, 0, 1, 0, 0, 0)); }
  void ApplyPauliY(unsigned q) { Apply1QubitGate(q, mat2(0, 0, 0, -1, 0, 1, 0, 0)); }
  void ApplyPauliZ(unsigned q) { Apply1QubitGate(q, mat2(1, 0, 0, 0, 0, 0, -1, 0)); }
  void ApplyPauliSqrtX(unsigned q) { Apply1QubitGate(q, mat2(.5, .5, .5, -.5, .5, -.5, .5, .5)); }
  void ApplyPauliSqrtY(unsigned q) { Apply1QubitGate(q, mat2(.5, .5, -.5, -.5, .5, .5, .5, .5)); }
  void ApplyPauliSqrtZ(unsigned q) { Apply1QubitGate(q, mat2(1, 0, 0, 0, 0, 0, 0, 1)); }
  void ApplyT(unsigned q) { Apply1QubitGate(q, mat2(1, 0, 0, 0, 0, 0, std::cos(M_PI / 4.0), std::sin(M_PI / 4.0))); }
  void ApplyHadamard(unsigned q) {
    const BaseType f = 1. / std::sqrt(2.);
    Apply1QubitGate(q, mat2(f, 0, f, 0, f, 0, -f, 0));
  }
  void ApplyRotationXY(unsigned q, BaseType phi, BaseType theta) {
    TM2x2<Type> m;
    m(0, 0) = m(1, 1) = Type(std::cos(theta / 2.), 0);
    m(0, 1) = Type(-std::sin(theta / 2.) * std::sin(phi), -std::sin(theta / 2.) * std::cos(phi));
    m(1, 0) = Type(std::sin(theta / 2.) * std::sin(phi), -std::sin(theta / 2.) * std::cos(phi));
    Apply1QubitGate(q, m);
  }

  // ---- named controlled gates (src/qureg_applyctrl1qubitgate.cpp:458-618) ----
  void ApplyCRotationX(unsigned c, unsigned q, BaseType t) {
    TM2x2<Type> m;
    m(0, 1) = m(1, 0) = Type(0, -std::sin(t / 2.));
    m(0, 0) = m(1, 1) = Type(std::cos(t / 2.), 0);
    ApplyControlled1QubitGate(c, q, m);
  }
  void ApplyCRotationY(unsigned c, unsigned q, BaseType t) {
    TM2x2<Type> m;
    m(0, 1) = Type(-std::sin(t / 2.), 0.);
    m(1, 0) = Type(std::sin(t / 2.), 0.);
    m(0, 0) = m(1, 1) = Type(std::cos(t / 2.), 0);
    ApplyControlled1QubitGate(c, q, m);
  }
  void ApplyCRotationZ(unsigned c, unsigned q, BaseType t) {
    TM2x2<Type> m;
    m(0, 0) = Type(std::cos(t / 2.), -std::sin(t / 2.));
    m(1, 1) = Type(std::cos(t / 2.), std::sin(t / 2.));
    ApplyControlled1QubitGate(c, q, m);
  }
  void ApplyCPauliX(unsigned c, unsigned q) { ApplyControlled1QubitGate(c, q, mat2(0, 0, 1, 0, 1, 0, 0, 0)); }
  void ApplyCPauliY(unsigned c, unsigned q) { ApplyControlled1QubitGate(c, q, mat2(0, 0, 0, -1, 0, 1, 0, 0)); }
  void ApplyCPauliZ(unsigned c, unsigned q) { ApplyControlled1QubitGate(c, q, mat2(1, 0, 0, 0, 0, 0, -1, 0)); }
  void ApplyCPauliSqrtZ(unsigned c, unsigned q) { ApplyControlled1QubitGate(c, q, mat2(1, 0, 0, 0, 0, 0, 0, 1)); }
  void ApplyCHadamard(unsigned c, unsigned q) {
    const BaseType f = 1. / std::sqrt(2.);
    ApplyControlled1QubitGate(c, q, mat2(f, 0, f, 0, f, 0, -f, 0));
  }
  void ApplyCPhaseRotation(unsigned c, unsigned q, BaseType t) {
    ApplyControlled1QubitGate(c, q, mat2(1, 0, 0, 0, 0, 0, std::cos(t), std::sin(t)));
  }

  // ---- swap family and Toffoli ----
  void ApplySwap(unsigned a, unsigned b) { swaplike(a, b, mat2(0, 0, 1, 0, 1, 0, 0, 0)); }
  void ApplyISwap(unsigned a, unsigned b) { swaplike(a, b, mat2(0, 0, 0, 1, 0, 1, 0, 0)); }
  void ApplySqrtISwap(unsigned a, unsigned b) {
    const BaseType f = 1. / std::sqrt(2.);
    swaplike(a, b, mat2(f, 0, 0, f, 0, f, f, 0));
  }
  void Apply4thRootISwap(unsigned a, unsigned b) {
    const auto x = std::polar(.5, M_PI / 8.), y = std::polar(.5, 7. * M_PI / 8.);
    const auto f0 = x - y, f1 = x + y;
    swaplike(a, b, mat2(f0.real(), f0.imag(), f1.real(), f1.imag(), f1.real(), f1.imag(), f0.real(), f0.imag()));
  }
  void ApplyISwapRotation(unsigned a, unsigned b, const TM2x2<Type>& m) {
    if (m(0, 1) != m(1, 0)) throw std::invalid_argument("ApplyISwapRotation: m01 must equal m10");
    swaplike(a, b, m);
  }
  void ApplyToffoli(unsigned c1, unsigned c2, unsigned t) {
    if (c1 == c2 || c1 == t || c2 == t) throw std::invalid_argument("ApplyToffoli: qubits must differ");
    const unsigned pc[2] = {pos(c1), pos(c2)};
    const unsigned pt = pos(t);
    if (gate_counter) {  // the reference's five two-qubit gates (src/qureg_applytoffoli.cpp:41-45)
      gate_counter->TwoQubitIncrement((int)c1, (int)t);
      gate_counter->TwoQubitIncrement((int)c2, (int)c1);
      gate_counter->TwoQubitIncrement((int)c1, (int)t);
      gate_counter->TwoQubitIncrement((int)c2, (int)c1);
      gate_counter->TwoQubitIncrement((int)c2, (int)t);
    }
    const double x[8] = {0, 0, 1, 0, 1, 0, 0, 0};
    iqsg_op op = make(IQSG_OP_CTRL, pt, 0, x, 8);
    op.nctrl = 2;
    op.ctrl[0] = pc[0];
    op.ctrl[1] = pc[1];
    if (fusion_) return queue(op);
    check_status(iqsg_apply_multi_controlled_1q(h_, 2, pc, pt, x));
  }

  // ---- permutation ----
  void PermuteQubits(std::vector<std::size_t> new_map, std::string style_of_map = "direct") {
    if (new_map.size() != n_) throw std::invalid_argument("PermuteQubits: map size differs from the qubit count");
    ApplyFusedGates();
    Permutation np(new_map, style_of_map);
    std::vector<unsigned> o(n_), m(n_);
    for (unsigned q = 0; q < n_; ++q) { o[q] = (unsigned)perm_.map[q]; m[q] = (unsigned)np.map[q]; }
    check_status(iqsg_permute(h_, o.data(), m.data()));
    perm_ = np;
  }
  // One GPU holds every qubit: local, global and pair-exchange reorders are the same reorder.
  void PermuteLocalQubits(std::vector<std::size_t> m, std::string s = "direct") { PermuteQubits(m, s); }
  void PermuteGlobalQubits(std::vector<std::size_t> m, std::string s = "direct") { PermuteQubits(m, s); }
  void PermuteByLocalGlobalExchangeOfQubitPairs(std::vector<std::size_t> m, std::string s = "direct") {
    PermuteQubits(m, s);
  }

  // Bit manipulation helpers of the reference (include/qureg.hpp:168-181).
  bool check_bit(std::size_t variable, std::size_t position) const { return (variable >> position) & 1u; }
  std::size_t set_bit(std::size_t variable, std::size_t position) const {
    return variable | (std::size_t(1) << position);
  }
  std::size_t clear_bit(std::size_t variable, std::size_t position) const {
    return variable & ~(std::size_t(1) << position);
  }
  void EmulateSwap(unsigned a, unsigned b) { pos(a); pos(b); perm_.ExchangeTwoElements(a, b); }

  // ---- measurement and expectation ----
  BaseType GetProbability(unsigned q) {
    ApplyFusedGates();
    double p = 0;
    check_status(iqsg_probability(h_, pos(q), &p));
    return (BaseType)p;
  }
  void CollapseQubit(unsigned q, bool value) {
    ApplyFusedGates();
    check_status(iqsg_collapse(h_, pos(q), value ? 1 : 0));
  }
  bool IsClassicalBit(unsigned q, BaseType tol = 1.e-13) {
    const BaseType p = GetProbability(q);
    return p < tol || std::abs(1 - p) < tol;
  }
  // The value of a classical qubit (src/qureg_measure.cpp:184-260); a qubit that is not
  // classical within the tolerance throws std::invalid_argument.
  bool GetClassicalValue(unsigned q, BaseType tol = 1.e-13) {
    const BaseType p = GetProbability(q);
    if (p < tol) return false;
    if (std::abs(1 - p) < tol) return true;
    throw std::invalid_argument("GetClassicalValue: the qubit is not classical");
  }
  BaseType ExpectationValue(std::vector<unsigned>& qubits, std::vector<unsigned>& observables, BaseType coeff = 1.) {
    if (qubits.size() != observables.size()) throw std::invalid_argument("ExpectationValue: size mismatch");
    if (qubits.empty()) return coeff;
    ApplyFusedGates();
    std::vector<unsigned> p(qubits.size());
    for (std::size_t k = 0; k < qubits.size(); ++k) p[k] = pos(qubits[k]);
    if (gate_counter)  // the reference's basis changes and their undo count as one-qubit gates
      for (std::size_t k = 0; k < qubits.size(); ++k)
        if (observables[k] == 1 || observables[k] == 2) {
          gate_counter->OneQubitIncrement((int)qubits[k]);
          gate_counter->OneQubitIncrement((int)qubits[k]);
        }
    double v = 0, n2 = 0;
    check_status(iqsg_expectation_pauli(h_, (unsigned)p.size(), p.data(), observables.data(), &v, &n2));
    const double e = qubits.size() > 1 ? v : 1.0 - n2 + v;  // single factor: 1 - 2 P(1), as the reference
    return coeff * (BaseType)e;
  }
  // ---- state statistics and formats (src/qureg_utils.cpp:303-657) ----
  std::vector<double> GoogleStats() {
    ApplyFusedGates();
    std::vector<double> v(11);
    check_status(iqsg_state_stats(h_, v.data()));
    return v;
  }
  double Entropy() { return GoogleStats()[0]; }
  void Print(std::string x, std::vector<std::size_t> /*qubits: unused, as in the reference*/ = {}) {
    const std::vector<Type> a = GetStateVector();
    BaseType cum = 0;
    std::printf("qubit permutation: %s\n", perm_.GetMapStr().c_str());
    std::printf("%s=[\n", x.c_str());
    for (std::size_t i = 0; i < a.size(); ++i) {
      std::printf("\t%-13.8lf + i * %-13.8lf   %% |%s> p=%lf\n", (double)a[i].real(), (double)a[i].imag(),
                  perm_.data2program(i).c_str(), (double)std::norm(a[i]));
      cum += std::norm(a[i]);
    }
    std::printf("]; %% cumulative probability = %lf\n", (double)cum);
  }
  void ExportAmplitudes(std::string ofname) {
    const std::vector<Type> a = GetStateVector();
    std::string body;
    char line[512];
    for (std::size_t i = 0; i < a.size(); ++i) {
      std::snprintf(line, sizeof line, "\t\t\"%s\" : [%-13.8lf, %-13.8lf, %lf],\n", perm_.data2program(i).c_str(),
                    (double)a[i].real(), (double)a[i].imag(), (double)std::norm(a[i]));
      body += line;
    }
    if (body.size() >= 2) body = body.substr(0, body.size() - 2) + "\n";
    std::FILE* f = std::fopen(ofname.c_str(), "a");
    if (!f) throw std::runtime_error("ExportAmplitudes: cannot open " + ofname);
    std::fprintf(f, "\t\"amplitudes\" :\n\t{\n%s\t}\n", body.c_str());
    std::fclose(f);
  }

  BaseType ExpectationValueX(unsigned q, BaseType c = 1.) { return ev({q}, {1}, c); }
  BaseType ExpectationValueY(unsigned q, BaseType c = 1.) { return ev({q}, {2}, c); }
  BaseType ExpectationValueZ(unsigned q, BaseType c = 1.) { return ev({q}, {3}, c); }
  BaseType ExpectationValueXX(unsigned a, unsigned b, BaseType c = 1.) { return ev({a, b}, {1, 1}, c); }
  BaseType ExpectationValueXY(unsigned a, unsigned b, BaseType c = 1.) { return ev({a, b}, {1, 2}, c); }
  BaseType ExpectationValueXZ(unsigned a, unsigned b, BaseType c = 1.) { return ev({a, b}, {1, 3}, c); }
  BaseType ExpectationValueYX(unsigned a, unsigned b, BaseType c = 1.) { return ev({a, b}, {2, 1}, c); }
  BaseType ExpectationValueYY(unsigned a, unsigned b, BaseType c = 1.) { return ev({a, b}, {2, 2}, c); }
  BaseType ExpectationValueYZ(unsigned a, unsigned b, BaseType c = 1.) { return ev({a, b}, {2, 3}, c); }
  BaseType ExpectationValueZX(unsigned a, unsigned b, BaseType c = 1.) { return ev({a, b}, {3, 1}, c); }
  BaseType ExpectationValueZY(unsigned a, unsigned b, BaseType c = 1.) { return ev({a, b}, {3, 2}, c); }
  BaseType ExpectationValueZZ(unsigned a, unsigned b, BaseType c = 1.) { return ev({a, b}, {3, 3}, c); }

  // ---- norms and amplitude-wise operations ----
  BaseType ComputeNorm() {
    ApplyFusedGates();
    double v = 0;
    check_status(iqsg_norm2(h_, &v));
    return (BaseType)std::sqrt(v);
  }
  void Normalize() { AmplitudeWiseScalarMultiplication(Type(1 / ComputeNorm(), 0)); }
  Type ComputeOverlap(QubitRegister& psi) {
    same_layout(psi);
    double o[2];
    check_status(iqsg_overlap(h_, psi.h_, o));
    return Type((BaseType)o[0], (BaseType)o[1]);
  }
  BaseType MaxAbsDiff(QubitRegister& x, Type sfactor = Type(1, 0)) {
    same_layout(x);
    double v = 0;
    check_status(iqsg_max_abs_diff(h_, x.h_, sfactor.real(), sfactor.imag(), &v));
    return (BaseType)v;
  }
  BaseType MaxL2NormDiff(QubitRegister& x) {
    same_layout(x);
    double v = 0;
    check_status(iqsg_l2_diff(h_, x.h_, &v));
    return (BaseType)v;
  }
  void AmplitudeWiseScalarMultiplication(Type f) {
    ApplyFusedGates();
    check_status(iqsg_scale(h_, f.real(), f.imag()));
  }
  void AmplitudeWiseSum(QubitRegister& psi, Type f = Type(1, 0)) {
    same_layout(psi);
    check_status(iqsg_axpy(h_, psi.h_, f.real(), f.imag()));
  }
  // All amplitudes (data order) to / from host memory.
  std::vector<Type> GetStateVector() {
    ApplyFusedGates();
    std::vector<Type> v(LocalSize());
    check_status(iqsg_download(h_, v.data(), 0, v.size()));
    return v;
  }
  void SetStateVector(const std::vector<Type>& v) {
    ApplyFusedGates();
    if (v.size() != LocalSize()) throw std::invalid_argument("SetStateVector: wrong size");
    check_status(iqsg_upload(h_, v.data(), 0, v.size()));
  }

 private:
  static constexpr int kPrec = std::is_same<Type, ComplexDP>::value ? IQSG_COMPLEX_DP : IQSG_COMPLEX_SP;

  unsigned pos(unsigned q) const {
    if (q >= n_) throw std::invalid_argument("qubit index out of range");
    return (unsigned)perm_.map[q];
  }
  std::size_t check_index(std::size_t i) const {
    if (i >= GlobalSize()) throw std::invalid_argument("amplitude index out of range");
    return i;
  }
  Type read(std::size_t i) {
    ApplyFusedGates();
    double v[2];
    check_status(iqsg_get_amplitude(h_, check_index(i), v));
    return Type((BaseType)v[0], (BaseType)v[1]);
  }
  void write(std::size_t i, Type v) {
    ApplyFusedGates();
    check_status(iqsg_set_amplitude(h_, check_index(i), v.real(), v.imag()));
  }
  static TM2x2<Type> mat2(double a, double b, double c, double d, double e, double f, double g, double h) {
    TM2x2<Type> m;
    m(0, 0) = Type(a, b);
    m(0, 1) = Type(c, d);
    m(1, 0) = Type(e, f);
    m(1, 1) = Type(g, h);
    return m;
  }
  static std::vector<double> m8(const TM2x2<Type>& m) {
    std::vector<double> d(8);
    for (int r = 0; r < 2; ++r)
      for (int c = 0; c < 2; ++c) { d[2 * (2 * r + c)] = (double)m(r, c).real(); d[2 * (2 * r + c) + 1] = (double)m(r, c).imag(); }
    return d;
  }
  static iqsg_op make(int kind, unsigned t0, unsigned t1, const double* m, int nm) {
    iqsg_op op;
    std::memset(&op, 0, sizeof op);
    op.kind = kind;
    op.t0 = t0;
    op.t1 = t1;
    std::memcpy(op.m, m, sizeof(double) * nm);
    return op;
  }
  void queue(const iqsg_op& op) {
    fwindow_.push_back(op);
    if (fwindow_.size() >= 4096) ApplyFusedGates();
  }
  void swaplike(unsigned a, unsigned b, const TM2x2<Type>& m) {
    const unsigned p1 = pos(a), p2 = pos(b);
    if (a == b) throw std::invalid_argument("swap: qubits coincide");
    if (p1 > p2 && m(0, 1) != m(1, 0)) throw std::invalid_argument("swap: the 2x2 block must be symmetric");
    if (gate_counter) gate_counter->TwoQubitIncrement((int)a, (int)b);
    iqsg_op op = make(IQSG_OP_SWAPLIKE, p1, p2, m8(m).data(), 8);
    if (fusion_) return queue(op);
    check_status(iqsg_apply_swaplike(h_, p1, p2, op.m));
  }
  BaseType ev(std::vector<unsigned> q, std::vector<unsigned> o, BaseType c) { return ExpectationValue(q, o, c); }
  void same_layout(QubitRegister& other) {
    if (other.perm_.map != perm_.map) throw std::invalid_argument("registers have different qubit orders");
    ApplyFusedGates();
    other.ApplyFusedGates();
  }

  template <class Chi>
  void channel_draw(unsigned M, const Chi& chi, double* gate) {
    if (!rng_ptr_) throw std::invalid_argument("ApplyChannel: SetRngPtr first");
    std::vector<double> ev, cum, vecs;
    chi.channel_arrays(ev, cum, vecs);
    unsigned k = 0;
    int negative = 0;
    check_status(iqsg_channel_gate(rng_ptr_->handle(), kPrec, M, ev.data(), cum.data(), vecs.data(), gate, &k,
                                   &negative));
    if (negative) overall_sign_of_channels *= -1;
  }

  RandomNumberGenerator<BaseType>* rng_ptr_ = nullptr;
  BaseType T_1_ = 0, T_2_ = 0, T_phi_ = 0;
  BaseType overall_sign_of_channels = 1;
  unsigned n_;
  iqsg_state* h_ = nullptr;
  Permutation perm_;
  bool fusion_ = false;
  unsigned log2llc_ = 20;
  std::vector<iqsg_op> fwindow_;
};

}  // namespace iqs

#include "noisy_qureg.hpp"
#include "qubit_register_metric.hpp"
