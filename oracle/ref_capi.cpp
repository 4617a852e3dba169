// Test infrastructure only: a flat C binding over the reference library's public
// C++ API (iqs::QubitRegister<Type>, include/qureg.hpp:127-417 of intel/intel-qs),
// used to generate golden vectors and to pin the C restatement in iqs_oracle.c.
// It is compiled by oracle/Makefile against the reference's own headers and linked
// with the reference's own sources (built into oracle/_ref/, never committed).
// Every function forwards to exactly one reference method; no arithmetic here.
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "qureg.hpp"
#include "qaoa_features.hpp"

using iqs::QubitRegister;
using CDP = ComplexDP;
using CSP = ComplexSP;

struct RefReg {
  int sp;  // 0 = ComplexDP, 1 = ComplexSP
  QubitRegister<CDP>* dp;
  QubitRegister<CSP>* spr;
};

template <class T> static QubitRegister<T>* R(RefReg* h);
template <> QubitRegister<CDP>* R<CDP>(RefReg* h) { return h->dp; }
template <> QubitRegister<CSP>* R<CSP>(RefReg* h) { return h->spr; }

template <class T>
static iqs::TinyMatrix<T, 2, 2, 32> tm2(const double* m) {
  iqs::TinyMatrix<T, 2, 2, 32> t;
  for (int r = 0; r < 2; ++r)
    for (int c = 0; c < 2; ++c) t(r, c) = T(m[2 * (2 * r + c)], m[2 * (2 * r + c) + 1]);
  return t;
}
template <class T>
static iqs::TinyMatrix<T, 4, 4, 32> tm4(const double* m) {
  iqs::TinyMatrix<T, 4, 4, 32> t;
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) t(r, c) = T(m[2 * (4 * r + c)], m[2 * (4 * r + c) + 1]);
  return t;
}

#define DISPATCH(h, EXPR)                      \
  do {                                         \
    if ((h)->sp) { using T = CSP; auto* q = R<T>(h); EXPR; } \
    else         { using T = CDP; auto* q = R<T>(h); EXPR; } \
  } while (0)

extern "C" {

RefReg* ref_create(unsigned n, int sp) {
  RefReg* h = new RefReg{sp, nullptr, nullptr};
  if (sp) h->spr = new QubitRegister<CSP>(n, "base", 0);
  else h->dp = new QubitRegister<CDP>(n, "base", 0);
  return h;
}
void ref_destroy(RefReg* h) { delete h->dp; delete h->spr; delete h; }

// state as interleaved (re, im) doubles, data order
void ref_set_state(RefReg* h, const double* s) {
  DISPATCH(h, { for (size_t i = 0; i < q->LocalSize(); ++i) (*q)[i] = T(s[2 * i], s[2 * i + 1]); });
}
void ref_get_state(RefReg* h, double* s) {
  DISPATCH(h, { for (size_t i = 0; i < q->LocalSize(); ++i) { s[2 * i] = (*q)[i].real(); s[2 * i + 1] = (*q)[i].imag(); } });
}
void ref_initialize(RefReg* h, const char* style, size_t base) { DISPATCH(h, q->Initialize(std::string(style), base)); }

void ref_apply1q(RefReg* h, unsigned qb, const double* m) { DISPATCH(h, q->Apply1QubitGate(qb, tm2<T>(m))); }
void ref_ctrl1q(RefReg* h, unsigned c, unsigned t, const double* m) { DISPATCH(h, q->ApplyControlled1QubitGate(c, t, tm2<T>(m))); }
void ref_2q(RefReg* h, unsigned qh, unsigned ql, const double* m) { DISPATCH(h, q->Apply2QubitGate(qh, ql, tm4<T>(m))); }
void ref_diag(RefReg* h, unsigned q1, unsigned q2, const double* m) { DISPATCH(h, q->ApplyDiag(q1, q2, tm4<T>(m))); }
void ref_iswaprot(RefReg* h, unsigned q1, unsigned q2, const double* m) { DISPATCH(h, q->ApplyISwapRotation(q1, q2, tm2<T>(m))); }

// named gates: op codes shared with the Python side of the oracle
void ref_named1(RefReg* h, const char* name, unsigned qb, double a, double b) {
  std::string s(name);
  DISPATCH(h, {
    if (s == "ApplyRotationX") q->ApplyRotationX(qb, a);
    else if (s == "ApplyRotationY") q->ApplyRotationY(qb, a);
    else if (s == "ApplyRotationZ") q->ApplyRotationZ(qb, a);
    else if (s == "ApplyPauliX") q->ApplyPauliX(qb);
    else if (s == "ApplyPauliY") q->ApplyPauliY(qb);
    else if (s == "ApplyPauliZ") q->ApplyPauliZ(qb);
    else if (s == "ApplyPauliSqrtX") q->ApplyPauliSqrtX(qb);
    else if (s == "ApplyPauliSqrtY") q->ApplyPauliSqrtY(qb);
    else if (s == "ApplyPauliSqrtZ") q->ApplyPauliSqrtZ(qb);
    else if (s == "ApplyT") q->ApplyT(qb);
    else if (s == "ApplyHadamard") q->ApplyHadamard(qb);
    else if (s == "ApplyRotationXY") q->ApplyRotationXY(qb, a, b);
  });
}
void ref_named2(RefReg* h, const char* name, unsigned c, unsigned t, double a) {
  std::string s(name);
  DISPATCH(h, {
    if (s == "ApplyCRotationX") q->ApplyCRotationX(c, t, a);
    else if (s == "ApplyCRotationY") q->ApplyCRotationY(c, t, a);
    else if (s == "ApplyCRotationZ") q->ApplyCRotationZ(c, t, a);
    else if (s == "ApplyCPauliX") q->ApplyCPauliX(c, t);
    else if (s == "ApplyCPauliY") q->ApplyCPauliY(c, t);
    else if (s == "ApplyCPauliZ") q->ApplyCPauliZ(c, t);
    else if (s == "ApplyCPauliSqrtZ") q->ApplyCPauliSqrtZ(c, t);
    else if (s == "ApplyCHadamard") q->ApplyCHadamard(c, t);
    else if (s == "ApplyCPhaseRotation") q->ApplyCPhaseRotation(c, t, a);
    else if (s == "ApplySwap") q->ApplySwap(c, t);
    else if (s == "ApplyISwap") q->ApplyISwap(c, t);
    else if (s == "ApplySqrtISwap") q->ApplySqrtISwap(c, t);
    else if (s == "Apply4thRootISwap") q->Apply4thRootISwap(c, t);
  });
}
void ref_toffoli(RefReg* h, unsigned c1, unsigned c2, unsigned t) { DISPATCH(h, q->ApplyToffoli(c1, c2, t)); }

void ref_permute(RefReg* h, const unsigned* map, unsigned n, int inverse) {
  std::vector<std::size_t> m(map, map + n);
  DISPATCH(h, q->PermuteQubits(m, inverse ? "inverse" : "direct"));
}
void ref_get_map(RefReg* h, unsigned* map) {
  DISPATCH(h, { for (size_t i = 0; i < q->NumQubits(); ++i) map[i] = (unsigned)q->qubit_permutation->map[i]; });
}
void ref_emulate_swap(RefReg* h, unsigned q1, unsigned q2) { DISPATCH(h, q->EmulateSwap(q1, q2)); }
void ref_get_global_amplitude(RefReg* h, size_t idx, double* out) {
  DISPATCH(h, { T a = q->GetGlobalAmplitude(idx); out[0] = a.real(); out[1] = a.imag(); });
}
void ref_set_global_amplitude(RefReg* h, size_t idx, double re, double im) { DISPATCH(h, q->SetGlobalAmplitude(idx, T(re, im))); }

double ref_probability(RefReg* h, unsigned qb) { double r = 0; DISPATCH(h, r = q->GetProbability(qb)); return r; }
void ref_collapse(RefReg* h, unsigned qb, int v) { DISPATCH(h, q->CollapseQubit(qb, v != 0)); }
double ref_expectation(RefReg* h, unsigned k, const unsigned* qubits, const unsigned* obs, double coeff) {
  std::vector<unsigned> qv(qubits, qubits + k), ov(obs, obs + k);
  double r = 0;
  DISPATCH(h, r = q->ExpectationValue(qv, ov, coeff));
  return r;
}
double ref_norm(RefReg* h) { double r = 0; DISPATCH(h, r = q->ComputeNorm()); return r; }
void ref_normalize(RefReg* h) { DISPATCH(h, q->Normalize()); }
void ref_overlap(RefReg* h, RefReg* o, double* out) {
  DISPATCH(h, { T v = q->ComputeOverlap(*R<T>(o)); out[0] = v.real(); out[1] = v.imag(); });
}
double ref_max_abs_diff(RefReg* h, RefReg* o, double re, double im) { double r = 0; DISPATCH(h, r = q->MaxAbsDiff(*R<T>(o), T(re, im))); return r; }
double ref_max_l2_diff(RefReg* h, RefReg* o) { double r = 0; DISPATCH(h, r = q->MaxL2NormDiff(*R<T>(o))); return r; }
void ref_scale(RefReg* h, double re, double im) { DISPATCH(h, q->AmplitudeWiseScalarMultiplication(T(re, im))); }
void ref_axpy(RefReg* h, RefReg* o, double re, double im) { DISPATCH(h, q->AmplitudeWiseSum(*R<T>(o), T(re, im))); }
void ref_fill(RefReg* h, double re, double im) { DISPATCH(h, q->InitializationWithSameAmplitudeEverywhere(T(re, im))); }

void ref_fusion_on(RefReg* h, unsigned log2llc) { DISPATCH(h, q->TurnOnFusion(log2llc)); }
void ref_fusion_off(RefReg* h) { DISPATCH(h, q->TurnOffFusion()); }

int ref_qaoa_maxcut_cost(RefReg* diag, const int* adj, unsigned nv) {
  std::vector<int> a(adj, adj + nv * nv);
  int r = 0;
  DISPATCH(diag, r = iqs::qaoa::InitializeVectorAsMaxCutCostFunction(*q, a));
  return r;
}
double ref_qaoa_weighted_cost(RefReg* diag, const double* adj, unsigned nv) {
  double r = 0;
  if (diag->sp) {
    std::vector<float> a(adj, adj + nv * nv);
    r = iqs::qaoa::InitializeVectorAsWeightedMaxCutCostFunction(*diag->spr, a);
  } else {
    std::vector<double> a(adj, adj + nv * nv);
    r = iqs::qaoa::InitializeVectorAsWeightedMaxCutCostFunction(*diag->dp, a);
  }
  return r;
}
void ref_qaoa_layer(RefReg* psi, RefReg* diag, double gamma) {
  DISPATCH(psi, iqs::qaoa::ImplementQaoaLayerBasedOnCostFunction(*q, *R<T>(diag), (typename QubitRegister<T>::BaseType)gamma));
}
double ref_qaoa_expectation(RefReg* psi, RefReg* diag) {
  double r = 0;
  DISPATCH(psi, r = iqs::qaoa::GetExpectationValueFromCostFunction(*q, *R<T>(diag)));
  return r;
}
// mode 0: GetHistogramFromCostFunction, 1: ...WithWeightsRounded, 2: ...WithWeightsBinned.
// Writes at most cap bins; returns the histogram's length.
int ref_qaoa_histogram(RefReg* psi, RefReg* diag, int mode, double max_value, double bin_width, double* out, int cap) {
  int len = 0;
  DISPATCH(psi, {
    std::vector<typename QubitRegister<T>::BaseType> h;
    if (mode == 0) h = iqs::qaoa::GetHistogramFromCostFunction(*q, *R<T>(diag), (int)max_value);
    else if (mode == 1) h = iqs::qaoa::GetHistogramFromCostFunctionWithWeightsRounded(*q, *R<T>(diag), max_value);
    else h = iqs::qaoa::GetHistogramFromCostFunctionWithWeightsBinned(*q, *R<T>(diag), max_value, bin_width);
    len = (int)h.size();
    for (int i = 0; i < len && i < cap; ++i) out[i] = (double)h[i];
  });
  return len;
}
// Initialize("rand", base_index) `times` times in a row with a RandomNumberGenerator seeded with seed.
void ref_init_rand(RefReg* h, unsigned long seed, int base_index, int times) {
  DISPATCH(h, {
    auto* rng = new iqs::RandomNumberGenerator<typename QubitRegister<T>::BaseType>();
    rng->SetSeedStreamPtrs(seed);
    q->SetRngPtr(rng);
    for (int t = 0; t < times; ++t) q->Initialize("rand", (std::size_t)base_index);
    q->ResetRngPtr();
    delete rng;
  });
}
double ref_entropy(RefReg* h) {
  double r = 0;
  DISPATCH(h, r = q->Entropy());
  return r;
}
int ref_google_stats(RefReg* h, double* out, int cap) {
  int len = 0;
  DISPATCH(h, {
    std::vector<double> v = q->GoogleStats();
    len = (int)v.size();
    for (int i = 0; i < len && i < cap; ++i) out[i] = v[i];
  });
  return len;
}
void ref_print(RefReg* h, const char* x) {
  DISPATCH(h, q->Print(std::string(x), std::vector<std::size_t>()));
  fflush(stdout);
}
void ref_export(RefReg* h, const char* fname) { DISPATCH(h, q->ExportAmplitudes(std::string(fname))); }
double ref_qaoa_expectation_sq(RefReg* psi, RefReg* diag) {
  double r = 0;
  DISPATCH(psi, r = iqs::qaoa::GetExpectationValueSquaredFromCostFunction(*q, *R<T>(diag)));
  return r;
}


}  // extern "C"

// ---- random numbers, noise gates, channels ----

// A sequence of draws on one RandomNumberGenerator<float|double>: ops holds triples
// (kind, n, stream) -- kind 0 uniform [0,1), 1 uniform [-2,5), 2 Gaussian, 3 integers in [-3,17),
// 4 SkipAhead, 5 replace the generator by a copy of itself (copy constructor); stream 0 pool,
// 1 state, 2 local. Values drawn are appended to out; counts[3] receives the final counts.
template <class B>
static int rng_sequence(unsigned long seed, const int* ops, int nops, double* out, int cap, unsigned long* counts) {
  static const char* names[3] = {"pool", "state", "local"};
  auto* rng = new iqs::RandomNumberGenerator<B>();
  rng->SetSeedStreamPtrs(seed);
  int len = 0;
  for (int i = 0; i < nops; ++i) {
    const int kind = ops[3 * i], n = ops[3 * i + 1];
    const std::string st = names[ops[3 * i + 2]];
    std::vector<B> v(n > 0 ? n : 1);
    std::vector<int> iv(n > 0 ? n : 1);
    if (kind == 0) rng->UniformRandomNumbers(v.data(), n, B(0), B(1), st);
    if (kind == 1) rng->UniformRandomNumbers(v.data(), n, B(-2), B(5), st);
    if (kind == 2) rng->GaussianRandomNumbers(v.data(), n, st);
    if (kind == 3) {
      rng->RandomIntegersInRange(iv.data(), n, -3, 17, st);
      for (int j = 0; j < n; ++j) v[j] = (B)iv[j];
    }
    if (kind == 4) rng->SkipAhead(n, st);
    if (kind == 5) {
      auto* c = new iqs::RandomNumberGenerator<B>(rng);
      delete rng;
      rng = c;
    }
    if (kind <= 3)
      for (int j = 0; j < n && len < cap; ++j) out[len++] = (double)v[j];
  }
  counts[0] = rng->GetNumGeneratedOrSkippedPoolNumbers();
  counts[1] = rng->GetNumGeneratedOrSkippedStateNumbers();
  counts[2] = rng->GetNumGeneratedOrSkippedLocalNumbers();
  delete rng;
  return len;
}
extern "C" int ref_rng_sequence(int sp, unsigned long seed, const int* ops, int nops, double* out, int cap, unsigned long* counts) {
  return sp ? rng_sequence<float>(seed, ops, nops, out, cap, counts)
            : rng_sequence<double>(seed, ops, nops, out, cap, counts);
}

// SetNoiseTimescales(T1, T2), then ApplyNoiseGate(qubits[i], durations[i]) for i < steps with a
// generator seeded with seed; counts[3] receives the generator's final counts.
extern "C" void ref_noise_run(RefReg* h, unsigned long seed, double T1, double T2, const unsigned* qubits,
                   const double* durations, int steps, unsigned long* counts) {
  DISPATCH(h, {
    using B = typename QubitRegister<T>::BaseType;
    iqs::RandomNumberGenerator<B> rng;
    rng.SetSeedStreamPtrs(seed);
    q->SetRngPtr(&rng);
    q->SetNoiseTimescales((B)T1, (B)T2);
    for (int i = 0; i < steps; ++i) q->ApplyNoiseGate(qubits[i], (B)durations[i]);
    q->ResetRngPtr();
    counts[0] = rng.GetNumGeneratedOrSkippedPoolNumbers();
    counts[1] = rng.GetNumGeneratedOrSkippedStateNumbers();
    counts[2] = rng.GetNumGeneratedOrSkippedLocalNumbers();
  });
}

// A NoisyQureg<Type>(n, seed, T1, T2) program: Initialize("base", 0), SetGateDurations(Ts, Td),
// then prog triples (kind, a, b) -- 0 H a, 1 RX a, 2 RY a, 3 RZ a (angle angles[i]),
// 4 CPauliX a b, 5 ApplyControlled1QubitGate a b mats[i], 6 Apply1QubitGate a mats[i],
// 7 ApplyNoiseGatesOnAllQubits. Writes the state, the 1- and 2-qubit gate counts and the n x n
// gate-count matrix.
template <class T>
static void noisy_run(unsigned n, unsigned seed, double T1, double T2, double Ts, double Td, const int* prog,
                      const double* angles, const double* mats, int nprog, double* state, unsigned* counts) {
  using B = typename QubitRegister<T>::BaseType;
  iqs::NoisyQureg<T> r(n, seed, (B)T1, (B)T2);
  r.Initialize("base", 0);
  r.SetGateDurations((B)Ts, (B)Td);
  for (int i = 0; i < nprog; ++i) {
    const int kind = prog[3 * i];
    const unsigned a = (unsigned)prog[3 * i + 1], b = (unsigned)prog[3 * i + 2];
    if (kind == 0) r.ApplyHadamard(a);
    if (kind == 1) r.ApplyRotationX(a, (B)angles[i]);
    if (kind == 2) r.ApplyRotationY(a, (B)angles[i]);
    if (kind == 3) r.ApplyRotationZ(a, (B)angles[i]);
    if (kind == 4) r.ApplyCPauliX(a, b);
    if (kind == 5) r.ApplyControlled1QubitGate(a, b, tm2<T>(mats + 8 * i));
    if (kind == 6) r.Apply1QubitGate(a, tm2<T>(mats + 8 * i));
    if (kind == 7) r.ApplyNoiseGatesOnAllQubits();
  }
  for (std::size_t i = 0; i < (std::size_t(1) << n); ++i) {
    const T v = r.GetGlobalAmplitude(i);
    state[2 * i] = v.real();
    state[2 * i + 1] = v.imag();
  }
  counts[0] = r.GetOneQubitExperimentalGateCount();
  counts[1] = r.GetTwoQubitExperimentalGateCount();
  for (unsigned x = 0; x < n; ++x)
    for (unsigned y = 0; y < n; ++y) counts[2 + x * n + y] = r.GetExperimentalGateCount(x, y);
}
extern "C" void ref_noisy_qureg_run(int sp, unsigned n, unsigned seed, double T1, double T2, double Ts, double Td,
                         const int* prog, const double* angles, const double* mats, int nprog, double* state,
                         unsigned* counts) {
  if (sp) noisy_run<CSP>(n, seed, T1, T2, Ts, Td, prog, angles, mats, nprog, state, counts);
  else noisy_run<CDP>(n, seed, T1, T2, Ts, Td, prog, angles, mats, nprog, state, counts);
}

// A chi matrix whose eigensystem is given by the caller (the reference's members are protected
// and its SolveEigenSystem needs Eigen, which is not vendored): eigenvalues, eigenvectors, then
// the reference's own NormalizeEigenProbAndRenormalizeEigenVect.
template <class T, unsigned M>
struct GivenChi : iqs::ChiMatrix<T, M, 32> {
  GivenChi(const double* evals, const double* evecs) {
    this->evalues_.assign(M, T(0));
    this->evectors_.assign(M, std::vector<T>(M, T(0)));
    for (unsigned k = 0; k < M; ++k) {
      this->evalues_[k] = T(evals[2 * k], evals[2 * k + 1]);
      for (unsigned i = 0; i < M; ++i)
        this->evectors_[k][i] = T(evecs[2 * (k * M + i)], evecs[2 * (k * M + i) + 1]);
    }
    this->NormalizeEigenProbAndRenormalizeEigenVect();
  }
};

// The normalised eigensystem (probabilities, cumulative probabilities, eigenvectors) of GivenChi.
template <class T, unsigned M>
static void chi_normalize(const double* evals, const double* evecs, double* probs, double* cum, double* vecs) {
  GivenChi<T, M> chi(evals, evecs);
  for (unsigned k = 0; k < M; ++k) {
    probs[k] = chi.GetEigenProbability(k);
    cum[k] = chi.GetEigenCumulativeProbability(k);
    const std::vector<T> v = chi.GetEigenVector(k);
    for (unsigned i = 0; i < M; ++i) {
      vecs[2 * (k * M + i)] = v[i].real();
      vecs[2 * (k * M + i) + 1] = v[i].imag();
    }
  }
}
extern "C" void ref_chi_normalize(int sp, unsigned M, const double* evals, const double* evecs, double* probs, double* cum,
                       double* vecs) {
  if (M == 4) {
    if (sp) chi_normalize<CSP, 4>(evals, evecs, probs, cum, vecs);
    else chi_normalize<CDP, 4>(evals, evecs, probs, cum, vecs);
  } else {
    if (sp) chi_normalize<CSP, 16>(evals, evecs, probs, cum, vecs);
    else chi_normalize<CDP, 16>(evals, evecs, probs, cum, vecs);
  }
}

// ApplyChannel `steps` times (qubits: one per step for M = 4, two for M = 16) with a generator
// seeded with seed; returns GetOverallSignOfChannels().
template <class T>
static double channel_run(QubitRegister<T>* q, unsigned long seed, unsigned M, const double* evals,
                          const double* evecs, const unsigned* qubits, int steps) {
  using B = typename QubitRegister<T>::BaseType;
  iqs::RandomNumberGenerator<B> rng;
  rng.SetSeedStreamPtrs(seed);
  q->SetRngPtr(&rng);
  if (M == 4) {
    GivenChi<T, 4> chi(evals, evecs);
    for (int i = 0; i < steps; ++i) q->ApplyChannel(qubits[i], chi);
  } else {
    GivenChi<T, 16> chi(evals, evecs);
    for (int i = 0; i < steps; ++i) q->ApplyChannel(qubits[2 * i], qubits[2 * i + 1], chi);
  }
  q->ResetRngPtr();
  return q->GetOverallSignOfChannels();
}
extern "C" double ref_channel_run(RefReg* h, unsigned long seed, unsigned M, const double* evals, const double* evecs,
                                  const unsigned* qubits, int steps) {
  return h->sp ? channel_run<CSP>(h->spr, seed, M, evals, evecs, qubits, steps)
               : channel_run<CDP>(h->dp, seed, M, evals, evecs, qubits, steps);
}

// The reference's unit test ApplyQuantumChannel.IdealHadamard: the eigensystem set by
// EigensystemOfIdealHadamardChannel (ComplexDP only), ApplyChannel `times` times on `qubit`.
extern "C" void ref_ideal_hadamard_channel(RefReg* h, unsigned long seed, unsigned qubit, int times) {
  CM4x4<CDP> chi;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) chi(i, j) = CDP(0, 0);
  chi(1, 1) = chi(1, 3) = chi(3, 1) = chi(3, 3) = CDP(0.5, 0);
  chi.EigensystemOfIdealHadamardChannel();
  iqs::RandomNumberGenerator<double> rng;
  rng.SetSeedStreamPtrs(seed);
  h->dp->SetRngPtr(&rng);
  for (int t = 0; t < times; ++t) h->dp->ApplyChannel(qubit, chi);
  h->dp->ResetRngPtr();
}
