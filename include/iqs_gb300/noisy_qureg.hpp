// iqs_gb300/noisy_qureg.hpp -- iqs::NoisyQureg<Type> (include/NoisyQureg.hpp of intel/intel-qs)
// over the drop-in QubitRegister, included at the end of qureg.hpp.
//
// Each qubit keeps the time since its last gate. Before a 1-qubit gate on q (2-qubit gate on q1,
// q2) the Pauli-twirl noise gate for that idle time is applied, every qubit's idle time grows by
// the gate duration and q's is reset. Noise angles come from this object's own
// std::default_random_engine + std::normal_distribution<BaseType>, held in libiqsg. As in the
// reference, only the gates listed here add noise (the base class's methods are not virtual).
#pragma once

#include <vector>

namespace iqs {

template <class Type = ComplexDP>
class NoisyQureg : public QubitRegister<Type> {
 public:
  using BaseType = typename QubitRegister<Type>::BaseType;

  NoisyQureg(unsigned num_qubits, unsigned RNG_seed = 12345, BaseType T1 = 2000, BaseType T2 = 1000)
      : QubitRegister<Type>(num_qubits) {
    T_1 = T1;
    T_2 = T2;
    time_from_last_gate.assign(num_qubits, 0.);
    experimental_gate_count_matrix.assign(num_qubits * num_qubits, 0);
    check_status(iqsg_noise_engine_create(RNG_seed, &engine_));
  }
  NoisyQureg(const NoisyQureg&) = delete;
  NoisyQureg& operator=(const NoisyQureg&) = delete;
  ~NoisyQureg() { iqsg_noise_engine_destroy(engine_); }

  void Initialize(std::string style, std::size_t base_index) {
    one_qubit_experimental_gate_count = 0;
    two_qubit_experimental_gate_count = 0;
    ResetTimeForAllQubits();
    QubitRegister<Type>::Initialize(style, base_index);
  }
  void ResetTimeForAllQubits() {
    for (auto& t : time_from_last_gate) t = 0.;
  }
  void ApplyNoiseGatesOnAllQubits() {
    for (unsigned q = 0; q < nq(); q++) NoiseGate(q);
    ResetTimeForAllQubits();
  }
  void SetDecoherenceTime(BaseType T1, BaseType T2) {
    T_1 = T1;
    T_2 = T2;
  }
  void SetGateDurations(BaseType Ts, BaseType Td) {
    time_one_qubit_experimental_gate = Ts;
    time_two_qubit_experimental_gate = Td;
  }

  unsigned GetTotalExperimentalGateCount() { return one_qubit_experimental_gate_count + two_qubit_experimental_gate_count; }
  unsigned GetOneQubitExperimentalGateCount() { return one_qubit_experimental_gate_count; }
  unsigned GetTwoQubitExperimentalGateCount() { return two_qubit_experimental_gate_count; }
  std::vector<unsigned> GetExperimentalGateCount(unsigned q) {
    return std::vector<unsigned>(experimental_gate_count_matrix.begin() + q * nq(),
                                 experimental_gate_count_matrix.begin() + (q + 1) * nq());
  }
  unsigned GetExperimentalGateCount(unsigned q1, unsigned q2) { return experimental_gate_count_matrix[q1 * nq() + q2]; }

  void AddNoiseOneQubitGate(unsigned const qubit) {
    NoiseGate(qubit);
    for (auto& t : time_from_last_gate) t += time_one_qubit_experimental_gate;
    time_from_last_gate[qubit] = 0.;
    one_qubit_experimental_gate_count++;
    experimental_gate_count_matrix[qubit * nq() + qubit]++;
  }
  void AddNoiseTwoQubitGate(unsigned const q1, unsigned const q2) {
    NoiseGate(q1);
    NoiseGate(q2);
    for (auto& t : time_from_last_gate) t += time_two_qubit_experimental_gate;
    time_from_last_gate[q1] = 0.;
    time_from_last_gate[q2] = 0.;
    two_qubit_experimental_gate_count++;
    experimental_gate_count_matrix[q1 * nq() + q2]++;
    experimental_gate_count_matrix[q2 * nq() + q1]++;
  }
  void NoiseGate(unsigned const qubit) {
    const BaseType t = time_from_last_gate[qubit];
    if (t == 0) return;
    double g[3], m[8];
    check_status(iqsg_noise_engine_gaussian(engine_, kPrec, g, 3));
    check_status(iqsg_noise_gate_matrix(kPrec, T_1, T_2, t, g, m));
    TM2x2<Type> u;
    for (int i = 0; i < 4; ++i) u(i / 2, i % 2) = Type((BaseType)m[2 * i], (BaseType)m[2 * i + 1]);
    QubitRegister<Type>::Apply1QubitGate(qubit, u);
  }

  void Apply1QubitGate(unsigned const q, TM2x2<Type> V) {
    AddNoiseOneQubitGate(q);
    QubitRegister<Type>::Apply1QubitGate(q, V);
  }
  void ApplyHadamard(unsigned const q) {
    AddNoiseOneQubitGate(q);
    QubitRegister<Type>::ApplyHadamard(q);
  }
  void ApplyRotationX(unsigned const q, BaseType theta) {
    AddNoiseOneQubitGate(q);
    QubitRegister<Type>::ApplyRotationX(q, theta);
  }
  void ApplyRotationY(unsigned const q, BaseType theta) {
    AddNoiseOneQubitGate(q);
    QubitRegister<Type>::ApplyRotationY(q, theta);
  }
  void ApplyRotationZ(unsigned const q, BaseType theta) {
    AddNoiseOneQubitGate(q);
    QubitRegister<Type>::ApplyRotationZ(q, theta);
  }
  void ApplyCPauliX(unsigned const q1, unsigned const q2) {
    AddNoiseTwoQubitGate(q1, q2);
    QubitRegister<Type>::ApplyCPauliX(q1, q2);
  }
  void ApplyControlled1QubitGate(unsigned const q1, unsigned const q2, TM2x2<Type> V) {
    AddNoiseTwoQubitGate(q1, q2);
    QubitRegister<Type>::ApplyControlled1QubitGate(q1, q2, V);
  }

 private:
  static constexpr int kPrec = std::is_same<Type, ComplexDP>::value ? IQSG_COMPLEX_DP : IQSG_COMPLEX_SP;
  unsigned nq() { return (unsigned)this->NumQubits(); }

  std::vector<BaseType> time_from_last_gate;
  BaseType time_one_qubit_experimental_gate = 1.;
  BaseType time_two_qubit_experimental_gate = 1.;
  std::vector<unsigned> experimental_gate_count_matrix;
  unsigned one_qubit_experimental_gate_count = 0;
  unsigned two_qubit_experimental_gate_count = 0;
  BaseType T_1 = 1000;
  BaseType T_2 = 100;
  iqsg_noise_engine* engine_ = nullptr;
};

}  // namespace iqs
