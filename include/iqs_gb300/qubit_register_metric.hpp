// iqs_gb300/qubit_register_metric.hpp -- iqs::QubitRegisterMetric<Type>
// (include/QubitRegisterMetric.hpp of intel/intel-qs) over the drop-in QubitRegister, included at
// the end of qureg.hpp: the gates below also count 1- and 2-qubit gates and track a per-qubit
// depth (a 2-qubit gate puts both qubits at one more than the deeper of the two).
#pragma once

#include <algorithm>
#include <vector>

namespace iqs {

template <class Type = ComplexDP>
class QubitRegisterMetric : public QubitRegister<Type> {
 public:
  explicit QubitRegisterMetric(int iNQubits) : QubitRegister<Type>(iNQubits) { depth_.assign(iNQubits, 0); }

  int GetTotalQubitGateCount() { return total_; }
  int GetOneQubitGateCount() { return one_; }
  int GetTwoQubitGateCount() { return two_; }
  int GetParallelDepth() { return depth_.empty() ? 0 : *std::max_element(depth_.begin(), depth_.end()); }

  void ApplyHadamard(int q) {
    QubitRegister<Type>::ApplyHadamard(q);
    one(q);
  }
  void ApplyRotationX(int q, double theta) {
    QubitRegister<Type>::ApplyRotationX(q, theta);
    one(q);
  }
  void ApplyRotationY(int q, double theta) {
    QubitRegister<Type>::ApplyRotationY(q, theta);
    one(q);
  }
  void ApplyRotationZ(int q, double theta) {
    QubitRegister<Type>::ApplyRotationZ(q, theta);
    one(q);
  }
  void ApplyCPauliX(int q1, int q2) {
    QubitRegister<Type>::ApplyCPauliX(q1, q2);
    two(q1, q2);
  }
  void ApplyControlled1QubitGate(int q1, int q2, TinyMatrix<Type, 2, 2, 32> V) {
    QubitRegister<Type>::ApplyControlled1QubitGate(q1, q2, V);
    two(q1, q2);
  }

 private:
  void one(int q) {
    ++total_;
    ++one_;
    ++depth_[q];
  }
  void two(int q1, int q2) {
    ++total_;
    ++two_;
    const int d = std::max(depth_[q1], depth_[q2]) + 1;
    depth_[q1] = depth_[q2] = d;
  }
  int total_ = 0, one_ = 0, two_ = 0;
  std::vector<int> depth_;
};

}  // namespace iqs
