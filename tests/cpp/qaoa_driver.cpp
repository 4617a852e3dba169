// Drives iqs::qaoa and the state statistics through the C++ drop-in headers on the weighted
// ring of 6 of unit_test/include/qaoa_features_test.hpp (vertical edges 1.4, gamma 0.4, beta
// 0.3) and prints the results one per line for tests/test_gpu_cpp_shim.py.
#include <cstdio>
#include <vector>

#include "iqs_gb300/qaoa_features.hpp"
#include "iqs_gb300/qureg.hpp"

int main() {
  std::vector<double> adj = {0, 1, 0, 0, 0, 1.4, 1, 0, 1, 0, 0, 0, 0, 1, 0, 1.4, 0, 0,
                             0, 0, 1.4, 0, 1, 0, 0, 0, 0, 1, 0, 1, 1.4, 0, 0, 0, 1, 0};
  iqs::QubitRegister<ComplexDP> diag(6, "base", 0);
  const double mx = iqs::qaoa::InitializeVectorAsWeightedMaxCutCostFunction(diag, adj);
  iqs::QubitRegister<ComplexDP> psi(6, "++++", 0);
  iqs::qaoa::ImplementQaoaLayerBasedOnCostFunction(psi, diag, 0.4);
  for (unsigned q = 0; q < 6; ++q) psi.ApplyRotationX(q, 0.3);
  const double e = iqs::qaoa::GetExpectationValueFromCostFunction(psi, diag);
  const auto h1 = iqs::qaoa::GetHistogramFromCostFunctionWithWeightsRounded(psi, diag, mx);
  const auto h2 = iqs::qaoa::GetHistogramFromCostFunctionWithWeightsBinned(psi, diag, mx, 0.1);
  std::printf("max %.17g\n", mx);
  std::printf("cost4 %.17g\ncost36 %.17g\n", diag.GetGlobalAmplitude(4).real(), diag.GetGlobalAmplitude(36).real());
  std::printf("expect %.17g\n", e);
  for (double v : h1) std::printf("h1 %.17g\n", v);
  for (double v : h2) std::printf("h2 %.17g\n", v);
  for (double v : psi.GoogleStats()) std::printf("stat %.17g\n", v);
  std::vector<int> ring = {0, 1, 0, 0, 0, 1, 1, 0, 1, 0, 0, 0, 0, 1, 0, 1, 0, 0,
                           0, 0, 1, 0, 1, 0, 0, 0, 0, 1, 0, 1, 1, 0, 0, 0, 1, 0};
  iqs::QubitRegister<ComplexDP> d2(6, "base", 0);
  const int m2 = iqs::qaoa::InitializeVectorAsMaxCutCostFunction(d2, ring);
  for (double v : iqs::qaoa::GetHistogramFromCostFunction(psi, d2, m2)) std::printf("h0 %.17g\n", v);
  iqs::QubitRegister<ComplexDP> small(2, "base", 2);
  small.ApplyHadamard(0);
  small.Print("small");
  return 0;
}
