// iqs::qaoa over GPU registers: the functions of include/qaoa_features.hpp of intel/intel-qs
// (src/qaoa_features.cpp:73-540) with the same names and arguments, for registers of the
// drop-in iqs::QubitRegister (qureg.hpp in this directory). The cost "vector" is a register
// whose real parts hold the cost of each basis state. Inputs the reference asserts on throw
// std::invalid_argument here.
#pragma once

#include <cmath>
#include <stdexcept>
#include <vector>

#include "qureg.hpp"

namespace iqs {
namespace qaoa {

namespace detail {
template <typename Type>
QubitRegister<Type>& mut(const QubitRegister<Type>& r) {
  return const_cast<QubitRegister<Type>&>(r);
}
template <typename Type>
void same_order(const QubitRegister<Type>& a, const QubitRegister<Type>& b) {
  if (mut(a).qubit_permutation_ptr()->map != mut(b).qubit_permutation_ptr()->map)
    throw std::invalid_argument("qaoa: psi and diag have different qubit orders");
  mut(a).ApplyFusedGates();
  mut(b).ApplyFusedGates();
}
template <typename Type>
std::vector<unsigned> positions(QubitRegister<Type>& r) {
  const auto& m = r.qubit_permutation_ptr()->map;
  return std::vector<unsigned>(m.begin(), m.end());
}
template <typename Type>
std::vector<typename QubitRegister<Type>::BaseType> histogram(const QubitRegister<Type>& psi,
                                                              const QubitRegister<Type>& diag, int mode,
                                                              double max_value, double bin_width, long long bins) {
  same_order(psi, diag);
  if (bins <= 0) throw std::invalid_argument("qaoa: max_value must be positive");
  std::vector<double> h((std::size_t)bins);
  const int st = iqsg_cost_histogram(mut(psi).handle(), mut(diag).handle(), mode, max_value, bin_width, h.data(),
                                     (unsigned)bins);
  if (st == IQSG_EINVAL) throw std::invalid_argument(iqsg_last_error());
  if (st != IQSG_OK) throw std::runtime_error(iqsg_last_error());
  return std::vector<typename QubitRegister<Type>::BaseType>(h.begin(), h.end());
}
inline void check(int st) {
  if (st == IQSG_EINVAL) throw std::invalid_argument(iqsg_last_error());
  if (st != IQSG_OK) throw std::runtime_error(iqsg_last_error());
}
}  // namespace detail

template <typename Type>
int InitializeVectorAsMaxCutCostFunction(QubitRegister<Type>& diag, std::vector<int>& adjacency) {
  const std::size_t n = diag.NumQubits();
  if (adjacency.size() != n * n) throw std::invalid_argument("qaoa: adjacency must have n*n entries");
  diag.ApplyFusedGates();
  const std::vector<unsigned> map = detail::positions(diag);
  int mx = 0;
  detail::check(iqsg_maxcut_cost(diag.handle(), adjacency.data(), map.data(), &mx));
  return mx;
}

template <typename Type>
typename QubitRegister<Type>::BaseType InitializeVectorAsWeightedMaxCutCostFunction(
    QubitRegister<Type>& diag, std::vector<typename QubitRegister<Type>::BaseType>& adjacency) {
  const std::size_t n = diag.NumQubits();
  if (adjacency.size() != n * n) throw std::invalid_argument("qaoa: adjacency must have n*n entries");
  diag.ApplyFusedGates();
  const std::vector<unsigned> map = detail::positions(diag);
  const std::vector<double> adj(adjacency.begin(), adjacency.end());
  double mx = 0;
  detail::check(iqsg_weighted_maxcut_cost(diag.handle(), adj.data(), map.data(), &mx));
  return (typename QubitRegister<Type>::BaseType)mx;
}

template <typename Type>
void ImplementQaoaLayerBasedOnCostFunction(QubitRegister<Type>& psi, QubitRegister<Type>& diag,
                                           typename QubitRegister<Type>::BaseType gamma) {
  detail::same_order(psi, diag);
  detail::check(iqsg_apply_cost_phase(psi.handle(), diag.handle(), (double)gamma));
}

template <typename Type>
typename QubitRegister<Type>::BaseType GetExpectationValueFromCostFunction(const QubitRegister<Type>& psi,
                                                                           const QubitRegister<Type>& diag) {
  detail::same_order(psi, diag);
  double v = 0;
  detail::check(iqsg_cost_expectation(detail::mut(psi).handle(), detail::mut(diag).handle(), 1, &v));
  return (typename QubitRegister<Type>::BaseType)v;
}

template <typename Type>
typename QubitRegister<Type>::BaseType GetExpectationValueSquaredFromCostFunction(const QubitRegister<Type>& psi,
                                                                                  const QubitRegister<Type>& diag) {
  detail::same_order(psi, diag);
  double v = 0;
  detail::check(iqsg_cost_expectation(detail::mut(psi).handle(), detail::mut(diag).handle(), 2, &v));
  return (typename QubitRegister<Type>::BaseType)v;
}

template <typename Type>
std::vector<typename QubitRegister<Type>::BaseType> GetHistogramFromCostFunction(const QubitRegister<Type>& psi,
                                                                                  const QubitRegister<Type>& diag,
                                                                                  int max_value) {
  return detail::histogram(psi, diag, IQSG_HIST_INTEGER, (double)max_value, 1.0, (long long)max_value + 1);
}

template <typename Type>
std::vector<typename QubitRegister<Type>::BaseType> GetHistogramFromCostFunctionWithWeightsRounded(
    const QubitRegister<Type>& psi, const QubitRegister<Type>& diag, double max_value) {
  return detail::histogram(psi, diag, IQSG_HIST_ROUNDED, max_value, 1.0, (long long)std::floor(max_value) + 1);
}

template <typename Type>
std::vector<typename QubitRegister<Type>::BaseType> GetHistogramFromCostFunctionWithWeightsBinned(
    const QubitRegister<Type>& psi, const QubitRegister<Type>& diag, double max_value, double bin_width) {
  if (!(bin_width > 0)) throw std::invalid_argument("qaoa: bin_width must be positive");
  return detail::histogram(psi, diag, IQSG_HIST_BINNED, max_value, bin_width,
                           (long long)std::ceil(max_value / bin_width) + 1);
}

}  // namespace qaoa
}  // namespace iqs
