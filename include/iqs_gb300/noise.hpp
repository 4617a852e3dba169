// iqs_gb300/noise.hpp -- iqs::RandomNumberGenerator<Type> and iqs::ChiMatrix over libiqsg,
// included by qureg.hpp.
//
// RandomNumberGenerator: the class of include/rng_utils.hpp (src/rng_utils.cpp:13-225 of
// intel/intel-qs) with the same methods and stream names ("pool", "state", "local"); the
// generators live in libiqsg (iqsg_rng), so the numbers are the reference's. One process is one
// state of a one-state pool.
//
// ChiMatrix: the class of include/chi_matrix.hpp. SolveEigenSystem uses libiqsg's Hermitian
// solver (the reference uses Eigen, which it does not ship): eigenvalues in increasing |E_k|,
// each eigenvector's largest component real and positive. SetEigenSystem takes a caller's
// eigensystem and normalises it as the reference does.
#pragma once

#include <cmath>
#include <complex>
#include <cstdio>
#include <initializer_list>
#include <iostream>
#include <random>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../iqsg.h"
#include "mpi_env.hpp"
#include "tinymatrix.hpp"

namespace iqs {

namespace detail {
inline void rng_check(int st) {
  if (st == IQSG_OK) return;
  if (st == IQSG_EINVAL) throw std::invalid_argument(iqsg_last_error());
  throw std::runtime_error(iqsg_last_error());
}
inline int stream_id(const std::string& shared) {
  if (shared == "pool") return 0;
  if (shared == "state") return 1;
  if (shared == "local") return 2;
  throw std::invalid_argument("random number stream must be \"pool\", \"state\" or \"local\"");
}
template <class B>
constexpr int precision_of() {
  return std::is_same<B, double>::value ? IQSG_COMPLEX_DP : IQSG_COMPLEX_SP;
}
}  // namespace detail

template <typename Type>
class RandomNumberGenerator {
  static_assert(std::is_same<Type, float>::value || std::is_same<Type, double>::value,
                "RandomNumberGenerator<float> or RandomNumberGenerator<double>");

 public:
  RandomNumberGenerator() { detail::rng_check(iqsg_rng_create(&r_)); }
  // A copy at the source's seed and stream positions (src/rng_utils.cpp:13-20).
  explicit RandomNumberGenerator(RandomNumberGenerator* source_rng) {
    detail::rng_check(iqsg_rng_clone(source_rng->r_, kPrec, &r_));
  }
  RandomNumberGenerator(const RandomNumberGenerator&) = delete;
  RandomNumberGenerator& operator=(const RandomNumberGenerator&) = delete;
  ~RandomNumberGenerator() { iqsg_rng_destroy(r_); }

  void SetSeedStreamPtrs(std::size_t seed) {
    detail::rng_check(iqsg_rng_set_seed_pool(r_, seed, (unsigned)mpi::Environment::GetNumStates(),
                                             (unsigned)mpi::Environment::GetStateId(),
                                             (unsigned)mpi::Environment::GetPoolRank()));
  }
  std::size_t GetSeed() { return info(-1); }
  void SkipAhead(std::size_t num_skip, std::string shared = "local") {
    detail::rng_check(iqsg_rng_skip(r_, kPrec, num_skip, detail::stream_id(shared)));
  }
  void UniformRandomNumbers(Type* value, std::size_t size = 1UL, Type a = 0., Type b = 1.,
                            std::string shared = "local") {
    std::vector<double> v(size);
    detail::rng_check(iqsg_rng_uniform(r_, kPrec, v.data(), size, a, b, detail::stream_id(shared)));
    for (std::size_t i = 0; i < size; ++i) value[i] = (Type)v[i];
  }
  void GaussianRandomNumbers(Type* value, std::size_t size = 1UL, std::string shared = "local") {
    std::vector<double> v(size);
    detail::rng_check(iqsg_rng_gaussian(r_, kPrec, v.data(), size, detail::stream_id(shared)));
    for (std::size_t i = 0; i < size; ++i) value[i] = (Type)v[i];
  }
  void RandomIntegersInRange(int* value, std::size_t size, int a, int b, std::string shared = "local") {
    detail::rng_check(iqsg_rng_integers(r_, kPrec, value, size, a, b, detail::stream_id(shared)));
  }
  std::size_t GetNumGeneratedOrSkippedLocalNumbers() { return info(2); }
  std::size_t GetNumGeneratedOrSkippedStateNumbers() { return info(1); }
  std::size_t GetNumGeneratedOrSkippedPoolNumbers() { return info(0); }

  iqsg_rng* handle() { return r_; }

 private:
  static constexpr int kPrec = detail::precision_of<Type>();
  std::size_t info(int which) {
    uint64_t seed = 0, counts[3] = {0, 0, 0};
    detail::rng_check(iqsg_rng_info(r_, &seed, counts));
    return which < 0 ? (std::size_t)seed : (std::size_t)counts[which];
  }
  iqsg_rng* r_ = nullptr;
};

template <class ValueType, unsigned M, unsigned align = alignof(ValueType)>
class ChiMatrix : public TinyMatrix<ValueType, M, M, align> {
  using Base = TinyMatrix<ValueType, M, M, align>;

 public:
  using value_type = ValueType;
  using BaseType = typename ValueType::value_type;
  using base_type = BaseType;
  using size_type = unsigned;

  ChiMatrix() = default;
  template <class U>
  ChiMatrix(U init[M][M]) : Base(init) {}
  template <class U>
  ChiMatrix(std::initializer_list<std::initializer_list<U>> const& init) : Base(init) {}
  // From a chi matrix of another type or alignment, with its eigensystem.
  template <class U, unsigned alignrhs>
  ChiMatrix(ChiMatrix<U, M, alignrhs> const& rhs) : Base(static_cast<TinyMatrix<U, M, M, alignrhs> const&>(rhs)) {
    for (auto const& x : rhs.GetEigenValues()) evalues_.push_back(value_type(x));
    for (auto const& x : rhs.GetEigenProbabilities()) eprobs_.push_back(base_type(x));
    for (auto const& x : rhs.GetEigenCumulativeProbabilities()) ecumprobs_.push_back(base_type(x));
    for (auto const& v : rhs.GetEigenVectors()) evectors_.emplace_back(v.begin(), v.end());
  }
  ChiMatrix(ChiMatrix const&) = default;
  ChiMatrix& operator=(ChiMatrix const&) = default;
  using Base::operator=;

  ValueType* GetPtrToData() { return &this->data_[0][0]; }

  // Eigenvalues and standardised eigenvectors, chi = sum_k E_k |E_k><E_k|, then the
  // normalisation of src/chi_matrix.cpp:166-200. chi must be Hermitian.
  void SolveEigenSystem() {
    std::vector<double> chi(2 * M * M), ev(2 * M), vecs(2 * M * M), probs(M), cum(M);
    for (unsigned i = 0; i < M; ++i)
      for (unsigned j = 0; j < M; ++j) {
        chi[2 * (i * M + j)] = this->data_[i][j].real();
        chi[2 * (i * M + j) + 1] = this->data_[i][j].imag();
      }
    detail::rng_check(iqsg_chi_eigensystem(kPrec, M, chi.data(), ev.data(), vecs.data(), probs.data(), cum.data()));
    store(ev, vecs, probs, cum);
  }
  // A caller's eigensystem (evectors[k] = eigenvector k), normalised like the reference.
  void SetEigenSystem(const std::vector<value_type>& evalues, const std::vector<std::vector<value_type>>& evectors) {
    if (evalues.size() != M || evectors.size() != M) throw std::invalid_argument("SetEigenSystem: M eigenpairs");
    std::vector<double> ev(2 * M), vecs(2 * M * M), probs(M), cum(M);
    for (unsigned k = 0; k < M; ++k) {
      ev[2 * k] = evalues[k].real();
      ev[2 * k + 1] = evalues[k].imag();
      if (evectors[k].size() != M) throw std::invalid_argument("SetEigenSystem: eigenvectors of length M");
      for (unsigned i = 0; i < M; ++i) {
        vecs[2 * (k * M + i)] = evectors[k][i].real();
        vecs[2 * (k * M + i) + 1] = evectors[k][i].imag();
      }
    }
    detail::rng_check(iqsg_chi_normalize(kPrec, M, ev.data(), vecs.data(), probs.data(), cum.data()));
    store(ev, vecs, probs, cum);
  }
  // src/chi_matrix.cpp:206-237: chi is 0.5 on {X, Z} x {X, Z}; eigenvalue 1 for (X + Z)/sqrt(2).
  void EigensystemOfIdealHadamardChannel() {
    if (M != 4) throw std::invalid_argument("EigensystemOfIdealHadamardChannel: 4x4 chi matrix expected");
    for (unsigned i = 0; i < M; ++i)
      for (unsigned j = 0; j < M; ++j) {
        const bool block = (i == 1 || i == 3) && (j == 1 || j == 3);
        if (this->data_[i][j] != (block ? value_type(0.5, 0) : value_type(0, 0)))
          throw std::invalid_argument("EigensystemOfIdealHadamardChannel: chi is not the ideal Hadamard channel");
      }
    const value_type one(1, 0), zero(0, 0), e(1 / std::sqrt(2.0), 0);
    std::vector<value_type> ev(M, zero);
    ev[0] = one;
    std::vector<std::vector<value_type>> vecs(M, std::vector<value_type>(M, zero));
    vecs[0] = {zero, e, zero, e};
    vecs[1] = {zero, e, zero, -e};
    vecs[2] = {one, zero, zero, zero};
    vecs[3] = {zero, zero, one, zero};
    SetEigenSystem(ev, vecs);
  }

  value_type GetEigenValue(size_type k) const { return evalues_.at(k); }
  std::vector<value_type> GetEigenValues() const { return evalues_; }
  base_type GetEigenProbability(size_type k) const { return eprobs_.at(k); }
  std::vector<base_type> GetEigenProbabilities() const { return eprobs_; }
  base_type GetEigenCumulativeProbability(size_type k) const { return ecumprobs_.at(k); }
  std::vector<base_type> GetEigenCumulativeProbabilities() const { return ecumprobs_; }
  std::vector<value_type> GetEigenVector(size_type k) const { return evectors_.at(k); }
  std::vector<std::vector<value_type>> GetEigenVectors() const { return evectors_; }

  // src/chi_matrix.cpp:129-160.
  void Print(bool with_eigensystem = true) {
    std::cout << "chi_matrix :\n";
    for (unsigned i = 0; i < M; ++i) {
      for (unsigned j = 0; j < M; ++j) std::cout << this->data_[i][j] << "\t";
      std::cout << "\n";
    }
    if (!with_eigensystem) return;
    std::cout << "eigenvalues :\n";
    for (auto& x : evalues_) std::cout << x << "\t";
    std::cout << "\neigenprobs :\n";
    for (auto& x : eprobs_) std::cout << x << "\t";
    for (unsigned k = 0; k < evectors_.size(); ++k) {
      std::cout << "\neigenvector " << k << " :\n";
      for (auto& x : evectors_[k]) std::cout << x << "\t";
    }
    std::cout << "\n";
  }

  // Flat arrays for iqsg_channel_gate.
  void channel_arrays(std::vector<double>& ev, std::vector<double>& cum, std::vector<double>& vecs) const {
    if (evalues_.size() != M) throw std::invalid_argument("chi matrix: no eigensystem (call SolveEigenSystem)");
    ev.assign(2 * M, 0);
    cum.assign(M, 0);
    vecs.assign(2 * M * M, 0);
    for (unsigned k = 0; k < M; ++k) {
      ev[2 * k] = evalues_[k].real();
      ev[2 * k + 1] = evalues_[k].imag();
      cum[k] = ecumprobs_[k];
      for (unsigned i = 0; i < M; ++i) {
        vecs[2 * (k * M + i)] = evectors_[k][i].real();
        vecs[2 * (k * M + i) + 1] = evectors_[k][i].imag();
      }
    }
  }

 private:
  static constexpr int kPrec = detail::precision_of<BaseType>();
  void store(const std::vector<double>& ev, const std::vector<double>& vecs, const std::vector<double>& probs,
             const std::vector<double>& cum) {
    evalues_.assign(M, value_type(0));
    evectors_.assign(M, std::vector<value_type>(M, value_type(0)));
    eprobs_.assign(M, 0);
    ecumprobs_.assign(M, 0);
    for (unsigned k = 0; k < M; ++k) {
      evalues_[k] = value_type((BaseType)ev[2 * k], (BaseType)ev[2 * k + 1]);
      eprobs_[k] = (BaseType)probs[k];
      ecumprobs_[k] = (BaseType)cum[k];
      for (unsigned i = 0; i < M; ++i)
        evectors_[k][i] = value_type((BaseType)vecs[2 * (k * M + i)], (BaseType)vecs[2 * (k * M + i) + 1]);
    }
  }
  std::vector<value_type> evalues_;
  std::vector<std::vector<value_type>> evectors_;
  std::vector<base_type> eprobs_;
  std::vector<base_type> ecumprobs_;
};

template <class Type>
using CM4x4 = ChiMatrix<Type, 4, 32>;
template <class Type>
using CM16x16 = ChiMatrix<Type, 16, 32>;

}  // namespace iqs

// The reference declares these aliases at global scope (include/qureg.hpp:51-55).
template <class Type>
using CM4x4 = iqs::ChiMatrix<Type, 4, 32>;
template <class Type>
using CM16x16 = iqs::ChiMatrix<Type, 16, 32>;
