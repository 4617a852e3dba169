// iqs_gb300/tinymatrix.hpp -- iqs::TinyMatrix, the fixed-size row-major matrix the gate API
// takes (include/tinymatrix.hpp:39-306 of intel/intel-qs), with the same members: m(i, j) and
// m[i][j] access, construction and assignment from C arrays, initializer lists and matrices of
// another alignment, element-wise == / != (also against C arrays), getPtr, getSubMatrix, print,
// tostr and the `name` string. Elements start at zero here.
#pragma once

#include <cassert>
#include <complex>
#include <cstdio>
#include <initializer_list>
#include <iostream>
#include <string>

namespace iqs {

template <class ValueType, unsigned M, unsigned N = M, unsigned align = alignof(ValueType)>
class TinyMatrix {
  static_assert(N * M != 0, "A zero-dimensional matrix is not allowed.");

 public:
  using value_type = ValueType;
  using pointer = ValueType*;
  using const_pointer = ValueType const*;
  using reference = ValueType&;
  using size_type = unsigned;
  using RowType = ValueType[N];

  TinyMatrix() {
    for (auto& r : data_)
      for (auto& x : r) x = ValueType(0);
  }
  template <class U>
  TinyMatrix(U init[M][N]) {
    for (size_type i = 0; i < M; ++i)
      for (size_type j = 0; j < N; ++j) data_[i][j] = ValueType(init[i][j]);
  }
  template <class U>
  TinyMatrix(std::initializer_list<std::initializer_list<U>> const& init) : TinyMatrix() {
    assert(init.size() == M);
    size_type i = 0;
    for (auto const& r : init) {
      assert(r.size() == N);
      size_type j = 0;
      for (auto const& x : r) data_[i][j++] = ValueType(x);
      ++i;
    }
  }
  template <class U, unsigned alignrhs>
  TinyMatrix(TinyMatrix<U, M, N, alignrhs> const& rhs) {
    for (size_type i = 0; i < M; ++i)
      for (size_type j = 0; j < N; ++j) data_[i][j] = ValueType(rhs(i, j));
  }
  TinyMatrix(TinyMatrix const&) = default;
  TinyMatrix& operator=(TinyMatrix const&) = default;
  template <class U, unsigned alignrhs>
  TinyMatrix& operator=(TinyMatrix<U, M, N, alignrhs> const& rhs) {
    for (size_type i = 0; i < M; ++i)
      for (size_type j = 0; j < N; ++j) data_[i][j] = ValueType(rhs(i, j));
    return *this;
  }
  template <class U>
  TinyMatrix& operator=(U const (&rhs)[M][N]) {
    for (size_type i = 0; i < M; ++i)
      for (size_type j = 0; j < N; ++j) data_[i][j] = ValueType(rhs[i][j]);
    return *this;
  }

  constexpr size_type numRows() const { return M; }
  constexpr size_type numCols() const { return N; }
  constexpr size_type size() const { return N * M; }

  value_type operator()(size_type i, size_type j) const {
    assert(i < M && j < N);
    return data_[i][j];
  }
  reference operator()(size_type i, size_type j) {
    assert(i < M && j < N);
    return data_[i][j];
  }
  RowType& operator[](unsigned i) {
    assert(i < M);
    return data_[i];
  }
  RowType const& operator[](unsigned i) const {
    assert(i < M);
    return data_[i];
  }

  template <class U, unsigned alignrhs>
  bool operator==(TinyMatrix<U, M, N, alignrhs> const& rhs) const {
    for (size_type i = 0; i < M; ++i)
      for (size_type j = 0; j < N; ++j)
        if (!(data_[i][j] == rhs(i, j))) return false;
    return true;
  }
  template <class U, unsigned alignrhs>
  bool operator!=(TinyMatrix<U, M, N, alignrhs> const& rhs) const {
    return !(*this == rhs);
  }
  template <class U>
  bool operator==(U const (&rhs)[M][N]) const {
    for (size_type i = 0; i < M; ++i)
      for (size_type j = 0; j < N; ++j)
        if (!(data_[i][j] == ValueType(rhs[i][j]))) return false;
    return true;
  }
  template <class U>
  bool operator!=(U const (&rhs)[M][N]) const {
    return !(*this == rhs);
  }

  const_pointer getPtr() const { return &data_[0][0]; }

  // The MSub x NSub block starting at (i_start, j_start), rows and columns taken with strides.
  template <unsigned MSub, unsigned NSub = MSub>
  TinyMatrix<ValueType, MSub, NSub, align> getSubMatrix(unsigned i_start = 0, unsigned j_start = 0,
                                                        unsigned i_stride = 1, unsigned j_stride = 1) const {
    assert(i_stride > 0 && j_stride > 0);
    assert((MSub - 1) * i_stride + i_start < M && (NSub - 1) * j_stride + j_start < N);
    TinyMatrix<ValueType, MSub, NSub, align> sub;
    for (unsigned a = 0; a < MSub; ++a)
      for (unsigned b = 0; b < NSub; ++b) sub(a, b) = data_[i_start + a * i_stride][j_start + b * j_stride];
    return sub;
  }

  // Complex element types: "name: <name>" then one line per row of "re + i*im " entries.
  void print(std::string label) {
    std::printf("name: %s\n", label.c_str());
    for (size_type i = 0; i < M; ++i) {
      for (size_type j = 0; j < N; ++j) std::cout << data_[i][j].real() << " + i*" << data_[i][j].imag() << " ";
      std::printf("\n");
    }
  }
  // Complex element types: "{{re+im ...}...{" with three decimals, as the reference prints it.
  std::string tostr() const {
    std::string str = "{";
    for (size_type i = 0; i < M; ++i) {
      str += "{";
      for (size_type j = 0; j < N; ++j) {
        char s[128];
        std::snprintf(s, sizeof s, "%.3lf+%.3lf ", (double)data_[i][j].real(), (double)data_[i][j].imag());
        str += s;
      }
      str += "}";
    }
    str += "{";
    return str;
  }

  std::string name;

 protected:
  alignas(align == 0 ? 8 : align) ValueType data_[M][N];
};

}  // namespace iqs

// The reference declares the gate-matrix aliases at global scope (include/qureg.hpp:44-48).
template <class Type>
using TM2x2 = iqs::TinyMatrix<Type, 2, 2, 32>;
template <class Type>
using TM4x4 = iqs::TinyMatrix<Type, 4, 4, 32>;
