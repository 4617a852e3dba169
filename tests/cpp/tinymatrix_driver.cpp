// The reference's TinyMatrix and ChiMatrix unit tests (unit_test/include/tinymatrix_test.hpp,
// unit_test/include/chi_matrix_test.hpp) written against the drop-in header: sizes, element
// access, construction and assignment across alignments and from C arrays and initializer
// lists, == / != and getPtr. Host code only; exits non-zero on the first failed check.
#include <complex>
#include <cstdio>

#include "iqs_gb300/qureg.hpp"

static int failures = 0;
#define CHECK(c)                                                   \
  do {                                                             \
    if (!(c)) {                                                    \
      std::fprintf(stderr, "%s:%d: %s\n", __FILE__, __LINE__, #c); \
      ++failures;                                                  \
    }                                                              \
  } while (0)

template <class Mat, class MatA>
void check_size_and_copies(Mat& mat, MatA& mata, unsigned rows, unsigned cols) {
  CHECK(mat.numRows() == rows);
  CHECK(mat.numCols() == cols);
  CHECK(mat.size() == rows * cols);
  for (unsigned i = 0; i < mat.numRows(); ++i)
    for (unsigned j = 0; j < mat.numCols(); ++j) {
      CHECK(mat[i][j] == mat(i, j));
      mat(i, j) = 1. + i + j;
    }
  Mat const& matc(mat);
  for (unsigned i = 0; i < mat.numRows(); ++i)
    for (unsigned j = 0; j < mat.numCols(); ++j) CHECK(mat(i, j) == typename Mat::value_type(1. + i + j));
  mata = mat;
  Mat matb = matc;
  MatA matd = matc;
  CHECK(matb == mat);
  CHECK(matb == mata);
  CHECK(matb == matc);
  CHECK(matc == matb);
  CHECK(matd == mat);
  CHECK(matd == mata);
  CHECK(matc == matd);
  CHECK(&mat(0, 0) == mat.getPtr());
  Mat mate, matf;
  mate = matc;
  matf = matc;
  CHECK(mat == mate);
  CHECK(mat == matf);
  mata(0, 0) = -100.;
  CHECK(mata != matc);
  CHECK(matc != mata);
}

template <class T, unsigned N, unsigned M>
void tinymatrix_testsize() {
  iqs::TinyMatrix<T, N, M> mat;
  iqs::TinyMatrix<T, N, M, 32> mata;
  check_size_and_copies(mat, mata, N, M);
}

template <class T, class Mat>
void testassign() {
  double init[2][2] = {{1., 2.}, {3., 4.}};
  Mat mat = init;
  for (unsigned i = 0; i < 2; ++i)
    for (unsigned j = 0; j < 2; ++j) CHECK(mat(i, j) == T(1. + 2. * i + j));
  Mat mat2 = {{T(1.), T(2.)}, {T(3.), T(4.)}};
  for (unsigned i = 0; i < 2; ++i)
    for (unsigned j = 0; j < 2; ++j) CHECK(mat2(i, j) == T(1. + 2. * i + j));
  CHECK(mat == init);
  CHECK(mat2 == init);
  CHECK(mat == mat2);
  CHECK(!(mat != init));
  CHECK(!(mat2 != init));
  CHECK(!(mat != mat2));
  mat = {{T(0.), T(1.)}, {T(1.), T(2.)}};
  for (unsigned i = 0; i < 2; ++i)
    for (unsigned j = 0; j < 2; ++j) CHECK(mat(i, j) == T(0. + i + j));
}

template <class T, unsigned N>
void chimatrix_testsize() {
  iqs::ChiMatrix<T, N> mat;
  iqs::ChiMatrix<T, N, 32> mata;
  check_size_and_copies(mat, mata, N, N);
}

int main() {
  tinymatrix_testsize<float, 1, 1>();
  tinymatrix_testsize<float, 1, 2>();
  tinymatrix_testsize<float, 2, 2>();
  testassign<float, iqs::TinyMatrix<float, 2>>();
  tinymatrix_testsize<int, 1, 1>();
  tinymatrix_testsize<int, 1, 2>();
  tinymatrix_testsize<int, 2, 2>();
  testassign<int, iqs::TinyMatrix<int, 2>>();
  tinymatrix_testsize<std::complex<double>, 1, 1>();
  tinymatrix_testsize<std::complex<double>, 1, 2>();
  tinymatrix_testsize<std::complex<double>, 2, 2>();
  testassign<std::complex<double>, iqs::TinyMatrix<std::complex<double>, 2>>();
  chimatrix_testsize<std::complex<double>, 1>();
  chimatrix_testsize<std::complex<double>, 2>();
  testassign<std::complex<double>, iqs::ChiMatrix<std::complex<double>, 2>>();
  // getSubMatrix with strides, tostr of a 2x2 gate matrix
  TM4x4<ComplexDP> m4;
  for (unsigned i = 0; i < 4; ++i)
    for (unsigned j = 0; j < 4; ++j) m4(i, j) = ComplexDP(i, j);
  auto sub = m4.getSubMatrix<2>(1, 0, 2, 3);
  CHECK(sub(0, 0) == ComplexDP(1, 0) && sub(0, 1) == ComplexDP(1, 3) && sub(1, 0) == ComplexDP(3, 0));
  TM2x2<ComplexDP> h = {{ComplexDP(0.5), ComplexDP(1.25)}, {ComplexDP(0, -1), ComplexDP(2)}};
  CHECK(h.tostr() == "{{0.500+0.000 1.250+0.000 }{0.000+-1.000 2.000+0.000 }{");
  // the eigen test of chimatrix_testeigen, eigenvalues only (eigenvectors are phase-free)
  iqs::ChiMatrix<ComplexDP, 2> chi2 = {{ComplexDP(1.), ComplexDP(3.)}, {ComplexDP(3.), ComplexDP(7.)}};
  chi2.SolveEigenSystem();
  CHECK(std::abs(chi2.GetEigenValue(0) - -0.24264069) < 1e-7);
  CHECK(std::abs(chi2.GetEigenValue(1) - 8.24264069) < 1e-7);
  std::printf("%d failures\n", failures);
  return failures ? 1 : 0;
}
