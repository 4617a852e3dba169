/* CPU oracle for the gate-application hot path: a plain-C restatement of the
 * reference's OpenMP CPU loops (intel/intel-qs, src/highperfkernels.cpp and the
 * src/qureg_*.cpp methods cited in iqs_oracle.c).
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * legs load this library, and only as the checker or the timed CPU baseline. The
 * product (libiqsg) never links, loads or calls it.
 *
 * Layout: a register of n qubits is 2^n complex amplitudes, interleaved (re, im),
 * in data order (bit k of the index = qubit position k). Suffix _d works on
 * double (ComplexDP), _f on float (ComplexSP). Gate matrices are always passed as
 * double, row-major, interleaved: m[2*(r*dim+c)] = Re m_rc, m[2*(r*dim+c)+1] = Im m_rc;
 * the _f variants round them to float first, as TinyMatrix<ComplexSP> stores them.
 * Positions are data positions: the program-qubit -> position map is kept by the
 * caller (oracle/__init__.py restates include/permutation.hpp for that).
 */
#ifndef IQS_ORACLE_H
#define IQS_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#define OR_DECL(T, S)                                                                          \
  void or_apply1q_##S(T* s, unsigned n, unsigned pos, const double* m);                        \
  void or_ctrl1q_##S(T* s, unsigned n, unsigned cpos, unsigned tpos, const double* m);         \
  void or_apply2q_##S(T* s, unsigned n, unsigned ph, unsigned pl, const double* m);            \
  void or_swaplike_##S(T* s, unsigned n, unsigned p1, unsigned p2, const double* m);           \
  void or_diag2_##S(T* s, unsigned n, unsigned p1, unsigned p2, const double* d);              \
  void or_permute_##S(T* s, unsigned n, const unsigned* old_map, const unsigned* new_map);     \
  double or_probability_##S(const T* s, unsigned n, unsigned pos);                             \
  void or_collapse_##S(T* s, unsigned n, unsigned pos, int value);                             \
  double or_parity_sum_##S(const T* s, unsigned n, uint64_t mask);                             \
  double or_norm_##S(const T* s, unsigned n);                                                  \
  void or_overlap_##S(const T* self, const T* psi, unsigned n, double* out);                   \
  double or_max_abs_diff_##S(const T* a, const T* b, unsigned n, double sre, double sim);      \
  double or_max_l2_diff_##S(const T* a, const T* b, unsigned n);                               \
  void or_scale_##S(T* s, unsigned n, double re, double im);                                   \
  void or_axpy_##S(T* s, const T* x, unsigned n, double re, double im);                        \
  void or_fill_##S(T* s, unsigned n, double re, double im);                                    \
  void or_qaoa_layer_##S(T* psi, const T* diag, unsigned n, double gamma);                     \
  double or_qaoa_expectation_##S(const T* psi, const T* diag, unsigned n);                     \
  double or_qaoa_expectation_sq_##S(const T* psi, const T* diag, unsigned n);                  \
  int or_qaoa_maxcut_cost_##S(T* diag, unsigned n, const int* adj, const unsigned* map);       \
  double or_qaoa_weighted_cost_##S(T* diag, unsigned n, const double* adj, const unsigned* map);

OR_DECL(double, d)
OR_DECL(float, f)

/* Number of OpenMP threads the oracle's parallel loops use (0 = OpenMP default). */
void or_set_threads(int nthreads);
int or_get_threads(void);

#endif
