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
