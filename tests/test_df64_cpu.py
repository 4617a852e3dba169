"""The emulated-FP64 arithmetic (intel-qs_gb300/csrc/df64.cuh) checked on the CPU: the same
header compiles for the host, and its split / merge / product-sum steps are compared with
exact (long double) arithmetic on random and edge-case inputs."""
import subprocess

import pytest

from conftest import REPO

SRC = r"""
#include <cstdio>
#include <cmath>
#include <random>
#include "df64.cuh"
using namespace df64;
int main() {
  std::mt19937_64 g(7);
  std::uniform_real_distribution<double> U(-1, 1);
  double split_err = 0; long split_fail = 0, merge_bad = 0;
  for (int t = 0; t < 400000; ++t) {
    double x = U(g) * std::ldexp(1.0, (int)(g() % 150) - 75);
    DF r;
    bool ok = split(x, r);
    int e = (int)((std::fabs(x) == 0) ? 0 : std::ilogb(x));
    bool expect_ok = (e >= -73 && e <= 77);
    if (ok != expect_ok) { ++split_fail; continue; }
    if (!ok) continue;
    double rel = std::fabs(((double)r.h + (double)r.l) - x) / std::fabs(x);
    if (rel > split_err) split_err = rel;
    float h = (float)x, l = (float)(x - (double)h);
    double out;
    if (merge(h, l, out) && out != (double)h + (double)l) ++merge_bad;
  }
  DF z; if (!split(0.0, z) || z.h != 0.f || z.l != 0.f) ++split_fail;
  if (!split(-0.0, z) || z.h != 0.f) ++split_fail;
  if (split(INFINITY, z) || split(NAN, z) || split(1e-300, z) || split(1e300, z)) ++split_fail;
  for (int e = -70; e < 90; ++e) for (int s = -1; s <= 1; s += 2) for (int k = -4; k <= 4; ++k) {
    float h = std::ldexp(1.0f, e) * s, l = h * std::ldexp(1.0f, -26) * k;
    double out;
    if (merge(h, l, out) && out != (double)h + (double)l) ++merge_bad;
  }
  double row_err = 0;
  for (int t = 0; t < 200000; ++t) {
    double m[4], a[4];
    for (int k = 0; k < 4; ++k) { m[k] = U(g); a[k] = U(g) * std::ldexp(1.0, -(int)(g() % 20)); }
    Acc s; float ph, pl; DF x;
    for (int k = 0; k < 4; ++k) {
      DF mm = split_host(m[k]); split(a[k], x);
      prod(mm.h, mm.l, x.h, x.l, ph, pl);
      if (k == 0) acc_init(s, ph, pl); else acc_add(s, ph, pl);
    }
    float h, l; acc_norm(s, h, l); double out; merge(h, l, out);
    long double ex = 0, mag = 0;
    for (int k = 0; k < 4; ++k) { ex += (long double)m[k] * a[k]; mag += std::fabs(m[k] * a[k]); }
    double rel = (double)(std::fabs((long double)out - ex) / mag);
    if (rel > row_err) row_err = rel;
  }
  printf("%.6e %ld %ld %.6e\n", split_err, split_fail, merge_bad, row_err);
  return 0;
}
"""


@pytest.fixture(scope="module")
def df64_results(tmp_path_factory):
    d = tmp_path_factory.mktemp("df64")
    src = d / "t.cpp"
    src.write_text(SRC)
    exe = d / "t"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(REPO / "intel-qs_gb300" / "csrc"),
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    return float(out[0]), int(out[1]), int(out[2]), float(out[3])


def test_split_is_accurate(df64_results):
    split_err, split_fail, _, _ = df64_results
    assert split_fail == 0
    assert split_err <= 2.0 ** -47


def test_merge_is_nearest_double(df64_results):
    assert df64_results[2] == 0


def test_gate_row_error_bound(df64_results):
    """A 4-term complex-gate row: error below 2^-44 of the sum of |terms|."""
    assert df64_results[3] <= 2.0 ** -44


CHAIN = r"""
#include <complex>
#include <cstdio>
#include <cmath>
#include <random>
#include <vector>
#include "df64.cuh"
using namespace df64;
using LC = std::complex<long double>;
struct CDF { DF re, im; };
// One 2x2 row (m0 a + m1 b) in double-float: four exact products per component, TwoSum sums.
static DF dot4(const DF* c, const DF* x, const float* sgn) {
  Acc s; float ph, pl;
  for (int k = 0; k < 4; ++k) {
    prod(sgn[k] * c[k].h, sgn[k] * c[k].l, x[k].h, x[k].l, ph, pl);
    if (k == 0) acc_init(s, ph, pl); else acc_add(s, ph, pl);
  }
  DF r; acc_norm(s, r.h, r.l); return r;
}
static CDF row(const CDF& m0, const CDF& m1, const CDF& a, const CDF& b) {
  const DF cr[4] = {m0.re, m0.im, m1.re, m1.im};
  const float sr[4] = {1, -1, 1, -1}, si[4] = {1, 1, 1, 1};
  const DF xr[4] = {a.re, a.im, b.re, b.im}, xi[4] = {a.im, a.re, b.im, b.re};
  return CDF{dot4(cr, xr, sr), dot4(cr, xi, si)};
}
static CDF split_c(std::complex<double> z) { CDF r; split(z.real(), r.re); split(z.imag(), r.im); return r; }
static std::complex<double> merge_c(const CDF& v) { double a, b; merge(v.re.h, v.re.l, a); merge(v.im.h, v.im.l, b); return {a, b}; }
int main() {
  const int n = 10, N = 1 << n, G = 60;
  std::mt19937_64 g(11);
  std::normal_distribution<double> nd;
  std::vector<LC> ex(N);
  std::vector<std::complex<double>> f64(N);
  std::vector<CDF> pairs(N);
  long double nrm = 0;
  for (int i = 0; i < N; ++i) { ex[i] = LC(nd(g), nd(g)); nrm += std::norm(ex[i]); }
  for (int i = 0; i < N; ++i) { ex[i] /= std::sqrt(nrm); f64[i] = std::complex<double>((double)ex[i].real(), (double)ex[i].imag()); ex[i] = LC(f64[i].real(), f64[i].imag()); pairs[i] = split_c(f64[i]); }
  for (int t = 0; t < G; ++t) {
    // Haar-like U(2) from a random complex matrix (Gram-Schmidt), the qubit at random
    std::complex<double> a(nd(g), nd(g)), b(nd(g), nd(g));
    double s = std::sqrt(std::norm(a) + std::norm(b)); a /= s; b /= s;
    std::complex<double> ph = std::polar(1.0, nd(g));
    std::complex<double> m[4] = {a, -std::conj(b) * ph, b, std::conj(a) * ph};
    int q = (int)(g() % n);
    CDF md[4]; for (int k = 0; k < 4; ++k) md[k] = CDF{split_host(m[k].real()), split_host(m[k].imag())};
    for (int i = 0; i < N; ++i) {
      if (i & (1 << q)) continue;
      int j = i | (1 << q);
      LC x = ex[i], y = ex[j];
      ex[i] = LC(m[0]) * x + LC(m[1]) * y; ex[j] = LC(m[2]) * x + LC(m[3]) * y;
      // FP64 storage: split, row, round to FP64 every gate
      CDF u = split_c(f64[i]), v = split_c(f64[j]);
      f64[i] = merge_c(row(md[0], md[1], u, v)); f64[j] = merge_c(row(md[2], md[3], u, v));
      // pair storage: rows on the pairs, no rounding in between
      CDF pu = pairs[i], pv = pairs[j];
      pairs[i] = row(md[0], md[1], pu, pv); pairs[j] = row(md[2], md[3], pu, pv);
    }
  }
  double e64 = 0, epair = 0, diff = 0;
  for (int i = 0; i < N; ++i) {
    std::complex<double> p = merge_c(pairs[i]);
    e64 = std::max(e64, (double)std::abs(LC(f64[i]) - ex[i]));
    epair = std::max(epair, (double)std::abs(LC(p) - ex[i]));
    diff = std::max(diff, std::abs(p - f64[i]));
  }
  printf("%.6e %.6e %.6e\n", e64, epair, diff);
  return 0;
}
"""


def test_pair_storage_chain_matches_fp64_storage(tmp_path):
    """60 Haar-random gates on a normalised 10-qubit state in double-float arithmetic, once
    rounding every amplitude to FP64 after each gate (FP64 storage) and once keeping the
    double-float pairs until the end (pair storage), against long double: both stay at the
    FP64 rounding level and agree with each other."""
    src = tmp_path / "chain.cpp"
    src.write_text(CHAIN)
    exe = tmp_path / "chain"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(REPO / "intel-qs_gb300" / "csrc"),
                    str(src), "-o", str(exe)], check=True)
    e64, epair, diff = map(float, subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split())
    assert e64 <= 1e-14 and epair <= 1e-14
    assert diff <= 1e-14
