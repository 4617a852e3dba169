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
