// ComplexDP gate kernels in emulated FP64 (double-float on the FP32 pipe, see df64.cuh).
// The amplitudes are IEEE FP64 in HBM before and after; a pair whose inputs or outputs
// leave the fast range is recomputed in native FP64 by the same thread.
#include "df64.cuh"
#include "iqsg_internal.cuh"

namespace iqsg {

namespace {

using df64::DF;

// 2x2 complex matrix as double-float constants: for entry k (m00, m01, m10, m11)
// re = (rh, rl), im = (ih, il), and the negated imaginary part for the real rows.
struct DFM2 {
  float rh[4], rl[4], ih[4], il[4];
};

__device__ __forceinline__ void dot4(float& oh, float& ol, const float* mh, const float* ml, const DF* x) {
  float ph, pl;
  df64::Acc s;
  df64::prod(mh[0], ml[0], x[0].h, x[0].l, ph, pl);
  df64::acc_init(s, ph, pl);
#pragma unroll
  for (int k = 1; k < 4; ++k) {
    df64::prod(mh[k], ml[k], x[k].h, x[k].l, ph, pl);
    df64::acc_add(s, ph, pl);
  }
  df64::acc_norm(s, oh, ol);
}

// One output amplitude of row r: m_r0 a + m_r1 b, a = (x[0], x[1]), b = (x[2], x[3]).
__device__ __forceinline__ bool row_df(const DFM2& m, int r, const DF* x, double2& out) {
  const int k0 = 2 * r, k1 = 2 * r + 1;
  // re = m0r a.re - m0i a.im + m1r b.re - m1i b.im
  const float reh[4] = {m.rh[k0], -m.ih[k0], m.rh[k1], -m.ih[k1]};
  const float rel[4] = {m.rl[k0], -m.il[k0], m.rl[k1], -m.il[k1]};
  // im = m0r a.im + m0i a.re + m1r b.im + m1i b.re
  const float imh[4] = {m.rh[k0], m.ih[k0], m.rh[k1], m.ih[k1]};
  const float iml[4] = {m.rl[k0], m.il[k0], m.rl[k1], m.il[k1]};
  const DF xr[4] = {x[0], x[1], x[2], x[3]};
  const DF xi[4] = {x[1], x[0], x[3], x[2]};
  float h, l;
  dot4(h, l, reh, rel, xr);
  bool ok = df64::merge(h, l, out.x);
  dot4(h, l, imh, iml, xi);
  ok &= df64::merge(h, l, out.y);
  return ok;
}

__device__ __forceinline__ double2 row_native(const M2<double>& m, int r, double2 a, double2 b) {
  double2 o;
  o.x = m.re[2 * r] * a.x - m.im[2 * r] * a.y + m.re[2 * r + 1] * b.x - m.im[2 * r + 1] * b.y;
  o.y = m.re[2 * r] * a.y + m.im[2 * r] * a.x + m.re[2 * r + 1] * b.y + m.im[2 * r + 1] * b.x;
  return o;
}

__device__ __forceinline__ void pair_update(const DFM2& m, const M2<double>& md, double2& a, double2& b) {
  DF x[4];
  bool ok = df64::split(a.x, x[0]);
  ok &= df64::split(a.y, x[1]);
  ok &= df64::split(b.x, x[2]);
  ok &= df64::split(b.y, x[3]);
  double2 r0, r1;
  ok &= row_df(m, 0, x, r0);
  ok &= row_df(m, 1, x, r1);
  if (!ok) {  // outside the fast range: native FP64 for this pair
    r0 = row_native(md, 0, a, b);
    r1 = row_native(md, 1, a, b);
  }
  a = r0;
  b = r1;
}

template <int U>
__global__ void __launch_bounds__(kThreads) k_1q_df(double2* __restrict__ s, uint64_t npairs, unsigned pos,
                                                    DFM2 m, M2<double> md) {
  const uint64_t d = uint64_t(1) << pos, stride = (uint64_t)gridDim.x * blockDim.x;
  uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; p + (U - 1) * stride < npairs; p += U * stride) {
    double2 a[U], b[U];
    uint64_t i0[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      i0[u] = insert_zero(p + u * stride, pos);
      a[u] = s[i0[u]];
      b[u] = s[i0[u] | d];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      pair_update(m, md, a[u], b[u]);
      s[i0[u]] = a[u];
      s[i0[u] | d] = b[u];
    }
  }
  for (; p < npairs; p += stride) {
    const uint64_t j0 = insert_zero(p, pos);
    double2 a = s[j0], b = s[j0 | d];
    pair_update(m, md, a, b);
    s[j0] = a;
    s[j0 | d] = b;
  }
}

DFM2 split_matrix(const M2<double>& m) {
  DFM2 r;
  for (int k = 0; k < 4; ++k) {
    const DF re = df64::split_host(m.re[k]), im = df64::split_host(m.im[k]);
    r.rh[k] = re.h;
    r.rl[k] = re.l;
    r.ih[k] = im.h;
    r.il[k] = im.l;
  }
  return r;
}

}  // namespace

void launch_1q_emulated(iqsg_state* h, unsigned pos, const M2<double>& m) {
  const uint64_t npairs = h->N >> 1;
  k_1q_df<2><<<grid_for(npairs, 2), kThreads, 0, h->stream>>>(reinterpret_cast<double2*>(h->amps), npairs, pos,
                                                              split_matrix(m), m);
}

}  // namespace iqsg
