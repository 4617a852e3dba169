// Native gate kernels: FP64 (ComplexDP) and FP32 (ComplexSP) arithmetic on HBM-resident
// amplitudes. Every kernel is a grid-stride loop over the independent amplitude groups a
// gate touches (pairs for 2x2 gates, quads for 4x4, single amplitudes for diagonals),
// enumerated by inserting zero bits at the gate's positions; each group is read once and
// written once, so each launch moves exactly the algorithmic bytes of its gate class.
#include "iqsg_internal.cuh"

namespace iqsg {

namespace {

template <typename V, typename R>
__device__ __forceinline__ V cmul(R mr, R mi, V a) {
  V r;
  cmul_fma<R>(mr, mi, a.x, a.y, r.x, r.y);
  return r;
}

// m_r0 a + m_r1 b for row r of a 2x2 matrix.
template <typename V, typename R>
__device__ __forceinline__ V row2(const M2<R>& m, int r, V a, V b) {
  V o;
  row2_fma<R>(m.re[2 * r], m.im[2 * r], m.re[2 * r + 1], m.im[2 * r + 1], a.x, a.y, b.x, b.y, o.x, o.y);
  return o;
}

__device__ __forceinline__ uint64_t insert_zeros(uint64_t x, const Positions& z) {
#pragma unroll 1
  for (unsigned k = 0; k < z.count; ++k) x = insert_zero(x, z.p[k]);
  return x;
}

__device__ __forceinline__ uint64_t gtid() { return (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ uint64_t gstride() { return (uint64_t)gridDim.x * blockDim.x; }

// ---- 1-qubit, general 2x2 (Loop_DN) ----
// U pairs per thread per iteration, all loads issued before the arithmetic.
template <typename R, int U>
__global__ void __launch_bounds__(kThreads) k_1q(typename V2<R>::type* __restrict__ s, uint64_t npairs,
                                                 unsigned pos, M2<R> m) {
  using V = typename V2<R>::type;
  const uint64_t d = uint64_t(1) << pos, stride = gstride();
  uint64_t p = gtid();
  for (; p + (U - 1) * stride < npairs; p += U * stride) {
    V a[U], b[U];
    uint64_t i0[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      i0[u] = insert_zero(p + u * stride, pos);
      a[u] = s[i0[u]];
      b[u] = s[i0[u] | d];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      s[i0[u]] = row2(m, 0, a[u], b[u]);
      s[i0[u] | d] = row2(m, 1, a[u], b[u]);
    }
  }
  for (; p < npairs; p += stride) {
    const uint64_t j0 = insert_zero(p, pos);
    V a = s[j0], b = s[j0 | d];
    s[j0] = row2(m, 0, a, b);
    s[j0 | d] = row2(m, 1, a, b);
  }
}

// ComplexSP with 16-byte accesses. pos == 0: one float4 = (a0, a1) of one pair.
// pos >= 1: two neighbouring pairs, one float4 holds their two a0, another their two a1.
template <int U>
__global__ void __launch_bounds__(kThreads) k_1q_sp_vec(float4* __restrict__ s4, uint64_t units, unsigned pos,
                                                        M2<float> m) {
  const uint64_t stride = gstride();
  uint64_t u0 = gtid();
  if (pos == 0) {
    for (; u0 < units; u0 += stride) {
      float4 v = s4[u0];
      float2 a = make_float2(v.x, v.y), b = make_float2(v.z, v.w);
      float2 r0 = row2(m, 0, a, b), r1 = row2(m, 1, a, b);
      s4[u0] = make_float4(r0.x, r0.y, r1.x, r1.y);
    }
    return;
  }
  const uint64_t d4 = (uint64_t(1) << pos) >> 1;  // partner offset in float4 units
  for (; u0 + (U - 1) * stride < units; u0 += U * stride) {
    float4 va[U], vb[U];
    uint64_t q[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      q[u] = insert_zero(2 * (u0 + u * stride), pos) >> 1;
      va[u] = s4[q[u]];
      vb[u] = s4[q[u] + d4];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      float2 a0 = make_float2(va[u].x, va[u].y), a1 = make_float2(va[u].z, va[u].w);
      float2 b0 = make_float2(vb[u].x, vb[u].y), b1 = make_float2(vb[u].z, vb[u].w);
      float2 r00 = row2(m, 0, a0, b0), r10 = row2(m, 1, a0, b0);
      float2 r01 = row2(m, 0, a1, b1), r11 = row2(m, 1, a1, b1);
      s4[q[u]] = make_float4(r00.x, r00.y, r01.x, r01.y);
      s4[q[u] + d4] = make_float4(r10.x, r10.y, r11.x, r11.y);
    }
  }
  for (; u0 < units; u0 += stride) {
    const uint64_t q = insert_zero(2 * u0, pos) >> 1;
    float4 va = s4[q], vb = s4[q + d4];
    float2 a0 = make_float2(va.x, va.y), a1 = make_float2(va.z, va.w);
    float2 b0 = make_float2(vb.x, vb.y), b1 = make_float2(vb.z, vb.w);
    float2 r00 = row2(m, 0, a0, b0), r10 = row2(m, 1, a0, b0);
    float2 r01 = row2(m, 0, a1, b1), r11 = row2(m, 1, a1, b1);
    s4[q] = make_float4(r00.x, r00.y, r01.x, r01.y);
    s4[q + d4] = make_float4(r10.x, r10.y, r11.x, r11.y);
  }
}

// ---- 1-qubit diagonal: a0 *= d0 (when touch0), a1 *= d1 ----
template <typename R>
__global__ void __launch_bounds__(kThreads) k_1q_diag(typename V2<R>::type* __restrict__ s, uint64_t npairs,
                                                      unsigned pos, C1<R> d0, C1<R> d1, bool touch0) {
  const uint64_t d = uint64_t(1) << pos;
  for (uint64_t p = gtid(); p < npairs; p += gstride()) {
    const uint64_t i0 = insert_zero(p, pos);
    if (touch0) s[i0] = cmul(d0.re, d0.im, s[i0]);
    s[i0 | d] = cmul(d1.re, d1.im, s[i0 | d]);
  }
}

// ---- (multi-)controlled 2x2: pairs with all control bits 1 (Loop_TN) ----
template <typename R>
__global__ void __launch_bounds__(kThreads) k_mc1q(typename V2<R>::type* __restrict__ s, uint64_t count,
                                                   Positions z, uint64_t ctrl, unsigned tpos, M2<R> m) {
  using V = typename V2<R>::type;
  const uint64_t d = uint64_t(1) << tpos;
  for (uint64_t p = gtid(); p < count; p += gstride()) {
    const uint64_t i0 = insert_zeros(p, z) | ctrl;
    V a = s[i0], b = s[i0 | d];
    s[i0] = row2(m, 0, a, b);
    s[i0 | d] = row2(m, 1, a, b);
  }
}

// ---- phase on the sub-block where all bits of `ones` are 1 (CZ, CPhase, Z/S/T/RZ halves) ----
template <typename R>
__global__ void __launch_bounds__(kThreads) k_phase_mask(typename V2<R>::type* __restrict__ s, uint64_t count,
                                                         Positions z, uint64_t ones, C1<R> f) {
  for (uint64_t p = gtid(); p < count; p += gstride()) {
    const uint64_t i = insert_zeros(p, z) | ones;
    s[i] = cmul(f.re, f.im, s[i]);
  }
}

// ---- dense 4x4 on quads {b, b+dl, b+dh, b+dh+dl} (Apply2QubitGate) ----
template <typename R>
__global__ void __launch_bounds__(kThreads) k_2q(typename V2<R>::type* __restrict__ s, uint64_t nquads,
                                                 unsigned plo, unsigned phi, uint64_t dh, uint64_t dl, M4<R> m) {
  using V = typename V2<R>::type;
  for (uint64_t p = gtid(); p < nquads; p += gstride()) {
    const uint64_t b = insert_zero(insert_zero(p, plo), phi);
    const uint64_t idx[4] = {b, b | dl, b | dh, b | dh | dl};
    V v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = s[idx[k]];
    const R vr[4] = {v[0].x, v[1].x, v[2].x, v[3].x}, vi[4] = {v[0].y, v[1].y, v[2].y, v[3].y};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      V o;
      row4_fma<R>(m.re + 4 * t, m.im + 4 * t, vr, vi, o.x, o.y);
      s[idx[t]] = o;
    }
  }
}

// ---- swap-type: in0 = bit plo set / phi clear, in1 = bits exchanged (ApplySwap_helper) ----
template <typename R>
__global__ void __launch_bounds__(kThreads) k_swaplike(typename V2<R>::type* __restrict__ s, uint64_t nquads,
                                                       unsigned plo, unsigned phi, M2<R> m) {
  using V = typename V2<R>::type;
  const uint64_t dlo = uint64_t(1) << plo, dhi = uint64_t(1) << phi;
  for (uint64_t p = gtid(); p < nquads; p += gstride()) {
    const uint64_t b = insert_zero(insert_zero(p, plo), phi);
    V a = s[b | dlo], c = s[b | dhi];
    s[b | dlo] = row2(m, 0, a, c);
    s[b | dhi] = row2(m, 1, a, c);
  }
}

// ---- diagonal 4-entry (ApplyDiag): amp[i] *= d[2 b(p1) + b(p2)] ----
template <typename R>
__global__ void __launch_bounds__(kThreads) k_diag2(typename V2<R>::type* __restrict__ s, uint64_t N,
                                                    unsigned p1, unsigned p2, M4<R> d) {
  for (uint64_t i = gtid(); i < N; i += gstride()) {
    const unsigned k = 2u * unsigned((i >> p1) & 1u) + unsigned((i >> p2) & 1u);
    s[i] = cmul(d.re[k], d.im[k], s[i]);
  }
}

// ---- cost-function phase: amp[i] *= (cos(g c_i), -sin(g c_i)) ----
template <typename R>
__global__ void __launch_bounds__(kThreads) k_cost_phase(typename V2<R>::type* __restrict__ s,
                                                         const typename V2<R>::type* __restrict__ diag,
                                                         uint64_t N, R gamma) {
  for (uint64_t i = gtid(); i < N; i += gstride()) {
    const R arg = gamma * diag[i].x;
    R sn, cs;
    if constexpr (sizeof(R) == 8) sincos(arg, &sn, &cs);
    else sincosf(arg, &sn, &cs);
    s[i] = cmul(cs, -sn, s[i]);
  }
}

template <typename R>
__global__ void __launch_bounds__(kThreads) k_collapse(typename V2<R>::type* __restrict__ s, uint64_t npairs,
                                                       unsigned pos, uint64_t set_bit) {
  using V = typename V2<R>::type;
  V zero;
  zero.x = 0;
  zero.y = 0;
  for (uint64_t p = gtid(); p < npairs; p += gstride()) s[insert_zero(p, pos) | set_bit] = zero;
}

template <typename R>
__global__ void __launch_bounds__(kThreads) k_scale(typename V2<R>::type* __restrict__ s, uint64_t N, C1<R> f) {
  for (uint64_t i = gtid(); i < N; i += gstride()) s[i] = cmul(f.re, f.im, s[i]);
}

template <typename R>
__global__ void __launch_bounds__(kThreads) k_axpy(typename V2<R>::type* __restrict__ s,
                                                   const typename V2<R>::type* __restrict__ x, uint64_t N,
                                                   C1<R> f, bool unit) {
  using V = typename V2<R>::type;
  for (uint64_t i = gtid(); i < N; i += gstride()) {
    V a = s[i], b = x[i];
    if (!unit) b = cmul(f.re, f.im, b);
    a.x += b.x;
    a.y += b.y;
    s[i] = a;
  }
}

template <typename R>
__global__ void __launch_bounds__(kThreads) k_fill(typename V2<R>::type* __restrict__ s, uint64_t N, C1<R> v) {
  using V = typename V2<R>::type;
  V a;
  a.x = v.re;
  a.y = v.im;
  for (uint64_t i = gtid(); i < N; i += gstride()) s[i] = a;
}

// Gather form of the qubit reorder: dst[j] = src[i(j)], bit src_bit[b] of i = bit b of j.
// Writes are coalesced; reads are scattered only along the moved positions.
struct BitMap { unsigned n; unsigned char src_bit[64]; };
template <typename R>
__global__ void __launch_bounds__(kThreads) k_permute(const typename V2<R>::type* __restrict__ src,
                                                      typename V2<R>::type* __restrict__ dst, uint64_t N, BitMap bm) {
  for (uint64_t j = gtid(); j < N; j += gstride()) {
    uint64_t i = 0;
#pragma unroll 8
    for (unsigned b = 0; b < bm.n; ++b) i |= ((j >> b) & 1u) << bm.src_bit[b];
    dst[j] = src[i];
  }
}

// MaxCut value per basis state from an edge list of (position_u, position_v, weight).
template <typename R>
__global__ void __launch_bounds__(kThreads) k_maxcut_cost(typename V2<R>::type* __restrict__ diag, uint64_t N,
                                                          const int* __restrict__ edges, unsigned num_edges) {
  extern __shared__ int sh_edges[];
  for (unsigned e = threadIdx.x; e < 3 * num_edges; e += blockDim.x) sh_edges[e] = edges[e];
  __syncthreads();
  for (uint64_t i = gtid(); i < N; i += gstride()) {
    int cut = 0;
    for (unsigned e = 0; e < num_edges; ++e) {
      const unsigned pu = (unsigned)sh_edges[3 * e], pv = (unsigned)sh_edges[3 * e + 1];
      cut += sh_edges[3 * e + 2] * int(((i >> pu) ^ (i >> pv)) & 1u);
    }
    typename V2<R>::type v;
    v.x = (R)cut;
    v.y = 0;
    diag[i] = v;
  }
}

}  // namespace

// ------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------
#define AMPS(R, h) reinterpret_cast<typename V2<R>::type*>((h)->amps)

template <typename R>
void launch_1q(iqsg_state* h, unsigned pos, const M2<R>& m) {
  const uint64_t npairs = h->N >> 1;
  if constexpr (sizeof(R) == 4) {
    if (h->N >= 4) {
      const uint64_t units = pos == 0 ? npairs : npairs >> 1;
      k_1q_sp_vec<2><<<grid_for(units, 2), kThreads, 0, h->stream>>>(reinterpret_cast<float4*>(h->amps), units, pos, m);
      return;
    }
  }
  k_1q<R, 2><<<grid_for(npairs, 2), kThreads, 0, h->stream>>>(AMPS(R, h), npairs, pos, m);
}

template <typename R>
void launch_1q_diag(iqsg_state* h, unsigned pos, C1<R> d0, C1<R> d1, bool touch0) {
  const uint64_t npairs = h->N >> 1;
  k_1q_diag<R><<<grid_for(npairs, 1), kThreads, 0, h->stream>>>(AMPS(R, h), npairs, pos, d0, d1, touch0);
}

template <typename R>
void launch_mc1q(iqsg_state* h, const Positions& z, uint64_t ctrl, unsigned tpos, const M2<R>& m) {
  const uint64_t count = h->N >> z.count;
  k_mc1q<R><<<grid_for(count, 1), kThreads, 0, h->stream>>>(AMPS(R, h), count, z, ctrl, tpos, m);
}

template <typename R>
void launch_phase_mask(iqsg_state* h, const Positions& z, uint64_t ones, C1<R> f) {
  const uint64_t count = h->N >> z.count;
  k_phase_mask<R><<<grid_for(count, 1), kThreads, 0, h->stream>>>(AMPS(R, h), count, z, ones, f);
}

template <typename R>
void launch_2q(iqsg_state* h, unsigned ph, unsigned pl, const M4<R>& m) {
  const uint64_t nq = h->N >> 2;
  const unsigned lo = ph < pl ? ph : pl, hi = ph < pl ? pl : ph;
  k_2q<R><<<grid_for(nq, 1), kThreads, 0, h->stream>>>(AMPS(R, h), nq, lo, hi, uint64_t(1) << ph,
                                                       uint64_t(1) << pl, m);
}

template <typename R>
void launch_swaplike(iqsg_state* h, unsigned plo, unsigned phi, const M2<R>& m) {
  const uint64_t nq = h->N >> 2;
  k_swaplike<R><<<grid_for(nq, 1), kThreads, 0, h->stream>>>(AMPS(R, h), nq, plo, phi, m);
}

template <typename R>
void launch_diag2(iqsg_state* h, unsigned p1, unsigned p2, const C1<R>* d) {
  M4<R> dd{};
  for (int k = 0; k < 4; ++k) { dd.re[k] = d[k].re; dd.im[k] = d[k].im; }
  k_diag2<R><<<grid_for(h->N, 1), kThreads, 0, h->stream>>>(AMPS(R, h), h->N, p1, p2, dd);
}

template <typename R>
void launch_cost_phase(iqsg_state* h, const void* diag, double gamma) {
  k_cost_phase<R><<<grid_for(h->N, 1), kThreads, 0, h->stream>>>(
      AMPS(R, h), reinterpret_cast<const typename V2<R>::type*>(diag), h->N, (R)gamma);
}

template <typename R>
void launch_collapse(iqsg_state* h, unsigned pos, int value) {
  const uint64_t npairs = h->N >> 1;
  // value = 1 keeps bit pos = 1: zero the amplitudes whose bit is 0, and vice versa.
  const uint64_t set_bit = value ? 0 : (uint64_t(1) << pos);
  k_collapse<R><<<grid_for(npairs, 1), kThreads, 0, h->stream>>>(AMPS(R, h), npairs, pos, set_bit);
}

template <typename R>
void launch_scale(iqsg_state* h, C1<R> f) {
  k_scale<R><<<grid_for(h->N, 1), kThreads, 0, h->stream>>>(AMPS(R, h), h->N, f);
}

template <typename R>
void launch_axpy(iqsg_state* h, const void* x, C1<R> f, bool unit) {
  k_axpy<R><<<grid_for(h->N, 1), kThreads, 0, h->stream>>>(
      AMPS(R, h), reinterpret_cast<const typename V2<R>::type*>(x), h->N, f, unit);
}

template <typename R>
void launch_fill(iqsg_state* h, C1<R> v) {
  k_fill<R><<<grid_for(h->N, 1), kThreads, 0, h->stream>>>(AMPS(R, h), h->N, v);
}

template <typename R>
void launch_permute(iqsg_state* h, const void* src, void* dst, const unsigned* src_bit_of_dst_bit) {
  BitMap bm{};
  bm.n = h->n;
  for (unsigned b = 0; b < h->n; ++b) bm.src_bit[b] = (unsigned char)src_bit_of_dst_bit[b];
  k_permute<R><<<grid_for(h->N, 1), kThreads, 0, h->stream>>>(
      reinterpret_cast<const typename V2<R>::type*>(src), reinterpret_cast<typename V2<R>::type*>(dst), h->N, bm);
}

template <typename R>
void launch_maxcut_cost(iqsg_state* h, const int* edges, unsigned num_edges, const unsigned*) {
  const size_t shmem = sizeof(int) * 3 * (size_t)(num_edges ? num_edges : 1);
  k_maxcut_cost<R><<<grid_for(h->N, 1), kThreads, shmem, h->stream>>>(AMPS(R, h), h->N, edges, num_edges);
}

#define INSTANTIATE(R)                                                                                  \
  template void launch_1q<R>(iqsg_state*, unsigned, const M2<R>&);                                     \
  template void launch_1q_diag<R>(iqsg_state*, unsigned, C1<R>, C1<R>, bool);                          \
  template void launch_mc1q<R>(iqsg_state*, const Positions&, uint64_t, unsigned, const M2<R>&);       \
  template void launch_phase_mask<R>(iqsg_state*, const Positions&, uint64_t, C1<R>);                  \
  template void launch_2q<R>(iqsg_state*, unsigned, unsigned, const M4<R>&);                           \
  template void launch_swaplike<R>(iqsg_state*, unsigned, unsigned, const M2<R>&);                     \
  template void launch_diag2<R>(iqsg_state*, unsigned, unsigned, const C1<R>*);                        \
  template void launch_cost_phase<R>(iqsg_state*, const void*, double);                                \
  template void launch_collapse<R>(iqsg_state*, unsigned, int);                                        \
  template void launch_scale<R>(iqsg_state*, C1<R>);                                                   \
  template void launch_axpy<R>(iqsg_state*, const void*, C1<R>, bool);                                 \
  template void launch_fill<R>(iqsg_state*, C1<R>);                                                    \
  template void launch_permute<R>(iqsg_state*, const void*, void*, const unsigned*);                   \
  template void launch_maxcut_cost<R>(iqsg_state*, const int*, unsigned, const unsigned*);

INSTANTIATE(double)
INSTANTIATE(float)

}  // namespace iqsg
