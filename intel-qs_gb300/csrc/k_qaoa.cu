// QAOA MaxCut circuits and their adjoint-mode gradients.
//
// Circuit: |psi> = prod_l [ exp(-i beta_l sum_q X_q) exp(-i gamma_l H_C) ] |psi0>, with
// H_C = 1/2 sum_e w_e Z_u Z_v and observable O = sum_e w_e Z_u Z_v = 2 H_C. In the
// computational basis H_C is diagonal: g(x) = W/2 - cut_w(x), W = sum_e w_e, cut_w(x) = sum
// of w_e over edges whose end bits differ. Phases exp(-i gamma g) take at most W + 1 values,
// computed once on the host in FP64 (exactly the numbers std::cos / std::sin give) and looked
// up by cut value, so the device evaluates no transcendental function.
//
// Adjoint gradient (reverse sweep over the layers): with psi and lambda = O psi taken at the
// point after a layer, dE/dbeta = 2 Im sum_q <lambda|X_q|psi> and, after the mixer has been
// undone, dE/dgamma = 2 Im <lambda|H_C|psi>. Each exp(-i beta X_q) commutes with X_q, so the
// X_q term of a qubit can be accumulated before or after its own rotation is undone; a backward
// pass therefore loads a group of 2^K amplitudes of both vectors, adds the K X_q terms, undoes
// the K rotations on both vectors, and (on the last pass of a layer) adds the H_C term and
// undoes the cost phase. Reductions accumulate in FP64 and finish in a fixed order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "iqsg_internal.cuh"

namespace iqsg {
namespace {

constexpr int kMaxEdges = 512;
constexpr int kMaxCut = 1024;  // largest total weight W

struct Graph {
  unsigned ne;
  unsigned char u[kMaxEdges], v[kMaxEdges];
  short w[kMaxEdges];
};

// Phase table: e^{-i gamma (W/2 - c)} for c = 0..W, plus the RX(2 beta) entries.
struct LayerParams {
  unsigned K;            // active positions in this pass
  unsigned pos[4];       // ascending
  double c, s;           // cos(beta), sin(beta) of exp(-i beta X) (s negated to undo it)
  int cost_pre;          // forward: apply the cost phase before the rotations
  int cost_post;         // backward: accumulate the H_C term and undo the cost phase after them
  int xterms;            // checkpointed backward: accumulate the X_q terms (lambda not yet walked back)
  int rotate;            // checkpointed backward: undo the rotations on lambda and store it
  unsigned W;
  double half_w;         // W / 2
};

__device__ __forceinline__ unsigned cut_of(uint64_t x, const Graph& G) {
  unsigned c = 0;
  for (unsigned e = 0; e < G.ne; ++e) c += (unsigned)G.w[e] * (unsigned)(((x >> G.u[e]) ^ (x >> G.v[e])) & 1u);
  return c;
}

template <typename R>
struct CX {
  R re, im;
};

template <typename R>
__device__ __forceinline__ void rx_pair(R c, R s, CX<R>& a, CX<R>& b) {
  // [[c, -i s], [-i s, c]] on (a, b)
  const CX<R> a0 = a, b0 = b;
  a.re = c * a0.re + s * b0.im;
  a.im = c * a0.im - s * b0.re;
  b.re = c * b0.re + s * a0.im;
  b.im = c * b0.im - s * a0.re;
}

template <int K>
__device__ __forceinline__ void group_index(const LayerParams& L, uint64_t g, uint64_t* idx) {
  uint64_t base = g;
#pragma unroll
  for (int k = 0; k < K; ++k) base = insert_zero(base, L.pos[k]);
#pragma unroll
  for (int s = 0; s < (1 << K); ++s) {
    uint64_t off = 0;
#pragma unroll
    for (int j = 0; j < K; ++j)
      if (s & (1 << j)) off |= uint64_t(1) << L.pos[j];
    idx[s] = base | off;
  }
}

// Forward pass: optional cost phase, then exp(-i beta X_q) on the K active positions.
// src may differ from psi (the first pass of a checkpointed layer reads the checkpoint).
template <typename R, int K>
__global__ void __launch_bounds__(kThreads) k_qaoa_fwd(typename V2<R>::type* __restrict__ psi,
                                                       const typename V2<R>::type* __restrict__ src, uint64_t ngroups,
                                                       const __grid_constant__ LayerParams L,
                                                       const __grid_constant__ Graph G,
                                                       const double2* __restrict__ table) {
  constexpr int Gs = 1 << K;
  const R c = (R)L.c, s = (R)L.s;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t idx[Gs];
    group_index<K>(L, g, idx);
    CX<R> a[Gs];
#pragma unroll
    for (int k = 0; k < Gs; ++k) {
      const auto v = src[idx[k]];
      a[k].re = v.x;
      a[k].im = v.y;
    }
    if (L.cost_pre) {
#pragma unroll
      for (int k = 0; k < Gs; ++k) {
        const double2 ph = table[cut_of(idx[k], G)];
        CX<R> o;
        cmul_fma<R>((R)ph.x, (R)ph.y, a[k].re, a[k].im, o.re, o.im);
        a[k] = o;
      }
    }
#pragma unroll
    for (int j = 0; j < K; ++j)
#pragma unroll
      for (int k = 0; k < Gs; ++k)
        if (!(k & (1 << j))) rx_pair(c, s, a[k], a[k | (1 << j)]);
#pragma unroll
    for (int k = 0; k < Gs; ++k) {
      typename V2<R>::type v;
      v.x = a[k].re;
      v.y = a[k].im;
      psi[idx[k]] = v;
    }
  }
}

__device__ __forceinline__ void block_sum2(double& a, double& b, double* out) {
  __shared__ double sh[2][kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = a;
    sh[1][threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    a = threadIdx.x < kThreads / 32 ? sh[0][threadIdx.x] : 0.0;
    b = threadIdx.x < kThreads / 32 ? sh[1][threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if (threadIdx.x == 0) {
      out[0] = a;
      out[1] = b;
    }
  }
}

// Backward pass on (psi, lambda): beta-gradient terms of the K active qubits, undo their
// rotations on both vectors; with cost_post, the gamma-gradient term and the inverse cost
// phase after them. partials[b] / partials[kMaxPartials + b]: beta / gamma sums of block b.
template <typename R, int K>
__global__ void __launch_bounds__(kThreads) k_qaoa_bwd(typename V2<R>::type* __restrict__ psi,
                                                       typename V2<R>::type* __restrict__ lam, uint64_t ngroups,
                                                       const __grid_constant__ LayerParams L,
                                                       const __grid_constant__ Graph G,
                                                       const double2* __restrict__ table,
                                                       double* __restrict__ partials) {
  constexpr int Gs = 1 << K;
  const R c = (R)L.c, s = (R)L.s;  // s already negated: the inverse rotation
  double gb = 0.0, gg = 0.0;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t idx[Gs];
    group_index<K>(L, g, idx);
    CX<R> p[Gs], l[Gs];
#pragma unroll
    for (int k = 0; k < Gs; ++k) {
      const auto v = psi[idx[k]], w = lam[idx[k]];
      p[k].re = v.x;
      p[k].im = v.y;
      l[k].re = w.x;
      l[k].im = w.y;
    }
#pragma unroll
    for (int j = 0; j < K; ++j)
#pragma unroll
      for (int k = 0; k < Gs; ++k)
        if (!(k & (1 << j))) {
          const int k1 = k | (1 << j);
          // Im(conj(l0) p1 + conj(l1) p0)
          gb += (double)l[k].re * (double)p[k1].im - (double)l[k].im * (double)p[k1].re +
                (double)l[k1].re * (double)p[k].im - (double)l[k1].im * (double)p[k].re;
        }
#pragma unroll
    for (int j = 0; j < K; ++j)
#pragma unroll
      for (int k = 0; k < Gs; ++k)
        if (!(k & (1 << j))) {
          rx_pair(c, s, p[k], p[k | (1 << j)]);
          rx_pair(c, s, l[k], l[k | (1 << j)]);
        }
    if (L.cost_post) {
#pragma unroll
      for (int k = 0; k < Gs; ++k) {
        const unsigned cut = cut_of(idx[k], G);
        const double gx = L.half_w - (double)cut;
        // Im(conj(l) g p)
        gg += gx * ((double)l[k].re * (double)p[k].im - (double)l[k].im * (double)p[k].re);
        const double2 ph = table[cut];  // e^{+i gamma g}: the inverse phase
        CX<R> o;
        cmul_fma<R>((R)ph.x, (R)ph.y, p[k].re, p[k].im, o.re, o.im);
        p[k] = o;
        cmul_fma<R>((R)ph.x, (R)ph.y, l[k].re, l[k].im, o.re, o.im);
        l[k] = o;
      }
    }
#pragma unroll
    for (int k = 0; k < Gs; ++k) {
      typename V2<R>::type v;
      v.x = p[k].re;
      v.y = p[k].im;
      psi[idx[k]] = v;
      v.x = l[k].re;
      v.y = l[k].im;
      lam[idx[k]] = v;
    }
  }
  double out[2];
  block_sum2(gb, gg, out);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = out[0];
    partials[kMaxPartials + blockIdx.x] = out[1];
  }
}

// dst = exp(-i gamma H_C) src (the after-cost checkpoint of a layer).
template <typename R>
__global__ void __launch_bounds__(kThreads) k_qaoa_cost_to(const typename V2<R>::type* __restrict__ src,
                                                           typename V2<R>::type* __restrict__ dst, uint64_t N,
                                                           const __grid_constant__ Graph G,
                                                           const double2* __restrict__ table) {
  for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < N; x += (uint64_t)gridDim.x * blockDim.x) {
    const auto v = src[x];
    const double2 ph = table[cut_of(x, G)];
    typename V2<R>::type o;
    cmul_fma<R>((R)ph.x, (R)ph.y, v.x, v.y, o.x, o.y);
    dst[x] = o;
  }
}

// Backward pass from checkpoints: psi after the mixer (pm) and after the cost phase (pc) are
// read, never changed; only lambda is walked back. The X_q terms pair lambda with pm, so they
// are taken in a first set of passes (xterms) before any rotation of the layer is undone on
// lambda; the rotate passes then undo the rotations and, on the last one, take the H_C term
// against pc and undo the cost phase.
template <typename R, int K>
__global__ void __launch_bounds__(kThreads) k_qaoa_bwd_ckpt(const typename V2<R>::type* __restrict__ pm,
                                                            const typename V2<R>::type* __restrict__ pc,
                                                            typename V2<R>::type* __restrict__ lam, uint64_t ngroups,
                                                            const __grid_constant__ LayerParams L,
                                                            const __grid_constant__ Graph G,
                                                            const double2* __restrict__ table,
                                                            double* __restrict__ partials) {
  constexpr int Gs = 1 << K;
  const R c = (R)L.c, s = (R)L.s;
  double gb = 0.0, gg = 0.0;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t idx[Gs];
    group_index<K>(L, g, idx);
    CX<R> l[Gs];
#pragma unroll
    for (int k = 0; k < Gs; ++k) {
      const auto w = lam[idx[k]];
      l[k].re = w.x;
      l[k].im = w.y;
    }
    if (L.xterms) {
#pragma unroll
      for (int j = 0; j < K; ++j)
#pragma unroll
        for (int k = 0; k < Gs; ++k)
          if (!(k & (1 << j))) {
            const int k1 = k | (1 << j);
            const auto p0 = pm[idx[k]], p1 = pm[idx[k1]];
            gb += (double)l[k].re * (double)p1.y - (double)l[k].im * (double)p1.x +
                  (double)l[k1].re * (double)p0.y - (double)l[k1].im * (double)p0.x;
          }
    }
    if (!L.rotate) continue;
#pragma unroll
    for (int j = 0; j < K; ++j)
#pragma unroll
      for (int k = 0; k < Gs; ++k)
        if (!(k & (1 << j))) rx_pair(c, s, l[k], l[k | (1 << j)]);
    if (L.cost_post) {
#pragma unroll
      for (int k = 0; k < Gs; ++k) {
        const unsigned cut = cut_of(idx[k], G);
        const double gx = L.half_w - (double)cut;
        const auto p = pc[idx[k]];
        gg += gx * ((double)l[k].re * (double)p.y - (double)l[k].im * (double)p.x);
        const double2 ph = table[cut];
        CX<R> o;
        cmul_fma<R>((R)ph.x, (R)ph.y, l[k].re, l[k].im, o.re, o.im);
        l[k] = o;
      }
    }
#pragma unroll
    for (int k = 0; k < Gs; ++k) {
      typename V2<R>::type v;
      v.x = l[k].re;
      v.y = l[k].im;
      lam[idx[k]] = v;
    }
  }
  double out[2];
  block_sum2(gb, gg, out);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = out[0];
    partials[kMaxPartials + blockIdx.x] = out[1];
  }
}

// lambda = o(x) psi with o = W - 2 cut; energy partials sum o |psi|^2.
template <typename R>
__global__ void __launch_bounds__(kThreads) k_qaoa_observable(const typename V2<R>::type* __restrict__ psi,
                                                              typename V2<R>::type* __restrict__ lam, uint64_t N,
                                                              const __grid_constant__ Graph G, double W,
                                                              double* __restrict__ partials) {
  double e = 0.0, n2 = 0.0;
  for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < N; x += (uint64_t)gridDim.x * blockDim.x) {
    const auto v = psi[x];
    const double o = W - 2.0 * (double)cut_of(x, G);
    const double a2 = (double)v.x * (double)v.x + (double)v.y * (double)v.y;
    e += o * a2;
    n2 += a2;
    if (lam) {
      typename V2<R>::type w;
      w.x = (R)(o * (double)v.x);
      w.y = (R)(o * (double)v.y);
      lam[x] = w;
    }
  }
  double out[2];
  block_sum2(e, n2, out);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = out[0];
    partials[kMaxPartials + blockIdx.x] = out[1];
  }
}

__global__ void k_finish2(const double* __restrict__ partials, int nparts, double* __restrict__ out) {
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    a += partials[i];
    b += partials[kMaxPartials + i];
  }
  double r[2];
  block_sum2(a, b, r);
  if (threadIdx.x == 0) {
    out[0] = r[0];
    out[1] = r[1];
  }
}

int make_graph(const iqsg_state* h, unsigned ne, const unsigned* uv, const int* w, Graph& G, unsigned& W) {
  if (ne > (unsigned)kMaxEdges) return fail(IQSG_EINVAL, "qaoa: at most %d edges", kMaxEdges);
  if (ne && !uv) return fail(IQSG_EINVAL, "qaoa: null edge list");
  std::memset(&G, 0, sizeof G);
  G.ne = ne;
  W = 0;
  for (unsigned e = 0; e < ne; ++e) {
    const unsigned a = uv[2 * e], b = uv[2 * e + 1];
    if (a >= h->n || b >= h->n || a == b) return fail(IQSG_EINVAL, "qaoa: edge %u (%u, %u) invalid", e, a, b);
    const int we = w ? w[e] : 1;
    if (we < 0 || we > 255) return fail(IQSG_EINVAL, "qaoa: edge weight %d not in [0, 255]", we);
    G.u[e] = (unsigned char)a;
    G.v[e] = (unsigned char)b;
    G.w[e] = (short)we;
    W += (unsigned)we;
  }
  if (W > (unsigned)kMaxCut) return fail(IQSG_EINVAL, "qaoa: total edge weight %u above %d", W, kMaxCut);
  return IQSG_OK;
}

// Device copy of the phase table e^{sign * -i gamma (W/2 - c)}, c = 0..W (in scratch).
int upload_table(iqsg_state* h, double gamma, unsigned W, double sign, double2** dev) {
  std::vector<double> t(2 * (W + 1));
  for (unsigned c = 0; c <= W; ++c) {
    const double arg = gamma * (0.5 * (double)W - (double)c);
    t[2 * c] = std::cos(arg);
    t[2 * c + 1] = -sign * std::sin(arg);
  }
  double* dst = h->scratch + kTableSlot;
  int st = cuda_status(cudaMemcpyAsync(dst, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream),
                       "qaoa: phase table");
  if (st) return st;
  // The pageable source must stay alive until the copy ran.
  st = cuda_status(cudaStreamSynchronize(h->stream), "qaoa: phase table");
  *dev = reinterpret_cast<double2*>(dst);
  return st;
}

void layer_positions(unsigned n, unsigned first, unsigned K, LayerParams& L) {
  L.K = K;
  for (unsigned k = 0; k < K; ++k) L.pos[k] = first + k;
  (void)n;
}

template <typename R, int K>
void launch_fwd(iqsg_state* h, const void* src, const LayerParams& L, const Graph& G, const double2* table) {
  const uint64_t ng = h->N >> K;
  using V = typename V2<R>::type;
  k_qaoa_fwd<R, K><<<grid_for(ng, 1), kThreads, 0, h->stream>>>(reinterpret_cast<V*>(h->amps),
                                                                  reinterpret_cast<const V*>(src), ng, L, G, table);
}

template <typename R, int K>
void launch_bwd_ckpt(iqsg_state* lam, const void* pm, const void* pc, const LayerParams& L, const Graph& G,
                     const double2* table, unsigned grid) {
  const uint64_t ng = lam->N >> K;
  using V = typename V2<R>::type;
  k_qaoa_bwd_ckpt<R, K><<<grid, kThreads, 0, lam->stream>>>(reinterpret_cast<const V*>(pm),
                                                             reinterpret_cast<const V*>(pc),
                                                             reinterpret_cast<V*>(lam->amps), ng, L, G, table,
                                                             lam->scratch);
}

template <typename R, int K>
void launch_bwd(iqsg_state* h, iqsg_state* lam, const LayerParams& L, const Graph& G, const double2* table,
                unsigned grid) {
  const uint64_t ng = h->N >> K;
  k_qaoa_bwd<R, K><<<grid, kThreads, 0, h->stream>>>(reinterpret_cast<typename V2<R>::type*>(h->amps),
                                                     reinterpret_cast<typename V2<R>::type*>(lam->amps), ng, L, G,
                                                     table, h->scratch);
}

template <typename R>
void dispatch_fwd(iqsg_state* h, const void* src, const LayerParams& L, const Graph& G, const double2* table) {
  switch (L.K) {
    case 1: launch_fwd<R, 1>(h, src, L, G, table); break;
    case 2: launch_fwd<R, 2>(h, src, L, G, table); break;
    case 3: launch_fwd<R, 3>(h, src, L, G, table); break;
  }
}

template <typename R>
void dispatch_bwd_ckpt(iqsg_state* lam, const void* pm, const void* pc, const LayerParams& L, const Graph& G,
                       const double2* table, unsigned grid) {
  switch (L.K) {
    case 1: launch_bwd_ckpt<R, 1>(lam, pm, pc, L, G, table, grid); break;
    case 2: launch_bwd_ckpt<R, 2>(lam, pm, pc, L, G, table, grid); break;
    case 3: launch_bwd_ckpt<R, 3>(lam, pm, pc, L, G, table, grid); break;
  }
}

template <typename R>
void dispatch_bwd(iqsg_state* h, iqsg_state* lam, const LayerParams& L, const Graph& G, const double2* table,
                  unsigned grid) {
  switch (L.K) {
    case 1: launch_bwd<R, 1>(h, lam, L, G, table, grid); break;
    case 2: launch_bwd<R, 2>(h, lam, L, G, table, grid); break;
    case 3: launch_bwd<R, 3>(h, lam, L, G, table, grid); break;
  }
}

int read2(iqsg_state* h, double* out, const char* what) {
  int st = cuda_status(cudaGetLastError(), what);
  if (st) return st;
  st = cuda_status(cudaMemcpyAsync(h->host_result, h->scratch + kResultSlot, 2 * sizeof(double),
                                   cudaMemcpyDeviceToHost, h->stream), what);
  if (st) return st;
  st = cuda_status(cudaStreamSynchronize(h->stream), what);
  if (st) return st;
  out[0] = h->host_result[0];
  out[1] = h->host_result[1];
  return IQSG_OK;
}

constexpr unsigned kQaoaWidth = 3;

}  // namespace
}  // namespace iqsg

using namespace iqsg;

extern "C" int iqsg_qaoa_layer(iqsg_state* h, unsigned num_edges, const unsigned* edges, const int* weights,
                               double gamma, double beta) {
  if (!h) return fail(IQSG_EINVAL, "null register handle");
  Graph G;
  unsigned W;
  int st = make_graph(h, num_edges, edges, weights, G, W);
  if (st) return st;
  double2* table = nullptr;
  if ((st = upload_table(h, gamma, W, 1.0, &table))) return st;
  const double c = std::cos(beta), s = std::sin(beta);
  for (unsigned first = 0; first < h->n; first += kQaoaWidth) {
    LayerParams L{};
    layer_positions(h->n, first, std::min(kQaoaWidth, h->n - first), L);
    L.c = c;
    L.s = s;
    L.cost_pre = first == 0;
    L.W = W;
    L.half_w = 0.5 * W;
    if (h->prec == IQSG_COMPLEX_DP) dispatch_fwd<double>(h, h->amps, L, G, table);
    else dispatch_fwd<float>(h, h->amps, L, G, table);
  }
  return cuda_status(cudaGetLastError(), "iqsg_qaoa_layer");
}

extern "C" int iqsg_qaoa_observable(iqsg_state* psi, iqsg_state* lam, unsigned num_edges, const unsigned* edges,
                                    const int* weights, double* energy, double* norm2) {
  if (!psi || !energy) return fail(IQSG_EINVAL, "iqsg_qaoa_observable: null argument");
  if (lam && (lam->n != psi->n || lam->prec != psi->prec))
    return fail(IQSG_EINVAL, "iqsg_qaoa_observable: lambda differs in size or precision");
  if (lam && lam->stream != psi->stream) cudaStreamSynchronize(lam->stream);
  Graph G;
  unsigned W;
  int st = make_graph(psi, num_edges, edges, weights, G, W);
  if (st) return st;
  unsigned grid = grid_for(psi->N, 4);
  if (grid > (unsigned)kMaxPartials) grid = kMaxPartials;
  if (psi->prec == IQSG_COMPLEX_DP)
    k_qaoa_observable<double><<<grid, kThreads, 0, psi->stream>>>(
        reinterpret_cast<const double2*>(psi->amps), lam ? reinterpret_cast<double2*>(lam->amps) : nullptr, psi->N, G,
        (double)W, psi->scratch);
  else
    k_qaoa_observable<float><<<grid, kThreads, 0, psi->stream>>>(
        reinterpret_cast<const float2*>(psi->amps), lam ? reinterpret_cast<float2*>(lam->amps) : nullptr, psi->N, G,
        (double)W, psi->scratch);
  k_finish2<<<1, kThreads, 0, psi->stream>>>(psi->scratch, (int)grid, psi->scratch + kResultSlot);
  double out[2];
  if ((st = read2(psi, out, "iqsg_qaoa_observable"))) return st;
  *energy = out[0];
  if (norm2) *norm2 = out[1];
  return IQSG_OK;
}

extern "C" int iqsg_qaoa_layer_backward(iqsg_state* psi, iqsg_state* lam, unsigned num_edges, const unsigned* edges,
                                        const int* weights, double gamma, double beta, double* grad_gamma,
                                        double* grad_beta) {
  if (!psi || !lam || !grad_gamma || !grad_beta) return fail(IQSG_EINVAL, "iqsg_qaoa_layer_backward: null argument");
  if (lam->n != psi->n || lam->prec != psi->prec)
    return fail(IQSG_EINVAL, "iqsg_qaoa_layer_backward: lambda differs in size or precision");
  if (lam->stream != psi->stream) cudaStreamSynchronize(lam->stream);
  Graph G;
  unsigned W;
  int st = make_graph(psi, num_edges, edges, weights, G, W);
  if (st) return st;
  double2* table = nullptr;
  if ((st = upload_table(psi, gamma, W, -1.0, &table))) return st;  // inverse cost phase
  const double c = std::cos(beta), s = -std::sin(beta);              // inverse rotation
  double gb = 0.0, gg = 0.0;
  for (unsigned first = 0; first < psi->n; first += kQaoaWidth) {
    LayerParams L{};
    layer_positions(psi->n, first, std::min(kQaoaWidth, psi->n - first), L);
    L.c = c;
    L.s = s;
    L.cost_post = first + kQaoaWidth >= psi->n;
    L.W = W;
    L.half_w = 0.5 * W;
    unsigned grid = grid_for(psi->N >> L.K, 1);
    if (grid > (unsigned)kMaxPartials) grid = kMaxPartials;
    if (psi->prec == IQSG_COMPLEX_DP) dispatch_bwd<double>(psi, lam, L, G, table, grid);
    else dispatch_bwd<float>(psi, lam, L, G, table, grid);
    k_finish2<<<1, kThreads, 0, psi->stream>>>(psi->scratch, (int)grid, psi->scratch + kResultSlot);
    double out[2];
    if ((st = read2(psi, out, "iqsg_qaoa_layer_backward"))) return st;
    gb += out[0];
    gg += out[1];
  }
  *grad_beta = 2.0 * gb;
  *grad_gamma = 2.0 * gg;
  return IQSG_OK;
}

namespace {
int check_same(const iqsg_state* a, const iqsg_state* b, const char* what) {
  if (!a || !b) return fail(IQSG_EINVAL, "%s: null register", what);
  if (a->n != b->n || a->prec != b->prec) return fail(IQSG_EINVAL, "%s: registers differ in size or precision", what);
  return IQSG_OK;
}
}  // namespace

extern "C" int iqsg_qaoa_layer_ckpt(iqsg_state* h, iqsg_state* after_cost, iqsg_state* after_mixer, unsigned num_edges,
                                    const unsigned* edges, const int* weights, double gamma, double beta) {
  int st = check_same(h, after_cost, "iqsg_qaoa_layer_ckpt");
  if (!st) st = check_same(h, after_mixer, "iqsg_qaoa_layer_ckpt");
  if (st) return st;
  for (iqsg_state* o : {after_cost, after_mixer})
    if (o->stream != h->stream) cudaStreamSynchronize(o->stream);
  Graph G;
  unsigned W;
  if ((st = make_graph(h, num_edges, edges, weights, G, W))) return st;
  double2* table = nullptr;
  if ((st = upload_table(h, gamma, W, 1.0, &table))) return st;
  unsigned grid = grid_for(h->N, 1);
  if (h->prec == IQSG_COMPLEX_DP)
    k_qaoa_cost_to<double><<<grid, kThreads, 0, h->stream>>>(reinterpret_cast<const double2*>(h->amps),
                                                             reinterpret_cast<double2*>(after_cost->amps), h->N, G, table);
  else
    k_qaoa_cost_to<float><<<grid, kThreads, 0, h->stream>>>(reinterpret_cast<const float2*>(h->amps),
                                                            reinterpret_cast<float2*>(after_cost->amps), h->N, G, table);
  const double c = std::cos(beta), s = std::sin(beta);
  for (unsigned first = 0; first < h->n; first += kQaoaWidth) {
    LayerParams L{};
    layer_positions(h->n, first, std::min(kQaoaWidth, h->n - first), L);
    L.c = c;
    L.s = s;
    const void* src = first == 0 ? after_cost->amps : h->amps;  // first pass reads the checkpoint
    if (h->prec == IQSG_COMPLEX_DP) dispatch_fwd<double>(h, src, L, G, table);
    else dispatch_fwd<float>(h, src, L, G, table);
  }
  const size_t bytes = h->N * (h->prec == IQSG_COMPLEX_DP ? 16 : 8);
  st = cuda_status(cudaMemcpyAsync(after_mixer->amps, h->amps, bytes, cudaMemcpyDeviceToDevice, h->stream),
                   "iqsg_qaoa_layer_ckpt");
  if (st) return st;
  if (after_mixer->stream != h->stream || after_cost->stream != h->stream) cudaStreamSynchronize(h->stream);
  return cuda_status(cudaGetLastError(), "iqsg_qaoa_layer_ckpt");
}

extern "C" int iqsg_qaoa_layer_backward_ckpt(iqsg_state* lam, const iqsg_state* after_cost,
                                             const iqsg_state* after_mixer, unsigned num_edges, const unsigned* edges,
                                             const int* weights, double gamma, double beta, double* grad_gamma,
                                             double* grad_beta) {
  int st = check_same(lam, after_cost, "iqsg_qaoa_layer_backward_ckpt");
  if (!st) st = check_same(lam, after_mixer, "iqsg_qaoa_layer_backward_ckpt");
  if (st) return st;
  if (!grad_gamma || !grad_beta) return fail(IQSG_EINVAL, "iqsg_qaoa_layer_backward_ckpt: null output");
  for (const iqsg_state* o : {after_cost, after_mixer})
    if (o->stream != lam->stream) cudaStreamSynchronize(o->stream);
  Graph G;
  unsigned W;
  if ((st = make_graph(lam, num_edges, edges, weights, G, W))) return st;
  double2* table = nullptr;
  if ((st = upload_table(lam, gamma, W, -1.0, &table))) return st;
  const double c = std::cos(beta), s = -std::sin(beta);
  double gb = 0.0, gg = 0.0;
  for (int phase = 0; phase < 2; ++phase) {  // 0: X_q terms, 1: undo the rotations (+ H_C term)
    for (unsigned first = 0; first < lam->n; first += kQaoaWidth) {
      LayerParams L{};
      layer_positions(lam->n, first, std::min(kQaoaWidth, lam->n - first), L);
      L.c = c;
      L.s = s;
      L.xterms = phase == 0;
      L.rotate = phase == 1;
      L.cost_post = phase == 1 && first + kQaoaWidth >= lam->n;
      L.W = W;
      L.half_w = 0.5 * W;
      unsigned grid = grid_for(lam->N >> L.K, 1);
      if (grid > (unsigned)kMaxPartials) grid = kMaxPartials;
      if (lam->prec == IQSG_COMPLEX_DP)
        dispatch_bwd_ckpt<double>(lam, after_mixer->amps, after_cost->amps, L, G, table, grid);
      else
        dispatch_bwd_ckpt<float>(lam, after_mixer->amps, after_cost->amps, L, G, table, grid);
      if (!L.xterms && !L.cost_post) continue;  // nothing summed in this pass
      k_finish2<<<1, kThreads, 0, lam->stream>>>(lam->scratch, (int)grid, lam->scratch + kResultSlot);
      double out[2];
      if ((st = read2(lam, out, "iqsg_qaoa_layer_backward_ckpt"))) return st;
      gb += out[0];
      gg += out[1];
    }
  }
  *grad_beta = 2.0 * gb;
  *grad_gamma = 2.0 * gg;
  return IQSG_OK;
}
