// Many small circuits of different sizes in one persistent launch: forward energy and
// adjoint gradient of a hardware-efficient ansatz per instance, replayed through a CUDA graph.
//
// Instance i has n_i qubits (n_i <= 24) and L_i layers; a layer applies RZ(phi) then RY(theta)
// to every qubit and then CZ(q, q+1) for q = 0..n-2. Its observable is a sum of Pauli strings
// c_k P_k. The persistent grid pulls instances (largest first) from an atomic work counter;
// one CTA owns an instance at a time and keeps its two state vectors (psi and lambda = O psi)
// in a per-instance slice of device memory; each pass over the instance applies the rotations
// of three qubits to groups of 8 amplitudes held in registers (the CZ ladder rides on the
// pass holding the last qubit), with a CTA barrier between passes. Gradients follow the adjoint method: walking the circuit backwards,
// dE/dtheta = Im <lambda|Y_q|psi> and dE/dphi = Im <lambda|Z_q|psi> at the point after the
// gate, then the gate is undone on both vectors. All sums are FP64 in a fixed order per CTA.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "iqsg_internal.cuh"

struct iqsg_batch {
  unsigned count = 0;
  int prec = IQSG_COMPLEX_SP;
  cudaStream_t stream = nullptr;
  bool owns_stream = false;
  // device
  unsigned* d_order = nullptr;       // instance ids, largest first
  uint32_t* d_meta = nullptr;        // per instance: n, L, nterms, term offset
  uint64_t* d_state_off = nullptr;   // per instance: amplitude offset in the state buffers
  uint64_t* d_param_off = nullptr;   // per instance: parameter offset
  iqsg_pauli_term* d_terms = nullptr;
  void* d_psi = nullptr;
  void* d_lam = nullptr;
  double* d_params = nullptr;
  double* d_energy = nullptr;
  double* d_grad = nullptr;
  unsigned* d_counter = nullptr;
  unsigned long long* d_error = nullptr;
  // host (pinned staging for graph replays)
  double* h_params = nullptr;
  double* h_energy = nullptr;
  double* h_grad = nullptr;
  uint64_t nparams = 0;
  uint64_t total_amps = 0;
  unsigned threads = 512;
  unsigned ctas_per_sm = 2;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // [with_grad]
};

namespace iqsg {
namespace {

constexpr unsigned kMaxBatchQubits = 24;
constexpr unsigned kChunk = 16;  // pairs per R-precision partial of a gradient sum

template <typename R>
struct CXb {
  R re, im;
};

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < nw; ++w) r += sh[w];  // fixed order
  return r;  // valid in thread 0
}

__device__ __forceinline__ void block_sum2(double& a, double& b, double* sh) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) {
    sh[warp] = a;
    sh[32 + warp] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0.0, y = 0.0;
    for (int w = 0; w < nw; ++w) {  // fixed order
      x += sh[w];
      y += sh[32 + w];
    }
    a = x;
    b = y;
  }
}

// 2x2 of RY(theta) RZ(phi) (RZ applied first), or of its inverse.
template <typename R>
struct Mat {
  R m[8];
};

template <typename R>
__device__ __forceinline__ Mat<R> ry_rz(double theta, double phi) {
  double st, ct, sp, cp;
  sincos(0.5 * theta, &st, &ct);
  sincos(0.5 * phi, &sp, &cp);
  // RY = [[c, -s], [s, c]], RZ = diag(e^{-i p/2}, e^{i p/2}); RY RZ = [[c e^-, -s e^+], [s e^-, c e^+]]
  Mat<R> M;
  M.m[0] = (R)(ct * cp); M.m[1] = (R)(-ct * sp);
  M.m[2] = (R)(-st * cp); M.m[3] = (R)(-st * sp);
  M.m[4] = (R)(st * cp); M.m[5] = (R)(-st * sp);
  M.m[6] = (R)(ct * cp); M.m[7] = (R)(ct * sp);
  return M;
}

template <typename R>
__device__ __forceinline__ void apply2(const Mat<R>& M, CXb<R>& a, CXb<R>& b) {
  CXb<R> o0, o1;
  row2_fma<R>(M.m[0], M.m[1], M.m[2], M.m[3], a.re, a.im, b.re, b.im, o0.re, o0.im);
  row2_fma<R>(M.m[4], M.m[5], M.m[6], M.m[7], a.re, a.im, b.re, b.im, o1.re, o1.im);
  a = o0;
  b = o1;
}

constexpr int kGroupsInFlight = 2;

// Forward: RZ then RY on qubits q0 .. q0+W-1 of one layer in a single pass over groups of 2^W
// amplitudes (the W qubits' index bits), in qubit order; the layer's CZ ladder rides on the
// pass that holds the last qubit.
template <typename R, int W>
__device__ __forceinline__ void fwd_chunk(typename V2<R>::type* __restrict__ psi, uint64_t N, unsigned q0,
                                          const double* prm_l, bool last, uint64_t ladder) {
  using V = typename V2<R>::type;
  constexpr int G = 1 << W;
  Mat<R> M[W];
#pragma unroll
  for (int k = 0; k < W; ++k) M[k] = ry_rz<R>(prm_l[2 * (q0 + k) + 1], prm_l[2 * (q0 + k)]);
  const uint64_t groups = N >> W, lowmask = (uint64_t(1) << q0) - 1;
  // kGroupsInFlight groups per iteration: all their loads are issued before any arithmetic,
  // so a thread keeps that many groups' worth of loads in flight.
  for (uint64_t p0 = threadIdx.x; p0 < groups; p0 += kGroupsInFlight * blockDim.x) {
    uint64_t base[kGroupsInFlight];
    bool ok[kGroupsInFlight];
    CXb<R> a[kGroupsInFlight][G];
#pragma unroll
    for (int u = 0; u < kGroupsInFlight; ++u) {
      const uint64_t p = p0 + (uint64_t)u * blockDim.x;
      ok[u] = p < groups;
      base[u] = (p & lowmask) | ((p >> q0) << (q0 + W));
#pragma unroll
      for (int j = 0; j < G; ++j) {
        V v;
        v.x = 0;
        v.y = 0;
        if (ok[u]) v = psi[base[u] | ((uint64_t)j << q0)];
        a[u][j].re = v.x;
        a[u][j].im = v.y;
      }
    }
#pragma unroll
    for (int u = 0; u < kGroupsInFlight; ++u) {
      if (!ok[u]) continue;
#pragma unroll
      for (int k = 0; k < W; ++k)
#pragma unroll
        for (int j = 0; j < G; ++j)
          if (!(j & (1 << k))) apply2(M[k], a[u][j], a[u][j | (1 << k)]);
#pragma unroll
      for (int j = 0; j < G; ++j) {
        const uint64_t i = base[u] | ((uint64_t)j << q0);
        if (last && (__popcll(i & (i >> 1) & ladder) & 1)) {
          a[u][j].re = -a[u][j].re;
          a[u][j].im = -a[u][j].im;
        }
        V o;
        o.x = a[u][j].re;
        o.y = a[u][j].im;
        psi[i] = o;
      }
    }
  }
}

// Backward over the same W qubits (last first): undo the CZ ladder if this pass holds the last
// qubit, then per qubit the RY gradient Im <lambda|Y|psi>, undo RY, the RZ gradient
// Im <lambda|Z|psi>, undo RZ, on psi and lambda. Gradient terms are summed in R over
// kChunk groups and then in FP64 per thread; the block sums land in grd.
template <typename R, int W>
__device__ __forceinline__ void bwd_chunk(typename V2<R>::type* __restrict__ psi, typename V2<R>::type* __restrict__ lam,
                                          uint64_t N, unsigned q0, const double* prm_l, bool last, uint64_t ladder,
                                          double* grd_l, double* s_red) {
  using V = typename V2<R>::type;
  constexpr int G = 1 << W;
  R c[W], s[W], zc[W], zs[W];
#pragma unroll
  for (int k = 0; k < W; ++k) {
    double st, ct, sp, cp;
    sincos(0.5 * prm_l[2 * (q0 + k) + 1], &st, &ct);
    sincos(0.5 * prm_l[2 * (q0 + k)], &sp, &cp);
    c[k] = (R)ct;
    s[k] = (R)st;
    zc[k] = (R)cp;
    zs[k] = (R)sp;
  }
  double gy[W], gz[W];
  R cy[W], cz[W];
#pragma unroll
  for (int k = 0; k < W; ++k) {
    gy[k] = gz[k] = 0.0;
    cy[k] = cz[k] = 0;
  }
  unsigned cnt = 0;
  const uint64_t groups = N >> W, lowmask = (uint64_t(1) << q0) - 1;
  for (uint64_t p = threadIdx.x; p < groups; p += blockDim.x) {
    const uint64_t base = (p & lowmask) | ((p >> q0) << (q0 + W));
    V ps[G], ls[G];
#pragma unroll
    for (int j = 0; j < G; ++j) {
      const uint64_t i = base | ((uint64_t)j << q0);
      ps[j] = psi[i];
      ls[j] = lam[i];
      if (last && (__popcll(i & (i >> 1) & ladder) & 1)) {  // the CZ ladder is its own inverse
        ps[j].x = -ps[j].x; ps[j].y = -ps[j].y;
        ls[j].x = -ls[j].x; ls[j].y = -ls[j].y;
      }
    }
#pragma unroll
    for (int k = W - 1; k >= 0; --k) {
#pragma unroll
      for (int j = 0; j < G; ++j) {
        if (j & (1 << k)) continue;
        const int j1 = j | (1 << k);
        const V p0 = ps[j], p1 = ps[j1], l0 = ls[j], l1 = ls[j1];
        cy[k] += (l1.x * p0.x + l1.y * p0.y) - (l0.x * p1.x + l0.y * p1.y);
        V a0, a1, b0, b1;
        a0.x = c[k] * p0.x + s[k] * p1.x; a0.y = c[k] * p0.y + s[k] * p1.y;
        a1.x = c[k] * p1.x - s[k] * p0.x; a1.y = c[k] * p1.y - s[k] * p0.y;
        b0.x = c[k] * l0.x + s[k] * l1.x; b0.y = c[k] * l0.y + s[k] * l1.y;
        b1.x = c[k] * l1.x - s[k] * l0.x; b1.y = c[k] * l1.y - s[k] * l0.y;
        cz[k] += (b0.x * a0.y - b0.y * a0.x) - (b1.x * a1.y - b1.y * a1.x);
        V o;
        o.x = zc[k] * a0.x - zs[k] * a0.y; o.y = zc[k] * a0.y + zs[k] * a0.x; ps[j] = o;
        o.x = zc[k] * a1.x + zs[k] * a1.y; o.y = zc[k] * a1.y - zs[k] * a1.x; ps[j1] = o;
        o.x = zc[k] * b0.x - zs[k] * b0.y; o.y = zc[k] * b0.y + zs[k] * b0.x; ls[j] = o;
        o.x = zc[k] * b1.x + zs[k] * b1.y; o.y = zc[k] * b1.y - zs[k] * b1.x; ls[j1] = o;
      }
    }
#pragma unroll
    for (int j = 0; j < G; ++j) {
      const uint64_t i = base | ((uint64_t)j << q0);
      psi[i] = ps[j];
      lam[i] = ls[j];
    }
    if (++cnt == kChunk) {
      cnt = 0;
#pragma unroll
      for (int k = 0; k < W; ++k) {
        gy[k] += (double)cy[k];
        gz[k] += (double)cz[k];
        cy[k] = cz[k] = 0;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < W; ++k) {
    double y = gy[k] + (double)cy[k], z = gz[k] + (double)cz[k];
    block_sum2(y, z, s_red);
    if (threadIdx.x == 0) {
      grd_l[2 * (q0 + k) + 1] = y;
      grd_l[2 * (q0 + k)] = z;
    }
    __syncthreads();
  }
}

// Qubits per pass: 3 in FP32 (8-amplitude groups, 127 registers), 2 in FP64 (the 3-qubit
// FP64 variant needs 168 registers).
template <typename R>
constexpr unsigned qubits_per_pass() {
  return sizeof(R) == 4 ? 3u : 2u;
}

constexpr unsigned kBatchMaxThreads = 512;

template <typename R>
__global__ void __launch_bounds__(kBatchMaxThreads) k_batched(unsigned count, const unsigned* __restrict__ order, const uint32_t* __restrict__ meta,
                          const uint64_t* __restrict__ state_off, const uint64_t* __restrict__ param_off,
                          const iqsg_pauli_term* __restrict__ terms, typename V2<R>::type* __restrict__ psi_all,
                          typename V2<R>::type* __restrict__ lam_all, const double* __restrict__ params,
                          double* __restrict__ energy, double* __restrict__ grad, unsigned* __restrict__ counter,
                          int with_grad) {
  using V = typename V2<R>::type;
  __shared__ unsigned s_item;
  __shared__ double s_red[64];
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1u);
    __syncthreads();
    const unsigned item = s_item;
    __syncthreads();
    if (item >= count) return;
    const unsigned inst = order[item];
    const unsigned n = meta[4 * inst], L = meta[4 * inst + 1], nt = meta[4 * inst + 2], t0 = meta[4 * inst + 3];
    const uint64_t N = uint64_t(1) << n;
    V* psi = psi_all + state_off[inst];
    V* lam = lam_all + state_off[inst];
    const double* prm = params + param_off[inst];
    double* grd = grad + param_off[inst];
    const unsigned tid = threadIdx.x, nth = blockDim.x;
    const uint64_t ladder = (N >> 1) - 1;  // bits 0..n-2: CZ(q, q+1) pairs

    // ---- forward ----
    for (uint64_t x = tid; x < N; x += nth) {
      V v;
      v.x = x == 0 ? (R)1 : (R)0;
      v.y = 0;
      psi[x] = v;
    }
    __syncthreads();
    for (unsigned l = 0; l < L; ++l) {
      const double* prm_l = prm + 2 * (uint64_t)l * n;
      constexpr unsigned QP = qubits_per_pass<R>();
      for (unsigned q0 = 0; q0 < n; q0 += QP) {
        const unsigned w = n - q0 < QP ? n - q0 : QP;
        const bool last = q0 + w == n;
        if constexpr (QP == 3) {
          if (w == 3) fwd_chunk<R, 3>(psi, N, q0, prm_l, last, ladder);
          else if (w == 2) fwd_chunk<R, 2>(psi, N, q0, prm_l, last, ladder);
          else fwd_chunk<R, 1>(psi, N, q0, prm_l, last, ladder);
        } else {
          if (w == 2) fwd_chunk<R, 2>(psi, N, q0, prm_l, last, ladder);
          else fwd_chunk<R, 1>(psi, N, q0, prm_l, last, ladder);
        }
        __syncthreads();
      }
    }
    // ---- lambda = O psi, energy = Re <psi|lambda> ----
    double e = 0.0;
    for (uint64_t x = tid; x < N; x += nth) {
      double lr = 0.0, li = 0.0;
      for (unsigned k = 0; k < nt; ++k) {
        const iqsg_pauli_term T = terms[t0 + k];
        const uint64_t y = x ^ (uint64_t)T.xmask;
        const V pv = psi[y];
        // (P psi)_x = i^ny (-1)^popcount(y & zmask) psi_y
        double pr = pv.x, pi = pv.y;
        if (__popcll(y & (uint64_t)T.zmask) & 1) { pr = -pr; pi = -pi; }
        switch (T.ny & 3) {
          case 1: { const double t = pr; pr = -pi; pi = t; break; }
          case 2: pr = -pr; pi = -pi; break;
          case 3: { const double t = pr; pr = pi; pi = -t; break; }
          default: break;
        }
        lr += T.coeff * pr;
        li += T.coeff * pi;
      }
      const V pv = psi[x];
      e += (double)pv.x * lr + (double)pv.y * li;
      if (with_grad) {
        V lv;
        lv.x = (R)lr;
        lv.y = (R)li;
        lam[x] = lv;
      }
    }
    const double etot = block_sum(e, s_red);
    if (tid == 0) energy[inst] = etot;
    __syncthreads();
    if (!with_grad) continue;
    // ---- backward: the same passes, layers and qubits in reverse ----
    for (int l = (int)L - 1; l >= 0; --l) {
      const double* prm_l = prm + 2 * (uint64_t)l * n;
      double* grd_l = grd + 2 * (uint64_t)l * n;
      constexpr unsigned QP = qubits_per_pass<R>();
      const unsigned nchunks = (n + QP - 1) / QP;
      for (int c = (int)nchunks - 1; c >= 0; --c) {
        const unsigned q0 = (unsigned)c * QP;
        const unsigned w = n - q0 < QP ? n - q0 : QP;
        const bool last = q0 + w == n;
        if constexpr (QP == 3) {
          if (w == 3) bwd_chunk<R, 3>(psi, lam, N, q0, prm_l, last, ladder, grd_l, s_red);
          else if (w == 2) bwd_chunk<R, 2>(psi, lam, N, q0, prm_l, last, ladder, grd_l, s_red);
          else bwd_chunk<R, 1>(psi, lam, N, q0, prm_l, last, ladder, grd_l, s_red);
        } else {
          if (w == 2) bwd_chunk<R, 2>(psi, lam, N, q0, prm_l, last, ladder, grd_l, s_red);
          else bwd_chunk<R, 1>(psi, lam, N, q0, prm_l, last, ladder, grd_l, s_red);
        }
      }
    }
  }
}

}  // namespace
}  // namespace iqsg

using namespace iqsg;

namespace {

void batch_free(iqsg_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (auto& g : b->graph)
    if (g) cudaGraphExecDestroy(g);
  cudaFree(b->d_order);
  cudaFree(b->d_meta);
  cudaFree(b->d_state_off);
  cudaFree(b->d_param_off);
  cudaFree(b->d_terms);
  cudaFree(b->d_psi);
  cudaFree(b->d_lam);
  cudaFree(b->d_params);
  cudaFree(b->d_energy);
  cudaFree(b->d_grad);
  cudaFree(b->d_counter);
  cudaFree(b->d_error);
  cudaFreeHost(b->h_params);
  cudaFreeHost(b->h_energy);
  cudaFreeHost(b->h_grad);
  if (b->owns_stream && b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

int launch_batched(iqsg_batch* b, int with_grad) {
  const unsigned grid = (unsigned)std::min<uint64_t>((uint64_t)num_sms() * b->ctas_per_sm, b->count);
  if (b->prec == IQSG_COMPLEX_SP)
    k_batched<float><<<grid, b->threads, 0, b->stream>>>(
        b->count, b->d_order, b->d_meta, b->d_state_off, b->d_param_off, b->d_terms, static_cast<float2*>(b->d_psi),
        static_cast<float2*>(b->d_lam), b->d_params, b->d_energy, b->d_grad, b->d_counter, with_grad);
  else
    k_batched<double><<<grid, b->threads, 0, b->stream>>>(
        b->count, b->d_order, b->d_meta, b->d_state_off, b->d_param_off, b->d_terms, static_cast<double2*>(b->d_psi),
        static_cast<double2*>(b->d_lam), b->d_params, b->d_energy, b->d_grad, b->d_counter, with_grad);
  return cuda_status(cudaGetLastError(), "iqsg_batch_run: launch");
}

// Record one evaluation (parameters in, counter reset, persistent launch, results out) on
// the batch stream.
int record(iqsg_batch* b, int with_grad) {
  int st = cuda_status(cudaMemcpyAsync(b->d_params, b->h_params, b->nparams * sizeof(double), cudaMemcpyHostToDevice,
                                       b->stream), "iqsg_batch_run: params");
  if (!st) st = cuda_status(cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned), b->stream), "iqsg_batch_run: counter");
  if (!st) st = launch_batched(b, with_grad);
  if (!st) st = cuda_status(cudaMemcpyAsync(b->h_energy, b->d_energy, b->count * sizeof(double), cudaMemcpyDeviceToHost,
                                            b->stream), "iqsg_batch_run: energies");
  if (!st && with_grad)
    st = cuda_status(cudaMemcpyAsync(b->h_grad, b->d_grad, b->nparams * sizeof(double), cudaMemcpyDeviceToHost,
                                     b->stream), "iqsg_batch_run: gradients");
  return st;
}

}  // namespace

extern "C" int iqsg_batch_create(unsigned count, const unsigned* num_qubits, const unsigned* num_layers,
                                 const unsigned* terms_per_instance, const iqsg_pauli_term* terms, int precision,
                                 void* stream, iqsg_batch** out) {
  if (!out) return fail(IQSG_EINVAL, "iqsg_batch_create: null output");
  *out = nullptr;
  if (!count || !num_qubits || !num_layers || !terms_per_instance)
    return fail(IQSG_EINVAL, "iqsg_batch_create: empty batch or null array");
  if (precision != IQSG_COMPLEX_DP && precision != IQSG_COMPLEX_SP)
    return fail(IQSG_EINVAL, "iqsg_batch_create: unknown precision %d", precision);
  std::vector<uint32_t> meta(4 * (size_t)count);
  std::vector<uint64_t> soff(count), poff(count);
  uint64_t amps = 0, nparams = 0, nterms = 0;
  for (unsigned i = 0; i < count; ++i) {
    const unsigned n = num_qubits[i];
    if (n < 1 || n > kMaxBatchQubits) return fail(IQSG_EINVAL, "iqsg_batch_create: instance %u has %u qubits", i, n);
    meta[4 * i] = n;
    meta[4 * i + 1] = num_layers[i];
    meta[4 * i + 2] = terms_per_instance[i];
    meta[4 * i + 3] = (uint32_t)nterms;
    soff[i] = amps;
    poff[i] = nparams;
    amps += uint64_t(1) << n;
    nparams += 2ull * n * num_layers[i];
    nterms += terms_per_instance[i];
  }
  if (nterms && !terms) return fail(IQSG_EINVAL, "iqsg_batch_create: null Pauli terms");
  for (uint64_t k = 0; k < nterms; ++k)
    if (terms[k].ny < 0 || terms[k].ny > 3) return fail(IQSG_EINVAL, "iqsg_batch_create: term %llu has ny not in 0..3",
                                                        (unsigned long long)k);
  std::vector<unsigned> order(count);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(), [&](unsigned a, unsigned b) {
    const uint64_t wa = (uint64_t)num_layers[a] << num_qubits[a], wb = (uint64_t)num_layers[b] << num_qubits[b];
    return wa > wb;  // largest first: the tail of the queue is short work
  });
  iqsg_batch* b = new iqsg_batch;
  b->count = count;
  b->prec = precision;
  b->nparams = nparams;
  b->total_amps = amps;
  const size_t ab = precision == IQSG_COMPLEX_DP ? 16 : 8;
  int st = IQSG_OK;
  if (stream) {
    b->stream = (cudaStream_t)stream;
  } else {
    st = cuda_status(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "iqsg_batch_create: stream");
    b->owns_stream = !st;
  }
  auto dalloc = [&](void** p, size_t bytes, const char* what) {
    if (!st) st = cuda_status(cudaMalloc(p, bytes ? bytes : 8), what);
  };
  dalloc((void**)&b->d_order, count * sizeof(unsigned), "iqsg_batch_create: order");
  dalloc((void**)&b->d_meta, meta.size() * sizeof(uint32_t), "iqsg_batch_create: meta");
  dalloc((void**)&b->d_state_off, count * sizeof(uint64_t), "iqsg_batch_create: offsets");
  dalloc((void**)&b->d_param_off, count * sizeof(uint64_t), "iqsg_batch_create: offsets");
  dalloc((void**)&b->d_terms, nterms * sizeof(iqsg_pauli_term), "iqsg_batch_create: terms");
  dalloc(&b->d_psi, amps * ab, "iqsg_batch_create: psi");
  dalloc(&b->d_lam, amps * ab, "iqsg_batch_create: lambda");
  dalloc((void**)&b->d_params, nparams * sizeof(double), "iqsg_batch_create: params");
  dalloc((void**)&b->d_energy, count * sizeof(double), "iqsg_batch_create: energies");
  dalloc((void**)&b->d_grad, nparams * sizeof(double), "iqsg_batch_create: gradients");
  dalloc((void**)&b->d_counter, sizeof(unsigned), "iqsg_batch_create: counter");
  if (!st) st = cuda_status(cudaMallocHost((void**)&b->h_params, (nparams ? nparams : 1) * sizeof(double)), "pinned");
  if (!st) st = cuda_status(cudaMallocHost((void**)&b->h_energy, count * sizeof(double)), "pinned");
  if (!st) st = cuda_status(cudaMallocHost((void**)&b->h_grad, (nparams ? nparams : 1) * sizeof(double)), "pinned");
  if (!st) st = cuda_status(cudaMemcpy(b->d_order, order.data(), count * sizeof(unsigned), cudaMemcpyHostToDevice), "copy");
  if (!st) st = cuda_status(cudaMemcpy(b->d_meta, meta.data(), meta.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "copy");
  if (!st) st = cuda_status(cudaMemcpy(b->d_state_off, soff.data(), count * sizeof(uint64_t), cudaMemcpyHostToDevice), "copy");
  if (!st) st = cuda_status(cudaMemcpy(b->d_param_off, poff.data(), count * sizeof(uint64_t), cudaMemcpyHostToDevice), "copy");
  if (!st && nterms)
    st = cuda_status(cudaMemcpy(b->d_terms, terms, nterms * sizeof(iqsg_pauli_term), cudaMemcpyHostToDevice), "copy");
  if (st) {
    cudaGetLastError();
    batch_free(b);
    return st;
  }
  *out = b;
  return IQSG_OK;
}

extern "C" int iqsg_batch_destroy(iqsg_batch* b) {
  batch_free(b);
  return IQSG_OK;
}

extern "C" int iqsg_batch_set_launch(iqsg_batch* b, unsigned threads, unsigned ctas_per_sm) {
  if (!b) return fail(IQSG_EINVAL, "null batch handle");
  if (threads < 32 || threads > kBatchMaxThreads || threads % 32)
    return fail(IQSG_EINVAL, "iqsg_batch_set_launch: threads %u (32..%u, a multiple of 32)", threads, kBatchMaxThreads);
  if (ctas_per_sm < 1 || ctas_per_sm > 16) return fail(IQSG_EINVAL, "iqsg_batch_set_launch: ctas_per_sm %u", ctas_per_sm);
  b->threads = threads;
  b->ctas_per_sm = ctas_per_sm;
  for (auto& g : b->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  return IQSG_OK;
}

extern "C" int iqsg_batch_run(iqsg_batch* b, const double* params, int with_grad, double* energies, double* grads) {
  if (!b || !params || !energies || (with_grad && !grads)) return fail(IQSG_EINVAL, "iqsg_batch_run: null argument");
  std::memcpy(b->h_params, params, b->nparams * sizeof(double));
  const int wg = with_grad ? 1 : 0;
  int st = IQSG_OK;
  if (!b->graph[wg]) {
    // Capture the whole evaluation once; later calls replay it.
    cudaGraph_t g = nullptr;
    st = cuda_status(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "iqsg_batch_run: capture");
    if (!st) {
      const int rst = record(b, wg);
      const int est = cuda_status(cudaStreamEndCapture(b->stream, &g), "iqsg_batch_run: end capture");
      st = rst ? rst : est;
    }
    if (!st) st = cuda_status(cudaGraphInstantiate(&b->graph[wg], g, 0), "iqsg_batch_run: instantiate");
    if (g) cudaGraphDestroy(g);
    if (st) {
      cudaGetLastError();
      return st;
    }
  }
  st = cuda_status(cudaGraphLaunch(b->graph[wg], b->stream), "iqsg_batch_run: graph launch");
  if (!st) st = cuda_status(cudaStreamSynchronize(b->stream), "iqsg_batch_run");
  if (st) return st;
  std::memcpy(energies, b->h_energy, b->count * sizeof(double));
  if (with_grad) std::memcpy(grads, b->h_grad, b->nparams * sizeof(double));
  return IQSG_OK;
}

extern "C" int iqsg_batch_info(const iqsg_batch* b, uint64_t* num_params, uint64_t* total_amplitudes) {
  if (!b) return fail(IQSG_EINVAL, "null batch handle");
  if (num_params) *num_params = b->nparams;
  if (total_amplitudes) *total_amplitudes = b->total_amps;
  return IQSG_OK;
}
