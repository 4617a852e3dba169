// Fused-sweep kernel and the scheduler that packs a gate stream into sweeps (iqsg_apply_ops).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "bulk.cuh"
#include "scheduler.h"
#include "sweep.cuh"

namespace iqsg {

namespace {

__device__ __forceinline__ uint64_t gtid() { return (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ uint64_t gstride() { return (uint64_t)gridDim.x * blockDim.x; }

template <int K>
__device__ __forceinline__ void group_indices(const SweepParams& P, uint64_t g, uint64_t* idx) {
  uint64_t base = g;
#pragma unroll
  for (int k = 0; k < K; ++k) base = insert_zero(base, P.sorted[k]);
#pragma unroll
  for (int s = 0; s < (1 << K); ++s) {
    uint64_t off = 0;
#pragma unroll
    for (int j = 0; j < K; ++j)
      if (s & (1 << j)) off |= uint64_t(1) << P.pos[j];
    idx[s] = base | off;
  }
}

// IEEE arithmetic in the storage precision.
template <typename R, int K>
__global__ void __launch_bounds__(kThreads) k_sweep_native(typename V2<R>::type* __restrict__ s, uint64_t ngroups,
                                                           const __grid_constant__ SweepParams P) {
  constexpr int G = 1 << K;
  using A = NativeArith<R>;
  for (uint64_t g = gtid(); g < ngroups; g += gstride()) {
    uint64_t idx[G];
    group_indices<K>(P, g, idx);
    typename A::VT v[G];
#pragma unroll
    for (int k = 0; k < G; ++k) {
      const auto a = s[idx[k]];
      v[k].re = a.x;
      v[k].im = a.y;
    }
    unsigned tm = 0;
    run_ops<A, K>(P, v, idx, tm);
#pragma unroll
    for (int k = 0; k < G; ++k) {
      if (!(tm & (1u << k))) continue;
      typename V2<R>::type a;
      a.x = v[k].re;
      a.y = v[k].im;
      s[idx[k]] = a;
    }
  }
}

// FP64 storage, double-float arithmetic; a group with a value outside the fast range is
// recomputed in native FP64. Untouched slots are not rewritten. With P.native16 > 0, whole
// warps (a fixed share of the group blocks) take the native FP64 path from the start, so the
// FP64 pipe works alongside the FP32 pipes that carry the double-float arithmetic.
// With only_if set, the kernel runs only when *only_if is nonzero (the state failed the
// double-float range check of a double-float storage run, see k_sweep_dfs).
template <int K>
__global__ void __launch_bounds__(kThreads) k_sweep_df(double2* __restrict__ s, uint64_t ngroups,
                                                       const __grid_constant__ SweepParams P,
                                                       const unsigned long long* __restrict__ only_if) {
  if (only_if && !*only_if) return;
  constexpr int G = 1 << K;
  for (uint64_t g = gtid(); g < ngroups; g += gstride()) {
    uint64_t idx[G];
    group_indices<K>(P, g, idx);
    double2 raw[G];
#pragma unroll
    for (int k = 0; k < G; ++k) raw[k] = s[idx[k]];
    DF64Arith::VT v[G];
    bool ok = ((g >> 5) & 15) >= P.native16;  // warp-uniform: gstride and the block size are multiples of 32
    if (ok) {
#pragma unroll
      for (int k = 0; k < G; ++k) {
        ok &= df64::split(raw[k].x, v[k].re);
        ok &= df64::split(raw[k].y, v[k].im);
      }
    }
    unsigned tm = 0;
    double2 out[G];
    if (ok) {
      run_ops<DF64Arith, K>(P, v, idx, tm);
#pragma unroll
      for (int k = 0; k < G; ++k) {
        if (tm & (1u << k)) {
          ok &= df64::merge(v[k].re.h, v[k].re.l, out[k].x);
          ok &= df64::merge(v[k].im.h, v[k].im.l, out[k].y);
        }
      }
    }
    if (!ok) {
      NativeArith<double>::VT w[G];
#pragma unroll
      for (int k = 0; k < G; ++k) {
        w[k].re = raw[k].x;
        w[k].im = raw[k].y;
      }
      tm = 0;
      run_ops<NativeArith<double>, K>(P, w, idx, tm);
#pragma unroll
      for (int k = 0; k < G; ++k) {
        out[k].x = w[k].re;
        out[k].y = w[k].im;
      }
    }
#pragma unroll
    for (int k = 0; k < G; ++k)
      if (tm & (1u << k)) s[idx[k]] = out[k];
  }
}

// ---- double-float storage runs ----------------------------------------------------------------
//
// A stream of emulated-FP64 sweeps keeps the state as double-float pairs between sweeps: each
// amplitude's 16 bytes hold (re.h, re.l, im.h, im.l) as four floats instead of two doubles. The
// first sweep reads FP64 and writes pairs, the middle ones read and write pairs, the last one
// writes FP64 again, so the split and the rounding back to FP64 happen once per run instead of
// once per sweep. Every value of the run is a double-float value; where a value fits FP64 this
// is the same number the per-sweep rounding would store, to within the last of its 53 bits.
//
// Range: pairs of floats cover |x| < 2^128, so a run starts only when every component is below
// 2^77 and finite (k_df_range) and every gate of the run is contractive (checked on the host),
// which bounds every value of the run by the state's norm. If the check fails on the device,
// the pair kernels return at once and the IEEE kernel k_sweep_df does each sweep instead.

// Sets *bad when a component is Inf, NaN or at least 2^77 in magnitude.
__global__ void __launch_bounds__(kThreads) k_df_range(const double2* __restrict__ s, uint64_t n,
                                                       unsigned long long* __restrict__ bad) {
  bool b = false;
  for (uint64_t i = gtid(); i < n; i += gstride()) {
    const double2 v = s[i];
    const uint32_t ex = (uint32_t)(df64::d2u(v.x) >> 52) & 0x7FFu, ey = (uint32_t)(df64::d2u(v.y) >> 52) & 0x7FFu;
    b |= (ex >= df64::kEmax) | (ey >= df64::kEmax);
  }
  if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31u) == 0u) atomicOr(bad, 1ull);
}

// FP64 -> pairs for the values the integer split does not take (|x| < 2^-73, the range check
// having excluded large ones), and pairs -> FP64 where the integer rounding does not apply.
// Called under a warp-uniform branch, so the fast path does not issue their FP64
// instructions predicated off.
template <int G>
__device__ __forceinline__ void split_slow(const double2* raw, DF64Arith::VT* v) {
#pragma unroll
  for (int k = 0; k < G; ++k) {
    v[k].re.h = __double2float_rn(raw[k].x);
    v[k].re.l = __double2float_rn(raw[k].x - (double)v[k].re.h);
    v[k].im.h = __double2float_rn(raw[k].y);
    v[k].im.l = __double2float_rn(raw[k].y - (double)v[k].im.h);
  }
}
template <int G>
__device__ __forceinline__ void merge_slow(const DF64Arith::VT* v, double2* out) {
#pragma unroll
  for (int k = 0; k < G; ++k) {
    out[k].x = (double)v[k].re.h + (double)v[k].re.l;
    out[k].y = (double)v[k].im.h + (double)v[k].im.l;
  }
}

// Resident blocks per SM the pair kernels are compiled for (register budget), by width. On
// GB300 (30-qubit layer): width 2 is fastest at 4 blocks (64 registers; 48 registers with 5
// blocks spill and lose 4 %); width 3 gains 24 % at 3 blocks (80 registers, 64 bytes of
// spills) over 2 blocks (128 registers).
#ifndef IQSG_DFS_MIN_BLOCKS_K2
#define IQSG_DFS_MIN_BLOCKS_K2 4
#endif
#ifndef IQSG_DFS_MIN_BLOCKS_K3
#define IQSG_DFS_MIN_BLOCKS_K3 3
#endif
template <int K>
constexpr int dfs_min_blocks() {
  return K == 3 ? IQSG_DFS_MIN_BLOCKS_K3 : (K == 2 ? IQSG_DFS_MIN_BLOCKS_K2 : 1);
}

template <int K, bool IN_PAIRS, bool OUT_PAIRS>
__global__ void __launch_bounds__(kThreads, dfs_min_blocks<K>()) k_sweep_dfs(double2* __restrict__ s, uint64_t ngroups,
                                                        const __grid_constant__ SweepParams P,
                                                        const unsigned long long* __restrict__ bad) {
  if (*bad) return;
  constexpr int G = 1 << K;
  // A sweep that changes the format rewrites every slot; one that keeps it, only touched ones.
  constexpr bool kAll = IN_PAIRS != OUT_PAIRS;
  float4* f = reinterpret_cast<float4*>(s);
  for (uint64_t g = gtid(); g < ngroups; g += gstride()) {
    uint64_t idx[G];
    group_indices<K>(P, g, idx);
    DF64Arith::VT v[G];
    if constexpr (IN_PAIRS) {
#pragma unroll
      for (int k = 0; k < G; ++k) {
        const float4 t = f[idx[k]];
        v[k].re = df64::DF{t.x, t.y};
        v[k].im = df64::DF{t.z, t.w};
      }
    } else {
      double2 raw[G];
      bool ok = true;
#pragma unroll
      for (int k = 0; k < G; ++k) {
        raw[k] = s[idx[k]];
        ok &= df64::split(raw[k].x, v[k].re);
        ok &= df64::split(raw[k].y, v[k].im);
      }
      if (__builtin_expect(__any_sync(__activemask(), !ok), 0)) {
        if (!ok) split_slow<G>(raw, v);
      }
    }
    unsigned tm = 0;
    run_ops<DF64Arith, K>(P, v, idx, tm);
    if constexpr (OUT_PAIRS) {
#pragma unroll
      for (int k = 0; k < G; ++k)
        if (kAll || (tm & (1u << k))) f[idx[k]] = make_float4(v[k].re.h, v[k].re.l, v[k].im.h, v[k].im.l);
    } else {
      double2 out[G];
      bool ok = true;
#pragma unroll
      for (int k = 0; k < G; ++k) {
        ok &= df64::merge(v[k].re.h, v[k].re.l, out[k].x);
        ok &= df64::merge(v[k].im.h, v[k].im.l, out[k].y);
      }
      if (__builtin_expect(__any_sync(__activemask(), !ok), 0)) {
        if (!ok) merge_slow<G>(v, out);
      }
#pragma unroll
      for (int k = 0; k < G; ++k)
        if (kAll || (tm & (1u << k))) s[idx[k]] = out[k];
    }
  }
}

// ---- adjoint sweep: psi and lambda together, gradient sums per slot -------------------------
//
// Gradient terms are summed in R over kGradChunk groups, then moved into FP64 per thread;
// per-block sums (fixed-order warp and block trees) land in partials[block * kGradSlots + s].
// The grid is fixed by the register size, so the order of every sum is too.
constexpr unsigned kGradChunk = 16;
constexpr unsigned kAdjBlocksPerSm = 2;

template <typename R, int K>
__global__ void __launch_bounds__(kThreads) k_sweep_adj(typename V2<R>::type* __restrict__ psi,
                                                        typename V2<R>::type* __restrict__ lam, uint64_t ngroups,
                                                        const __grid_constant__ SweepParams P, unsigned nslots,
                                                        double* __restrict__ partials) {
  constexpr int G = 1 << K;
  using A = NativeArith<R>;
  R racc[kGradSlots];
  double dacc[kGradSlots];
#pragma unroll
  for (int k = 0; k < kGradSlots; ++k) {
    racc[k] = 0;
    dacc[k] = 0.0;
  }
  unsigned cnt = 0;
  for (uint64_t g = gtid(); g < ngroups; g += gstride()) {
    uint64_t idx[G];
    group_indices<K>(P, g, idx);
    typename A::VT v[G], w[G];
#pragma unroll
    for (int k = 0; k < G; ++k) {
      const auto a = psi[idx[k]], b = lam[idx[k]];
      v[k].re = a.x;
      v[k].im = a.y;
      w[k].re = b.x;
      w[k].im = b.y;
    }
    unsigned tm = 0;
    run_ops_dual<R, K>(P, v, w, idx, tm, racc);
#pragma unroll
    for (int k = 0; k < G; ++k) {
      if (!(tm & (1u << k))) continue;
      typename V2<R>::type a, b;
      a.x = v[k].re;
      a.y = v[k].im;
      b.x = w[k].re;
      b.y = w[k].im;
      psi[idx[k]] = a;
      lam[idx[k]] = b;
    }
    if (++cnt == kGradChunk) {
      cnt = 0;
      for (unsigned k = 0; k < nslots; ++k) {
        dacc[k] += (double)racc[k];
        racc[k] = 0;
      }
    }
  }
  __shared__ double red[kThreads / 32][kGradSlots];
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (unsigned k = 0; k < nslots; ++k) {
    double x = dacc[k] + (double)racc[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < nslots) {
    double t = 0.0;
    for (unsigned w = 0; w < kThreads / 32; ++w) t += red[w][threadIdx.x];
    partials[(uint64_t)blockIdx.x * kGradSlots + threadIdx.x] = t;
  }
}

__global__ void k_grad_finish(const double* __restrict__ partials, unsigned nblocks, const GradMap map,
                              double* __restrict__ grad) {
  __shared__ double tot[kGradSlots];
  if (threadIdx.x < map.nslots) {
    double t = 0.0;
    for (unsigned b = 0; b < nblocks; ++b) t += partials[(uint64_t)b * kGradSlots + threadIdx.x];
    tot[threadIdx.x] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (unsigned k = 0; k < map.nslots; ++k) grad[map.param[k]] += tot[k];  // two slots may share a parameter
}

// ---- bulk-copy pipelined sweep (large registers) ------------------------------------------
//
// A persistent grid streams tiles through shared memory: thread 0 keeps kTmaStages - 1 tiles
// in flight with cp.async.bulk copies that complete on per-stage mbarriers, while all 256
// threads apply the sweep to the tile that has landed (one group of 2^K amplitudes each) and
// store the results straight to global memory. A tile is 2^kh contiguous chunks of T = 2^t
// amplitudes: the active positions below t lie inside a chunk, those at or above t select the
// chunk. t = 8 + kl (kl = number of active positions below t), so a tile holds exactly 256
// groups. Memory latency is hidden by the copies in flight instead of by warps.

constexpr int kTmaThreads = 256;
constexpr int kTmaStages = 3;

struct TileGeom {
  unsigned t, kh, kl;
  unsigned hi_sorted[kSweepMaxK];  // active positions >= t, ascending
  unsigned lo_sorted[kSweepMaxK];  // active positions < t, ascending
  uint64_t chunk_off[1 << kSweepMaxK];
  uint32_t slot_chunk[1 << kSweepMaxK];
  uint32_t slot_lowoff[1 << kSweepMaxK];
  uint64_t slot_off[1 << kSweepMaxK];
};

template <typename R, bool DF, int K>
__global__ void __launch_bounds__(kTmaThreads) k_sweep_bulk(typename V2<R>::type* __restrict__ s, uint64_t ntiles,
                                                            const __grid_constant__ TileGeom geo,
                                                            const __grid_constant__ SweepParams P,
                                                            unsigned long long* __restrict__ err) {
  using V = typename V2<R>::type;
  constexpr int G = 1 << K;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full[kTmaStages];
  V* sm = reinterpret_cast<V*>(smem_raw);
  const uint32_t T = 1u << geo.t;
  const uint32_t nchunks = 1u << geo.kh;
  const uint32_t chunk_bytes = T * (uint32_t)sizeof(V);

  if (threadIdx.x == 0) {
    for (int i = 0; i < kTmaStages; ++i) mbar_init(&full[i], 1);
    fence_mbar_init();
  }
  __syncthreads();

  const uint64_t first = blockIdx.x, stride = gridDim.x;
  const uint64_t mine = first < ntiles ? (ntiles - 1 - first) / stride + 1 : 0;

  auto tile_base = [&](uint64_t tile) {
    uint64_t b = tile << geo.t;
    for (unsigned k = 0; k < geo.kh; ++k) b = insert_zero(b, geo.hi_sorted[k]);
    return b;
  };
  auto issue = [&](uint64_t j) {  // j-th tile of this CTA into stage j % kTmaStages
    const int st = (int)(j % kTmaStages);
    const uint64_t tb = tile_base(first + j * stride);
    mbar_arrive_expect_tx(&full[st], chunk_bytes * nchunks);
    for (uint32_t c = 0; c < nchunks; ++c)
      bulk_g2s(sm + (size_t)(st * nchunks + c) * T, s + (tb | geo.chunk_off[c]), chunk_bytes, &full[st]);
  };

  uint64_t issued = 0;
  if (threadIdx.x == 0)
    for (; issued < (uint64_t)(kTmaStages - 1) && issued < mine; ++issued) issue(issued);

  uint64_t lb = threadIdx.x;
  for (unsigned k = 0; k < geo.kl; ++k) lb = insert_zero(lb, geo.lo_sorted[k]);

  uint64_t i = 0;
  bool failed = false;
  for (; i < mine; ++i) {
    const int st = (int)(i % kTmaStages);
    if (threadIdx.x == 0 && issued < mine) {
      // The stage refilled here held tile i - 1, whose reads ended at the barrier below.
      fence_proxy_async_smem();
      issue(issued++);
    }
    const bool ok_wait = mbar_wait(&full[st], (uint32_t)((i / kTmaStages) & 1));
    if (ok_wait) {
      const uint64_t tb = tile_base(first + i * stride) | lb;
      const V* stage = sm + (size_t)st * nchunks * T;
      uint64_t idx[G];
      V raw[G];
#pragma unroll
      for (int k = 0; k < G; ++k) {
        idx[k] = tb | geo.slot_off[k];
        raw[k] = stage[(size_t)geo.slot_chunk[k] * T + (lb | geo.slot_lowoff[k])];
      }
      unsigned tm = 0;
      if constexpr (DF) {
        DF64Arith::VT v[G];
        bool ok = true;
#pragma unroll
        for (int k = 0; k < G; ++k) {
          ok &= df64::split(raw[k].x, v[k].re);
          ok &= df64::split(raw[k].y, v[k].im);
        }
        V out[G];
        if (ok) {
          run_ops<DF64Arith, K>(P, v, idx, tm);
#pragma unroll
          for (int k = 0; k < G; ++k)
            if (tm & (1u << k)) {
              ok &= df64::merge(v[k].re.h, v[k].re.l, out[k].x);
              ok &= df64::merge(v[k].im.h, v[k].im.l, out[k].y);
            }
        }
        if (!ok) {
          NativeArith<double>::VT w[G];
#pragma unroll
          for (int k = 0; k < G; ++k) {
            w[k].re = raw[k].x;
            w[k].im = raw[k].y;
          }
          tm = 0;
          run_ops<NativeArith<double>, K>(P, w, idx, tm);
#pragma unroll
          for (int k = 0; k < G; ++k) {
            out[k].x = w[k].re;
            out[k].y = w[k].im;
          }
        }
#pragma unroll
        for (int k = 0; k < G; ++k)
          if (tm & (1u << k)) s[idx[k]] = out[k];
      } else {
        typename NativeArith<R>::VT v[G];
#pragma unroll
        for (int k = 0; k < G; ++k) {
          v[k].re = raw[k].x;
          v[k].im = raw[k].y;
        }
        run_ops<NativeArith<R>, K>(P, v, idx, tm);
#pragma unroll
        for (int k = 0; k < G; ++k)
          if (tm & (1u << k)) {
            V a;
            a.x = v[k].re;
            a.y = v[k].im;
            s[idx[k]] = a;
          }
      }
    }
    // Block-uniform decision: every thread reaches this barrier each iteration.
    if (__syncthreads_or(!ok_wait)) {
      failed = true;
      break;
    }
  }
  if (failed && threadIdx.x == 0) {
    atomicExch(err, 1ull);
    // Let the copies this CTA still has in flight land (bounded) before it exits.
    for (uint64_t j = i; j < issued; ++j) (void)mbar_wait(&full[j % kTmaStages], (uint32_t)((j / kTmaStages) & 1));
  }
}

bool make_geometry(const SweepParams& P, unsigned n, TileGeom& g) {
  const unsigned K = P.K;
  unsigned kl = 0;
  for (; kl <= K; ++kl) {
    unsigned below = 0;
    for (unsigned j = 0; j < K; ++j) below += P.pos[j] < 8 + kl ? 1u : 0u;
    if (below == kl) break;
  }
  if (kl > K) return false;
  std::memset(&g, 0, sizeof g);
  g.t = 8 + kl;
  g.kl = kl;
  g.kh = K - kl;
  if (n < g.t + g.kh) return false;
  unsigned nh = 0, nl = 0;
  for (unsigned j = 0; j < K; ++j) {
    if (P.sorted[j] >= g.t) g.hi_sorted[nh++] = P.sorted[j];
    else g.lo_sorted[nl++] = P.sorted[j];
  }
  for (unsigned c = 0; c < (1u << g.kh); ++c)
    for (unsigned b = 0; b < g.kh; ++b)
      if (c & (1u << b)) g.chunk_off[c] |= uint64_t(1) << g.hi_sorted[b];
  for (unsigned sl = 0; sl < (1u << K); ++sl) {
    uint32_t chunk = 0, low = 0;
    for (unsigned j = 0; j < K; ++j) {
      if (!(sl & (1u << j))) continue;
      const unsigned p = P.pos[j];
      if (p >= g.t) {
        unsigned rank = 0;
        while (g.hi_sorted[rank] != p) ++rank;
        chunk |= 1u << rank;
      } else {
        low |= 1u << p;
      }
    }
    g.slot_chunk[sl] = chunk;
    g.slot_lowoff[sl] = low;
    g.slot_off[sl] = g.chunk_off[chunk] | low;
  }
  return true;
}

template <typename R, bool DF, int K>
void launch_bulk(iqsg_state* h, const SweepParams& P, const TileGeom& g) {
  using V = typename V2<R>::type;
  const size_t smem = (size_t)kTmaStages * (size_t(256) << K) * sizeof(V);
  static int per_device[kMaxDevices] = {};  // per instantiation and device; 0 = not configured yet
  const int dev = current_device();
  if (!per_device[dev]) {
    cudaFuncSetAttribute(k_sweep_bulk<R, DF, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_sweep_bulk<R, DF, K>, kTmaThreads, smem) != cudaSuccess ||
        b < 1)
      b = 1;
    per_device[dev] = b;
  }
  const int blocks_per_sm = per_device[dev];
  const uint64_t ntiles = h->N >> (K + 8);
  uint64_t grid = (uint64_t)num_sms() * (uint64_t)blocks_per_sm;
  if (grid > ntiles) grid = ntiles;
  k_sweep_bulk<R, DF, K><<<(unsigned)grid, kTmaThreads, smem, h->stream>>>(
      reinterpret_cast<V*>(h->amps), ntiles, g, P, reinterpret_cast<unsigned long long*>(h->scratch + kErrorSlot));
}

template <int K>
void launch_k(iqsg_state* h, const SweepParams& P) {
  const uint64_t ngroups = h->N >> K;
  const bool df = h->prec == IQSG_COMPLEX_DP && h->math == IQSG_MATH_EMULATED && K <= 3;
  TileGeom g;
  if (h->bulk && h->n >= kBulkMinQubits && make_geometry(P, h->n, g)) {
    if (h->prec == IQSG_COMPLEX_SP) launch_bulk<float, false, K>(h, P, g);
    else if (df) launch_bulk<double, (K <= 3), K>(h, P, g);
    else launch_bulk<double, false, K>(h, P, g);
    return;
  }
  const unsigned grid = grid_for(ngroups, 1);
  if (h->prec == IQSG_COMPLEX_SP) {
    k_sweep_native<float, K><<<grid, kThreads, 0, h->stream>>>(reinterpret_cast<float2*>(h->amps), ngroups, P);
  } else if (df) {
    if constexpr (K <= 3) {
      k_sweep_df<K><<<grid, kThreads, 0, h->stream>>>(reinterpret_cast<double2*>(h->amps), ngroups, P, nullptr);
    }
  } else {
    k_sweep_native<double, K><<<grid, kThreads, 0, h->stream>>>(reinterpret_cast<double2*>(h->amps), ngroups, P);
  }
}

}  // namespace

namespace {

// One sweep of a double-float storage run: the pair kernel, and the IEEE kernel that runs in
// its place when the range check failed.
template <int K>
void launch_dfs_k(iqsg_state* h, const SweepParams& P, bool first, bool last) {
  if constexpr (K <= 3) {
    const uint64_t ngroups = h->N >> K;
    const unsigned grid = grid_for(ngroups, 1);
    double2* s = reinterpret_cast<double2*>(h->amps);
    const auto* bad = reinterpret_cast<const unsigned long long*>(h->scratch + kRangeSlot);
    if (first && last) k_sweep_dfs<K, false, false><<<grid, kThreads, 0, h->stream>>>(s, ngroups, P, bad);
    else if (first) k_sweep_dfs<K, false, true><<<grid, kThreads, 0, h->stream>>>(s, ngroups, P, bad);
    else if (last) k_sweep_dfs<K, true, false><<<grid, kThreads, 0, h->stream>>>(s, ngroups, P, bad);
    else k_sweep_dfs<K, true, true><<<grid, kThreads, 0, h->stream>>>(s, ngroups, P, bad);
    k_sweep_df<K><<<grid, kThreads, 0, h->stream>>>(s, ngroups, P, bad);
  }
}

}  // namespace

void launch_df_storage_run(iqsg_state* h, const std::vector<SweepParams>& progs) {
  auto* bad = reinterpret_cast<unsigned long long*>(h->scratch + kRangeSlot);
  cudaMemsetAsync(bad, 0, sizeof(unsigned long long), h->stream);
  k_df_range<<<grid_for(h->N, 1), kThreads, 0, h->stream>>>(reinterpret_cast<const double2*>(h->amps), h->N, bad);
  for (size_t i = 0; i < progs.size(); ++i) {
    const bool first = i == 0, last = i + 1 == progs.size();
    switch (progs[i].K) {
      case 0: launch_dfs_k<0>(h, progs[i], first, last); break;
      case 1: launch_dfs_k<1>(h, progs[i], first, last); break;
      case 2: launch_dfs_k<2>(h, progs[i], first, last); break;
      case 3: launch_dfs_k<3>(h, progs[i], first, last); break;
    }
  }
}

void launch_sweep(iqsg_state* h, const SweepParams& P) {
  switch (P.K) {
    case 0: launch_k<0>(h, P); break;
    case 1: launch_k<1>(h, P); break;
    case 2: launch_k<2>(h, P); break;
    case 3: launch_k<3>(h, P); break;
    case 4: launch_k<4>(h, P); break;
  }
}

namespace {

template <int K>
void launch_adj_k(iqsg_state* psi, iqsg_state* lam, const SweepParams& P, const GradMap& map, double* grad) {
  const uint64_t ngroups = psi->N >> K;
  uint64_t blocks = (ngroups + kThreads - 1) / kThreads;
  const uint64_t cap = (uint64_t)num_sms() * kAdjBlocksPerSm;
  if (blocks > cap) blocks = cap;
  if (blocks * kGradSlots > 2 * (uint64_t)kMaxPartials) blocks = 2 * kMaxPartials / kGradSlots;
  double* partials = psi->scratch;
  if (psi->prec == IQSG_COMPLEX_SP)
    k_sweep_adj<float, K><<<(unsigned)blocks, kThreads, 0, psi->stream>>>(
        reinterpret_cast<float2*>(psi->amps), reinterpret_cast<float2*>(lam->amps), ngroups, P, map.nslots, partials);
  else
    k_sweep_adj<double, K><<<(unsigned)blocks, kThreads, 0, psi->stream>>>(
        reinterpret_cast<double2*>(psi->amps), reinterpret_cast<double2*>(lam->amps), ngroups, P, map.nslots,
        partials);
  if (map.nslots) k_grad_finish<<<1, 32, 0, psi->stream>>>(partials, (unsigned)blocks, map, grad);
}

}  // namespace

void launch_sweep_adj(iqsg_state* psi, iqsg_state* lam, const SweepParams& P, const GradMap& map, double* grad) {
  switch (P.K) {
    case 0: launch_adj_k<0>(psi, lam, P, map, grad); break;
    case 1: launch_adj_k<1>(psi, lam, P, map, grad); break;
    case 2: launch_adj_k<2>(psi, lam, P, map, grad); break;
    case 3: launch_adj_k<3>(psi, lam, P, map, grad); break;
    case 4: launch_adj_k<4>(psi, lam, P, map, grad); break;
  }
}

namespace {

unsigned default_width(const iqsg_state* h) {
  if (h->prec == IQSG_COMPLEX_SP) return 4;
  return h->math == IQSG_MATH_EMULATED ? 2 : 3;
}

}  // namespace

unsigned sweep_width(const iqsg_state* h) {
  unsigned k = h->sweep_width ? h->sweep_width : default_width(h);
  if (h->prec == IQSG_COMPLEX_DP && h->math == IQSG_MATH_EMULATED && k > 3) k = 3;
  return std::min(k, std::min(h->n, (unsigned)kSweepMaxK));
}

}  // namespace iqsg

using namespace iqsg;

namespace {

}  // namespace

extern "C" int iqsg_set_sweep_width(iqsg_state* h, unsigned kmax) {
  if (!h) return fail(IQSG_EINVAL, "null register handle");
  if (kmax > (unsigned)kSweepMaxK) return fail(IQSG_EINVAL, "iqsg_set_sweep_width: width %u above %d", kmax, kSweepMaxK);
  h->sweep_width = kmax;
  return IQSG_OK;
}

extern "C" int iqsg_set_option(iqsg_state* h, int option, int value) {
  if (!h) return fail(IQSG_EINVAL, "null register handle");
  switch (option) {
    case IQSG_OPT_SWEEP_WIDTH:
      return iqsg_set_sweep_width(h, (unsigned)value);
    case IQSG_OPT_SWEEP_PIPELINE:
      h->bulk = value != 0;
      return IQSG_OK;
    case IQSG_OPT_NATIVE_SHARE:
      if (value < 0 || value > 16) return fail(IQSG_EINVAL, "iqsg_set_option: native share %d outside 0..16", value);
      h->native16 = (unsigned)value;
      return IQSG_OK;
    case IQSG_OPT_DF_STORAGE:
      h->df_storage = value != 0;
      return IQSG_OK;
    case IQSG_OPT_TILE_QUBITS:
      if (value < 0 || value > 14) return fail(IQSG_EINVAL, "iqsg_set_option: tile size %d outside 0..14", value);
      h->tile_qubits = (unsigned)value;
      return IQSG_OK;
    default:
      return fail(IQSG_EINVAL, "iqsg_set_option: unknown option %d", option);
  }
}

namespace {

// Sweeps a double-float storage run needs at least: the range check costs about a fifth of a
// sweep, and each sweep between the first and the last saves about a third of one.
constexpr size_t kDfStoreMinSweeps = 3;

// Upper bound of the spectral norm of an op on the whole space (identity outside its block):
// the square root of the largest Gershgorin row sum of M^H M.
double op_norm_bound(const iqsg_op& op) {
  auto gersh = [](const double* m, int d) {
    double best = 0;
    for (int i = 0; i < d; ++i) {
      double rs = 0;
      for (int j = 0; j < d; ++j) {
        double re = 0, im = 0;  // (M^H M)_ij = sum_k conj(M_ki) M_kj
        for (int k = 0; k < d; ++k) {
          const double ar = m[2 * (k * d + i)], ai = m[2 * (k * d + i) + 1];
          const double br = m[2 * (k * d + j)], bi = m[2 * (k * d + j) + 1];
          re += ar * br + ai * bi;
          im += ar * bi - ai * br;
        }
        rs += std::sqrt(re * re + im * im);
      }
      best = std::max(best, rs);
    }
    return std::sqrt(best);
  };
  auto absc = [](const double* z) { return std::sqrt(z[0] * z[0] + z[1] * z[1]); };
  switch (op.kind) {
    case IQSG_OP_1Q: return gersh(op.m, 2);
    case IQSG_OP_CTRL:
    case IQSG_OP_SWAPLIKE: return std::max(1.0, gersh(op.m, 2));
    case IQSG_OP_2Q: return gersh(op.m, 4);
    case IQSG_OP_DIAG2: return std::max(std::max(absc(op.m), absc(op.m + 2)), std::max(absc(op.m + 4), absc(op.m + 6)));
    case IQSG_OP_PHASE: return std::max(1.0, absc(op.m));
    default: return HUGE_VAL;
  }
}

class CollectSweeps : public SweepSink {
 public:
  void take(const SweepParams& P, const GradMap&) override { progs.push_back(P); }
  std::vector<SweepParams> progs;
};

}  // namespace

extern "C" int iqsg_apply_ops(iqsg_state* h, const iqsg_op* ops, unsigned count, unsigned* sweeps) {
  if (!h) return fail(IQSG_EINVAL, "null register handle");
  if (count && !ops) return fail(IQSG_EINVAL, "iqsg_apply_ops: null op array");
  for (unsigned i = 0; i < count; ++i) {
    const int st = check_op(h, ops[i], i);
    if (st) return st;
  }
  const bool df = h->prec == IQSG_COMPLEX_DP && h->math == IQSG_MATH_EMULATED;
  const unsigned kt = df ? 0u : tile_qubits(h, false);
  if (kt) return tile_schedule(h, nullptr, ops, count, kt, std::max(1u, sweep_width(h)), nullptr, sweeps);
  if (df && h->df_storage && !h->bulk && h->native16 == 0 && h->n >= 2) {
    // Emulated FP64: collect the sweeps, then run them with the state as double-float pairs
    // when the run is long enough and every gate is contractive.
    CollectSweeps c;
    {
      SweepBuilder b(&c, std::max(1u, sweep_width(h)));
      for (unsigned i = 0; i < count; ++i) queue_op(b, ops[i]);
      b.flush();
    }
    bool pairs = c.progs.size() >= kDfStoreMinSweeps;
    for (unsigned i = 0; pairs && i < count; ++i) pairs = op_norm_bound(ops[i]) <= 1.0 + 1e-9;
    for (const auto& P : c.progs) pairs = pairs && P.K <= 3;
    if (pairs) {
      launch_df_storage_run(h, c.progs);
      h->df_runs += 1;
      h->df_launches += 1 + 2 * c.progs.size();
    } else {
      for (auto& P : c.progs) launch_sweep(h, P);
    }
    if (sweeps) *sweeps = (unsigned)c.progs.size();
    return cuda_status(cudaGetLastError(), "iqsg_apply_ops");
  }
  SweepBuilder b(h, std::max(1u, sweep_width(h)));
  for (unsigned i = 0; i < count; ++i) queue_op(b, ops[i]);
  b.flush();
  if (sweeps) *sweeps = b.launched();
  return cuda_status(cudaGetLastError(), "iqsg_apply_ops");
}

// The sweeps iqsg_apply_ops would run for a gate stream on a register of num_qubits positions
// with default options (no tile passes, no bulk pipeline, no native share), computed on the
// host only: nothing is allocated or launched, no GPU is needed.
extern "C" int iqsg_plan_ops(unsigned num_qubits, int precision, int math, unsigned width, const iqsg_op* ops,
                             unsigned count, iqsg_sweep_info* out, unsigned cap, unsigned* nsweeps,
                             int* pair_storage) {
  if (count && !ops) return fail(IQSG_EINVAL, "iqsg_plan_ops: null op array");
  if (num_qubits == 0 || num_qubits > 40) return fail(IQSG_EINVAL, "iqsg_plan_ops: %u qubits (1..40)", num_qubits);
  if (precision != IQSG_COMPLEX_DP && precision != IQSG_COMPLEX_SP)
    return fail(IQSG_EINVAL, "iqsg_plan_ops: unknown precision %d", precision);
  if (math != IQSG_MATH_NATIVE && math != IQSG_MATH_EMULATED)
    return fail(IQSG_EINVAL, "iqsg_plan_ops: unknown math %d", math);
  if (width > (unsigned)kSweepMaxK) return fail(IQSG_EINVAL, "iqsg_plan_ops: width %u above %d", width, kSweepMaxK);
  iqsg_state shape;  // sizes and options only: no memory behind it
  shape.n = num_qubits;
  shape.N = uint64_t(1) << num_qubits;
  shape.prec = precision;
  shape.math = math;
  shape.sweep_width = width;
  for (unsigned i = 0; i < count; ++i) {
    const int st = check_op(&shape, ops[i], i);
    if (st) return st;
  }
  CollectSweeps c;
  {
    SweepBuilder b(&c, std::max(1u, sweep_width(&shape)));
    for (unsigned i = 0; i < count; ++i) queue_op(b, ops[i]);
    b.flush();
  }
  if (nsweeps) *nsweeps = (unsigned)c.progs.size();
  if (pair_storage) {  // the rule iqsg_apply_ops applies
    bool pairs = precision == IQSG_COMPLEX_DP && math == IQSG_MATH_EMULATED && num_qubits >= 2 &&
                 c.progs.size() >= kDfStoreMinSweeps;
    for (unsigned i = 0; pairs && i < count; ++i) pairs = op_norm_bound(ops[i]) <= 1.0 + 1e-9;
    for (const auto& P : c.progs) pairs = pairs && P.K <= 3;
    *pair_storage = pairs ? 1 : 0;
  }
  if (out && cap < c.progs.size())
    return fail(IQSG_EINVAL, "iqsg_plan_ops: %zu sweeps do not fit %u entries", c.progs.size(), cap);
  for (size_t s = 0; out && s < c.progs.size(); ++s) {
    const SweepParams& P = c.progs[s];
    iqsg_sweep_info& o = out[s];
    std::memset(&o, 0, sizeof o);
    o.k = P.K;
    for (unsigned j = 0; j < P.K; ++j) o.pos[j] = P.pos[j];
    o.ops = P.nops;
    for (unsigned k = 0; k < P.nops; ++k) {
      switch (P.ops[k].kind) {
        case SW_U2: ++o.one_qubit; break;
        case SW_U4:
        case SW_SWAPLIKE:
        case SW_EXC: ++o.two_qubit; break;
        default: ++o.diagonal; break;  // SW_PHASE, SW_CZSHIFT
      }
    }
  }
  return IQSG_OK;
}

extern "C" int iqsg_counters(const iqsg_state* h, uint64_t* counters) {
  if (!h || !counters) return fail(IQSG_EINVAL, "iqsg_counters: null argument");
  counters[0] = h->df_runs;
  counters[1] = h->df_launches;
  return IQSG_OK;
}

extern "C" int iqsg_adjoint_ops(iqsg_state* psi, iqsg_state* lam, const iqsg_op* ops, unsigned count, double* grads,
                                unsigned nparams, unsigned* sweeps) {
  if (!psi || !lam) return fail(IQSG_EINVAL, "null register handle");
  if (psi == lam) return fail(IQSG_EINVAL, "iqsg_adjoint_ops: psi and lam must be different registers");
  if (psi->n != lam->n || psi->prec != lam->prec || psi->device != lam->device)
    return fail(IQSG_EINVAL, "iqsg_adjoint_ops: registers differ in size, precision or device");
  if (count && !ops) return fail(IQSG_EINVAL, "iqsg_adjoint_ops: null op array");
  if (nparams > (unsigned)kTableDoubles) return fail(IQSG_EINVAL, "iqsg_adjoint_ops: more than %d parameters", kTableDoubles);
  if (nparams && !grads) return fail(IQSG_EINVAL, "iqsg_adjoint_ops: null gradient array");
  for (unsigned i = 0; i < count; ++i) {
    const int st = check_op(psi, ops[i], i, true, nparams);
    if (st) return st;
  }
  int st = IQSG_OK;
  if (lam->stream != psi->stream && (st = sync_and_check(lam, "iqsg_adjoint_ops"))) return st;
  double* dgrad = psi->scratch + kTableSlot;
  if (nparams && (st = cuda_status(cudaMemsetAsync(dgrad, 0, sizeof(double) * nparams, psi->stream),
                                   "iqsg_adjoint_ops: clear")))
    return st;
  const unsigned kmax = std::max(1u, std::min(sweep_width(psi), psi->prec == IQSG_COMPLEX_SP ? 4u : 3u));
  const unsigned kt = tile_qubits(psi, true);
  if (kt) {
    if ((st = tile_schedule(psi, lam, ops, count, kt, kmax, dgrad, sweeps))) return st;
  } else {
    SweepBuilder b(psi, lam, dgrad, kmax);
    for (unsigned i = 0; i < count; ++i) {
      // A gradient op followed by its excitation-preserving gate on the same pair becomes one
      // operation (one pass over each quad of psi and lambda).
      const iqsg_op& g = ops[i];
      if (i + 1 < count && g.kind == IQSG_OP_GRAD2 && ops[i + 1].kind == IQSG_OP_2Q && ops[i + 1].t0 == g.t0 &&
          ops[i + 1].t1 == g.t1 && SweepBuilder::is_excitation(g.m) && SweepBuilder::is_excitation(ops[i + 1].m)) {
        b.add_grad_and_excitation(g.t0, g.t1, g.m, ops[i + 1].m, (unsigned)g.value);
        ++i;
        continue;
      }
      queue_op(b, g);
    }
    b.flush();
    if (sweeps) *sweeps = b.launched();
  }
  if ((st = cuda_status(cudaGetLastError(), "iqsg_adjoint_ops"))) return st;
  std::vector<double> g(nparams);
  if (nparams && (st = cuda_status(cudaMemcpyAsync(g.data(), dgrad, sizeof(double) * nparams, cudaMemcpyDeviceToHost,
                                                   psi->stream), "iqsg_adjoint_ops: gradients")))
    return st;
  if ((st = sync_and_check(psi, "iqsg_adjoint_ops"))) return st;
  for (unsigned k = 0; k < nparams; ++k) grads[k] += g[k];
  return IQSG_OK;
}
