// Tile passes: one pass over the state applies a long stretch of the gate stream by staging
// tiles of 2^kt amplitudes in shared memory.
//
// A tile spans the tl lowest positions (tl = log2(128 B / amplitude size), so every run of
// the tile in HBM is a whole 128-byte line) plus up to kt - tl higher positions hi[]; the
// other n - kt index bits select the tile. A CTA loads a tile (coalesced), runs the pass's
// phases on it -- each phase is an ordinary fused sweep program (sweep.cuh) over at most 4
// of the tile's positions, applied group by group out of shared memory -- and stores it
// back. Any gate whose non-diagonal positions all lie in the tile can run in the pass;
// diagonal gates and controls may use any position.
//
// The scheduler (tile_schedule) picks each pass's positions greedily while it walks the
// gate stream, and moves a gate ahead of gates it was not placed with only when their
// supports are disjoint (or both are diagonal), so the product of the passes equals the
// product of the gates in stream order.
//
// The adjoint variant stages a tile of psi and the same tile of lambda and runs two-vector
// phases with gradient operations (sweep.cuh, run_ops_dual).
#include <algorithm>
#include <cstring>
#include <iterator>
#include <memory>
#include <vector>

#include "scheduler.h"
#include "sweep.cuh"

namespace iqsg {

namespace {

constexpr int kTileThreads = 256;
constexpr int kTileMaxHigh = 12;
constexpr int kTileMaxPhases = 40;
constexpr int kTileMaxOps = 192;
constexpr int kTileMaxEntries = 560;

struct TilePhase {
  uint8_t K;
  uint8_t lpos[4];     // slot j <-> local bit lpos[j]
  uint8_t lsorted[4];  // local bits ascending
  uint8_t needs_idx;   // some operation reads the data index (controls, phases, CZ runs)
  uint8_t pad[2];
  uint16_t op0, nops;
};

struct TileParams {
  uint32_t kt, tl, nhi, nphases;
  uint32_t hi[kTileMaxHigh];  // data positions of local bits tl .. kt-1, ascending
  TilePhase ph[kTileMaxPhases];
  SweepOp ops[kTileMaxOps];
  SweepEntry ent[kTileMaxEntries];
};
static_assert(sizeof(TileParams) < 32000, "kernel parameter space");

// Bank swizzle: XOR the next log2(S) bits into the low ones (S amplitudes per 128 B).
template <typename V>
__device__ __forceinline__ uint32_t swz(uint32_t l) {
  constexpr uint32_t S = 128 / sizeof(V);
  constexpr uint32_t B = S == 16 ? 4 : 3;
  return l ^ ((l >> B) & (S - 1));
}

template <typename R, int K, bool DUAL>
__device__ __forceinline__ void tile_phase(const TileParams& P, const TilePhase& ph, typename V2<R>::type* sm,
                                           typename V2<R>::type* sl, const uint64_t* hiexp, uint64_t base,
                                           uint32_t T, R* acc) {
  using A = NativeArith<R>;
  using V = typename V2<R>::type;
  constexpr int G = 1 << K;
  const uint32_t groups = T >> K;
  const uint32_t lowmask = (1u << P.tl) - 1;
  const bool need_idx = ph.needs_idx != 0;
  uint32_t off[G];  // local offset of each slot, the same for every group of the phase
#pragma unroll
  for (int s = 0; s < G; ++s) {
    uint32_t o = 0;
#pragma unroll
    for (int j = 0; j < K; ++j)
      if (s & (1 << j)) o |= 1u << ph.lpos[j];
    off[s] = o;
  }
  for (uint32_t g = threadIdx.x; g < groups; g += blockDim.x) {
    uint32_t lb = g;
#pragma unroll
    for (int k = 0; k < K; ++k) lb = (uint32_t)insert_zero(lb, ph.lsorted[k]);
    uint32_t loc[G];
    uint64_t idx[G];
    typename A::VT v[G], w[DUAL ? G : 1];
#pragma unroll
    for (int s = 0; s < G; ++s) {
      const uint32_t o = lb | off[s];
      loc[s] = o;
      idx[s] = need_idx ? (base | (o & lowmask) | hiexp[o >> P.tl]) : 0;
      const V a = sm[swz<V>(o)];
      v[s].re = a.x;
      v[s].im = a.y;
      if constexpr (DUAL) {
        const V b = sl[swz<V>(o)];
        w[s].re = b.x;
        w[s].im = b.y;
      }
    }
    unsigned tm = 0;
    if constexpr (DUAL) {
#pragma unroll 1
      for (unsigned o = ph.op0; o < (unsigned)ph.op0 + ph.nops; ++o) {
        const SweepOp op = P.ops[o];
        if (op.kind == SW_EXCADJ) {
          acc[op.value] += excadj_op<R, K>(P.ent, op, v, w, idx, tm);
        } else if (op.kind == SW_GRAD1 || op.kind == SW_GRAD2 || op.kind == SW_GRADEXC) {
          acc[op.value] += grad_op<R, K>(P.ent, op, v, w, idx);
        } else {
          apply_op<A, K>(P.ent, op, v, idx, tm);
          apply_op<A, K>(P.ent, op, w, idx, tm);
        }
      }
    } else {
#pragma unroll 1
      for (unsigned o = ph.op0; o < (unsigned)ph.op0 + ph.nops; ++o) apply_op<A, K>(P.ent, P.ops[o], v, idx, tm);
    }
#pragma unroll
    for (int s = 0; s < G; ++s) {
      if (!(tm & (1u << s))) continue;
      V a;
      a.x = v[s].re;
      a.y = v[s].im;
      sm[swz<V>(loc[s])] = a;
      if constexpr (DUAL) {
        V b;
        b.x = w[s].re;
        b.y = w[s].im;
        sl[swz<V>(loc[s])] = b;
      }
    }
  }
}

template <typename R, bool DUAL>
__device__ __forceinline__ void run_phases(const TileParams& P, typename V2<R>::type* sm, typename V2<R>::type* sl,
                                           const uint64_t* hiexp, uint64_t base, uint32_t T, R* acc) {
  for (uint32_t p = 0; p < P.nphases; ++p) {
    const TilePhase& ph = P.ph[p];
    switch (ph.K) {
      case 0: tile_phase<R, 0, DUAL>(P, ph, sm, sl, hiexp, base, T, acc); break;
      case 1: tile_phase<R, 1, DUAL>(P, ph, sm, sl, hiexp, base, T, acc); break;
      case 2: tile_phase<R, 2, DUAL>(P, ph, sm, sl, hiexp, base, T, acc); break;
      case 3: tile_phase<R, 3, DUAL>(P, ph, sm, sl, hiexp, base, T, acc); break;
      case 4: tile_phase<R, 4, DUAL>(P, ph, sm, sl, hiexp, base, T, acc); break;
    }
    __syncthreads();
  }
}

__device__ __forceinline__ void fill_hiexp(const TileParams& P, uint64_t* hiexp) {
  for (uint32_t i = threadIdx.x; i < (1u << P.nhi); i += blockDim.x) {
    uint64_t o = 0;
    for (uint32_t b = 0; b < P.nhi; ++b)
      if (i & (1u << b)) o |= uint64_t(1) << P.hi[b];
    hiexp[i] = o;
  }
}

__device__ __forceinline__ uint64_t tile_base(const TileParams& P, uint64_t t) {
  uint64_t base = t << P.tl;
  for (uint32_t b = 0; b < P.nhi; ++b) base = insert_zero(base, P.hi[b]);
  return base;
}

template <typename R>
__global__ void __launch_bounds__(kTileThreads) k_tile(typename V2<R>::type* __restrict__ s, uint64_t ntiles,
                                                       const __grid_constant__ TileParams P) {
  using V = typename V2<R>::type;
  extern __shared__ __align__(16) unsigned char tsm[];
  const uint32_t T = 1u << P.kt, lowmask = (1u << P.tl) - 1;
  V* sm = reinterpret_cast<V*>(tsm);
  uint64_t* hiexp = reinterpret_cast<uint64_t*>(tsm + (size_t)T * sizeof(V));
  fill_hiexp(P, hiexp);
  __syncthreads();
  for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const uint64_t base = tile_base(P, t);
#pragma unroll 8
    for (uint32_t l = threadIdx.x; l < T; l += kTileThreads) sm[swz<V>(l)] = s[base | (l & lowmask) | hiexp[l >> P.tl]];
    __syncthreads();
    run_phases<R, false>(P, sm, nullptr, hiexp, base, T, nullptr);
#pragma unroll 8
    for (uint32_t l = threadIdx.x; l < T; l += kTileThreads) s[base | (l & lowmask) | hiexp[l >> P.tl]] = sm[swz<V>(l)];
    __syncthreads();
  }
}

constexpr unsigned kTileGradChunkTiles = 4;

template <typename R>
__global__ void __launch_bounds__(kTileThreads) k_tile_adj(typename V2<R>::type* __restrict__ psi,
                                                           typename V2<R>::type* __restrict__ lam, uint64_t ntiles,
                                                           const __grid_constant__ TileParams P, unsigned nslots,
                                                           double* __restrict__ partials) {
  using V = typename V2<R>::type;
  extern __shared__ __align__(16) unsigned char tsm[];
  const uint32_t T = 1u << P.kt, lowmask = (1u << P.tl) - 1;
  V* sm = reinterpret_cast<V*>(tsm);
  V* sl = sm + T;
  uint64_t* hiexp = reinterpret_cast<uint64_t*>(tsm + 2 * (size_t)T * sizeof(V));
  fill_hiexp(P, hiexp);
  R racc[kGradSlots];
  double dacc[kGradSlots];
#pragma unroll
  for (int k = 0; k < kGradSlots; ++k) {
    racc[k] = 0;
    dacc[k] = 0.0;
  }
  __syncthreads();
  unsigned cnt = 0;
  for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const uint64_t base = tile_base(P, t);
#pragma unroll 4
    for (uint32_t l = threadIdx.x; l < T; l += kTileThreads) {
      const uint64_t i = base | (l & lowmask) | hiexp[l >> P.tl];
      sm[swz<V>(l)] = psi[i];
      sl[swz<V>(l)] = lam[i];
    }
    __syncthreads();
    run_phases<R, true>(P, sm, sl, hiexp, base, T, racc);
#pragma unroll 4
    for (uint32_t l = threadIdx.x; l < T; l += kTileThreads) {
      const uint64_t i = base | (l & lowmask) | hiexp[l >> P.tl];
      psi[i] = sm[swz<V>(l)];
      lam[i] = sl[swz<V>(l)];
    }
    __syncthreads();
    if (++cnt == kTileGradChunkTiles) {
      cnt = 0;
      for (unsigned k = 0; k < nslots; ++k) {
        dacc[k] += (double)racc[k];
        racc[k] = 0;
      }
    }
  }
  __shared__ double red[kTileThreads / 32][kGradSlots];
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (unsigned k = 0; k < nslots; ++k) {
    double x = dacc[k] + (double)racc[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < nslots) {
    double t = 0.0;
    for (unsigned w = 0; w < kTileThreads / 32; ++w) t += red[w][threadIdx.x];
    partials[(uint64_t)blockIdx.x * kGradSlots + threadIdx.x] = t;
  }
}

__global__ void k_tile_grad_finish(const double* __restrict__ partials, unsigned nblocks, const GradMap map,
                                   double* __restrict__ grad) {
  __shared__ double tot[kGradSlots];
  if (threadIdx.x < map.nslots) {
    double t = 0.0;
    for (unsigned b = 0; b < nblocks; ++b) t += partials[(uint64_t)b * kGradSlots + threadIdx.x];
    tot[threadIdx.x] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (unsigned k = 0; k < map.nslots; ++k) grad[map.param[k]] += tot[k];
}

// ---- host: assembling a pass from sweep programs ------------------------------------------

unsigned entries_of(const SweepOp& op) {
  switch (op.kind) {
    case SW_CZSHIFT: return 0;
    case SW_PHASE: return 1;
    case SW_U2: case SW_SWAPLIKE: case SW_GRAD1: return 4;
    case SW_EXC: case SW_GRADEXC: return 6;
    case SW_EXCADJ: return 12;
    default: return 16;  // SW_U4, SW_GRAD2
  }
}

class TileAssembler : public SweepSink {
 public:
  TileAssembler(uint64_t tmask, unsigned tl) {
    std::memset(&P_, 0, sizeof(P_));
    std::memset(&map_, 0, sizeof(map_));
    P_.tl = tl;
    unsigned kt = 0;
    for (unsigned p = 0; p < 64; ++p) {
      if (!(tmask & (uint64_t(1) << p))) continue;
      if (p >= tl) P_.hi[P_.nhi++] = p;
      ++kt;
    }
    P_.kt = kt;
  }
  unsigned local(unsigned p) const {
    if (p < P_.tl) return p;
    for (unsigned i = 0; i < P_.nhi; ++i)
      if (P_.hi[i] == p) return P_.tl + i;
    return ~0u;
  }
  void take(const SweepParams& S, const GradMap& m) override {
    TilePhase ph{};
    ph.K = (uint8_t)S.K;
    for (unsigned j = 0; j < S.K; ++j) ph.lpos[j] = (uint8_t)local(S.pos[j]);
    std::copy(ph.lpos, ph.lpos + S.K, ph.lsorted);
    std::sort(ph.lsorted, ph.lsorted + S.K);
    ph.op0 = (uint16_t)nops_;
    ph.nops = (uint16_t)S.nops;
    for (unsigned o = 0; o < S.nops; ++o)
      if (S.ops[o].mask || S.ops[o].kind == SW_PHASE || S.ops[o].kind == SW_CZSHIFT) ph.needs_idx = 1;
    unsigned used = 0;
    for (unsigned o = 0; o < S.nops; ++o) used = std::max(used, (unsigned)S.ops[o].ent + entries_of(S.ops[o]));
    if (overflow || P_.nphases + 1 > (unsigned)kTileMaxPhases || nops_ + S.nops > (unsigned)kTileMaxOps ||
        nent_ + used > (unsigned)kTileMaxEntries || map_.nslots + m.nslots > (unsigned)kGradSlots) {
      overflow = true;
      return;
    }
    for (unsigned o = 0; o < S.nops; ++o) {
      SweepOp op = S.ops[o];
      op.ent = (uint16_t)(op.ent + nent_);
      if (op.kind == SW_GRAD1 || op.kind == SW_GRAD2 || op.kind == SW_GRADEXC || op.kind == SW_EXCADJ)
        op.value += map_.nslots;
      P_.ops[nops_++] = op;
    }
    std::copy(S.ent, S.ent + used, P_.ent + nent_);
    nent_ += used;
    for (unsigned k = 0; k < m.nslots; ++k) map_.param[map_.nslots++] = m.param[k];
    P_.ph[P_.nphases++] = ph;
  }
  TileParams P_;
  GradMap map_;
  unsigned nops_ = 0, nent_ = 0;
  bool overflow = false;
};

// What a gate op needs from a pass: the positions it acts on non-diagonally (must be tile
// positions) and every position it reads (for reordering).
struct OpNeeds {
  uint64_t targets = 0, support = 0;
  bool diagonal = false;
  unsigned max_ops = 1, max_entries = 16, slots = 0;
};

bool offdiag_zero2(const double* m) { return m[2] == 0.0 && m[3] == 0.0 && m[4] == 0.0 && m[5] == 0.0; }

OpNeeds needs_of(const iqsg_op& op) {
  OpNeeds r;
  const uint64_t b0 = uint64_t(1) << op.t0, b1 = uint64_t(1) << op.t1;
  switch (op.kind) {
    case IQSG_OP_1Q:
    case IQSG_OP_CTRL: {
      uint64_t cm = 0;
      if (op.kind == IQSG_OP_CTRL)
        for (unsigned c = 0; c < op.nctrl; ++c) cm |= uint64_t(1) << op.ctrl[c];
      r.support = b0 | cm;
      r.diagonal = offdiag_zero2(op.m);
      r.targets = r.diagonal ? 0 : b0;
      r.max_ops = 2;
      r.max_entries = 4;
      break;
    }
    case IQSG_OP_2Q: {
      bool diag = true;
      for (int rr = 0; rr < 4; ++rr)
        for (int c = 0; c < 4; ++c)
          if (rr != c && (op.m[2 * (4 * rr + c)] != 0.0 || op.m[2 * (4 * rr + c) + 1] != 0.0)) diag = false;
      r.support = b0 | b1;
      r.diagonal = diag;
      r.targets = diag ? 0 : (b0 | b1);
      r.max_ops = 4;
      r.max_entries = 16;
      break;
    }
    case IQSG_OP_SWAPLIKE:
      r.support = r.targets = b0 | b1;
      r.max_entries = 4;
      break;
    case IQSG_OP_DIAG2:
      r.support = b0 | b1;
      r.diagonal = true;
      r.max_ops = 4;
      r.max_entries = 4;
      break;
    case IQSG_OP_PHASE:
      r.support = op.mask;
      r.diagonal = true;
      r.max_entries = 1;
      break;
    case IQSG_OP_GRAD1:
      r.support = r.targets = b0;
      r.max_entries = 4;
      r.slots = 1;
      break;
    case IQSG_OP_GRAD2:
      r.support = r.targets = b0 | b1;
      r.slots = 1;
      break;
  }
  return r;
}

template <typename V>
size_t tile_smem(unsigned kt, unsigned nhi, bool dual) {
  return (dual ? 2 : 1) * (size_t(1) << kt) * sizeof(V) + (size_t(1) << nhi) * sizeof(uint64_t);
}

template <typename R>
int launch_tile(iqsg_state* h, iqsg_state* lam, const TileAssembler& a, double* grad) {
  using V = typename V2<R>::type;
  const TileParams& P = a.P_;
  const bool dual = lam != nullptr;
  const size_t smem = tile_smem<V>(P.kt, P.nhi, dual);
  const void* fn = dual ? (const void*)k_tile_adj<R> : (const void*)k_tile<R>;
  static size_t configured[kMaxDevices][2] = {};  // largest dynamic smem set per device and kernel of this R
  const int dev = current_device();
  if (smem > 48 * 1024 && smem > configured[dev][dual]) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "tile pass: shared memory");
    configured[dev][dual] = smem;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kTileThreads, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const uint64_t ntiles = h->N >> P.kt;
  uint64_t grid = (uint64_t)num_sms() * (uint64_t)per_sm;
  if (dual && grid * kGradSlots > 2 * (uint64_t)kMaxPartials) grid = 2 * kMaxPartials / kGradSlots;
  if (grid > ntiles) grid = ntiles;
  if (!dual) {
    k_tile<R><<<(unsigned)grid, kTileThreads, smem, h->stream>>>(reinterpret_cast<V*>(h->amps), ntiles, P);
  } else {
    k_tile_adj<R><<<(unsigned)grid, kTileThreads, smem, h->stream>>>(
        reinterpret_cast<V*>(h->amps), reinterpret_cast<V*>(lam->amps), ntiles, P, a.map_.nslots, h->scratch);
    if (a.map_.nslots) k_tile_grad_finish<<<1, 32, 0, h->stream>>>(h->scratch, (unsigned)grid, a.map_, grad);
  }
  return cuda_status(cudaGetLastError(), "tile pass");
}

}  // namespace

unsigned tile_low_bits(const iqsg_state* h) { return h->prec == IQSG_COMPLEX_SP ? 4u : 3u; }

unsigned tile_qubits(const iqsg_state* h, bool dual) {
  if (!h->tile_qubits) return 0;
  const unsigned cap = h->prec == IQSG_COMPLEX_SP ? (dual ? 13u : 14u) : (dual ? 12u : 13u);
  unsigned kt = std::min(h->tile_qubits, cap);
  if (h->n < kt + 1 || kt <= tile_low_bits(h) || kt - tile_low_bits(h) > (unsigned)kTileMaxHigh) return 0;
  return kt;
}

// Run ops (validated) as tile passes: greedy light-cone packing into passes of at most kt
// positions, each pass split into register phases of at most kmax positions.
int tile_schedule(iqsg_state* h, iqsg_state* lam, const iqsg_op* ops, unsigned count, unsigned kt, unsigned kmax,
                  double* grad, unsigned* passes) {
  const unsigned tl = tile_low_bits(h);
  const uint64_t low = (uint64_t(1) << tl) - 1;
  std::vector<unsigned> pending(count);
  for (unsigned i = 0; i < count; ++i) pending[i] = i;
  std::vector<OpNeeds> need(count);
  for (unsigned i = 0; i < count; ++i) need[i] = needs_of(ops[i]);
  unsigned launched = 0;
  std::vector<unsigned> chosen, deferred;
  while (!pending.empty()) {
    uint64_t T = low, blocked_any = 0, blocked_diag = 0;
    unsigned nops = 0, nent = 0, nslots = 0;
    chosen.clear();
    deferred.clear();
    bool full = false;
    for (unsigned i : pending) {
      const OpNeeds& r = need[i];
      bool take = !full;
      if (take) take = (r.support & (r.diagonal ? blocked_any : (blocked_any | blocked_diag))) == 0;
      if (take) take = (unsigned)__builtin_popcountll(T | r.targets) <= kt;
      if (take && (nops + r.max_ops > (unsigned)kTileMaxOps || nent + r.max_entries > (unsigned)kTileMaxEntries ||
                   chosen.size() + 1 > (size_t)kTileMaxPhases - 1 || nslots + r.slots > (unsigned)kGradSlots)) {
        take = false;
        full = true;
      }
      if (take) {
        chosen.push_back(i);
        T |= r.targets;
        nops += r.max_ops;
        nent += r.max_entries;
        nslots += r.slots;
      } else {
        deferred.push_back(i);
        if (r.diagonal) blocked_diag |= r.support;
        else blocked_any |= r.support;
      }
    }
    // Widen the tile to kt positions (free: the pass reads every amplitude once anyway).
    for (unsigned p = 0; p < h->n && (unsigned)__builtin_popcountll(T) < kt; ++p) T |= uint64_t(1) << p;
    // Assemble; if the phases overflow the parameter block, keep the first half of the
    // chosen ops and return the rest to the stream in their original order.
    size_t keep = chosen.size();
    TileAssembler* a = nullptr;
    std::unique_ptr<TileAssembler> holder;
    for (;;) {
      holder.reset(new TileAssembler(T, tl));
      a = holder.get();
      {
        SweepBuilder b(a, kmax);
        for (size_t k = 0; k < keep; ++k) queue_op(b, ops[chosen[k]]);
        b.flush();
      }
      if (!a->overflow) break;
      if (keep <= 1) return fail(IQSG_EINVAL, "tile pass: one operation does not fit a pass");
      keep /= 2;
    }
    int st = h->prec == IQSG_COMPLEX_SP ? launch_tile<float>(h, lam, *a, grad) : launch_tile<double>(h, lam, *a, grad);
    if (st) return st;
    ++launched;
    if (keep < chosen.size()) {
      std::vector<unsigned> rest;
      rest.reserve(deferred.size() + chosen.size() - keep);
      std::merge(chosen.begin() + (std::ptrdiff_t)keep, chosen.end(), deferred.begin(), deferred.end(),
                 std::back_inserter(rest));
      deferred.swap(rest);
    }
    pending.swap(deferred);
  }
  if (passes) *passes = launched;
  return IQSG_OK;
}

}  // namespace iqsg
