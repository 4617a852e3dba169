// Fused sweeps: one pass over the state that applies an ordered list of gate operations.
//
// A sweep has K "active" positions (0 <= K <= 4). Each thread owns groups of 2^K amplitudes:
// the indices that differ only in the active bits. Non-diagonal operations act inside a
// group (2x2 on one active bit, 4x4 or swap-type on two), so the group is loaded once,
// every operation is applied in registers in program order, and the group is stored once.
// Diagonal operations (phases, controlled phases, CZ, the ApplyDiag entries) act on single
// amplitudes selected by their index bits and may involve any position, active or not.
// Control bits may sit on any position too. Applying the list group by group gives exactly
// the result of applying it operation by operation, because a group is closed under every
// operation of the sweep.
#pragma once

#include <vector>

#include "df64.cuh"
#include "iqsg_internal.cuh"

namespace iqsg {

constexpr int kSweepMaxK = 4;
constexpr int kSweepMaxOps = 48;
constexpr int kSweepMaxEntries = 160;
constexpr int kGradSlots = 16;  // gradient accumulators per adjoint sweep

enum SweepKind : uint8_t {
  SW_U2 = 0,        // 2x2 on active bit j0, applied where (idx & mask) == mask
  SW_PHASE = 1,     // amp *= entry where (idx & mask) == value
  SW_U4 = 2,        // 4x4 on active bits (j0 = high, j1 = low), where (idx & mask) == mask
  SW_SWAPLIKE = 3,  // 2x2 on the (j0 = 1, j1 = 0) / (j0 = 0, j1 = 1) pair, where (idx & mask) == mask
  SW_GRAD1 = 4,     // adjoint sweeps only: accumulate Im <w|M|v>, M 2x2 on j0
  SW_GRAD2 = 5,     // adjoint sweeps only: accumulate Im <w|M|v>, M 4x4 on (j0 high, j1 low)
  SW_EXC = 6,       // excitation-preserving 4x4 on (j0 = lower, j1 = higher position): entry 0
                    // scales |00>, entries 1-4 are the 2x2 on (|lo=1,hi=0>, |lo=0,hi=1>), entry 5
                    // scales |11>; where (idx & mask) == mask
  SW_GRADEXC = 7,   // adjoint sweeps only: Im <w|M|v> for M with the SW_EXC layout
  SW_CZSHIFT = 8,   // amp *= (-1)^popcount(idx & (idx >> j0) & mask): the product of CZ(a, a + j0)
                    // over the bits a of mask (exact sign flips)
  SW_EXCADJ = 9,    // adjoint sweeps only: SW_GRADEXC with entries 0-5, then SW_EXC with entries
                    // 6-11 on both vectors, quad by quad (one parameterised excitation gate undone)
};

enum SweepFlags : uint8_t {
  SF_NONE = 0,
  SF_NEG = 1,    // PHASE by -1: exact sign flip
  SF_X = 2,      // U2/SWAPLIKE with m = [[0,1],[1,0]]: exact exchange
  SF_ONE_I = 4,  // PHASE by +i: exact (re, im) -> (-im, re)
  SF_NEG_I = 8,  // PHASE by -i: exact (re, im) -> (im, -re)
};

struct SweepOp {
  uint64_t mask, value;
  uint16_t ent;  // first matrix entry
  uint8_t kind, flags;
  uint8_t j0, j1;
  uint8_t pad[2];
};

// One complex matrix entry in both representations: native (re, im) in the register's
// precision, and the double-float split used by the emulated path.
struct SweepEntry {
  double re, im;
  float rh, rl, ih, il;
};

struct SweepParams {
  unsigned K;
  unsigned pos[kSweepMaxK];     // active slot bit j <-> position pos[j]
  unsigned sorted[kSweepMaxK];  // active positions ascending (zero insertion)
  unsigned nops;
  unsigned native16;  // emulated FP64 sweeps: warps whose group block (g / 32) % 16 < native16 use FP64
  SweepOp ops[kSweepMaxOps];
  SweepEntry ent[kSweepMaxEntries];
};

// ---- arithmetic policies -----------------------------------------------------------------

// IEEE arithmetic in R (double or float): the same formulas as the per-gate kernels.
template <typename R>
struct NativeArith {
  struct VT {
    R re, im;
  };
  // FP32 uses the float head of the entry, which is the double rounded to nearest float
  // (no double -> float conversion on the device).
  __device__ static __forceinline__ R re_of(const SweepEntry& e) {
    if constexpr (sizeof(R) == 4) return e.rh;
    else return e.re;
  }
  __device__ static __forceinline__ R im_of(const SweepEntry& e) {
    if constexpr (sizeof(R) == 4) return e.ih;
    else return e.im;
  }
  // r0 = m0 a + m1 b
  __device__ static __forceinline__ VT row(const SweepEntry& m0, const SweepEntry& m1, const VT& a, const VT& b) {
    VT o;
    row2_fma<R>(re_of(m0), im_of(m0), re_of(m1), im_of(m1), a.re, a.im, b.re, b.im, o.re, o.im);
    return o;
  }
  __device__ static __forceinline__ VT mul(const SweepEntry& f, const VT& a) {
    VT o;
    cmul_fma<R>(re_of(f), im_of(f), a.re, a.im, o.re, o.im);
    return o;
  }
  // row of a 4x4: sum_c m_c v_c
  __device__ static __forceinline__ VT row4(const SweepEntry* m, const VT* v) {
    R mr[4], mi[4], vr[4], vi[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      mr[c] = re_of(m[c]);
      mi[c] = im_of(m[c]);
      vr[c] = v[c].re;
      vi[c] = v[c].im;
    }
    VT o;
    row4_fma<R>(mr, mi, vr, vi, o.re, o.im);
    return o;
  }
};

// Double-float arithmetic on FP64 data (see df64.cuh); VT holds (h, l) pairs.
struct DF64Arith {
  struct VT {
    df64::DF re, im;
  };
  // sum of n double-float products c_k * x_k, c given as (h, l) constants
  template <int NT>
  __device__ static __forceinline__ df64::DF dot(const float* ch, const float* cl, const df64::DF* x) {
    float ph, pl;
    df64::Acc s;
    df64::prod(ch[0], cl[0], x[0].h, x[0].l, ph, pl);
    df64::acc_init(s, ph, pl);
#pragma unroll
    for (int k = 1; k < NT; ++k) {
      df64::prod(ch[k], cl[k], x[k].h, x[k].l, ph, pl);
      df64::acc_add(s, ph, pl);
    }
    df64::DF r;
    r.h = df64::add_rn(s.h, s.l);  // Fast2Sum renormalisation: |s.l| << |s.h|
    r.l = df64::sub_rn(s.l, df64::sub_rn(r.h, s.h));
    return r;
  }
  __device__ static __forceinline__ VT row(const SweepEntry& m0, const SweepEntry& m1, const VT& a, const VT& b) {
    const float reh[4] = {m0.rh, -m0.ih, m1.rh, -m1.ih}, rel[4] = {m0.rl, -m0.il, m1.rl, -m1.il};
    const float imh[4] = {m0.rh, m0.ih, m1.rh, m1.ih}, iml[4] = {m0.rl, m0.il, m1.rl, m1.il};
    const df64::DF xr[4] = {a.re, a.im, b.re, b.im};
    const df64::DF xi[4] = {a.im, a.re, b.im, b.re};
    VT o;
    o.re = dot<4>(reh, rel, xr);
    o.im = dot<4>(imh, iml, xi);
    return o;
  }
  __device__ static __forceinline__ VT mul(const SweepEntry& f, const VT& a) {
    const float reh[2] = {f.rh, -f.ih}, rel[2] = {f.rl, -f.il};
    const float imh[2] = {f.rh, f.ih}, iml[2] = {f.rl, f.il};
    const df64::DF xr[2] = {a.re, a.im}, xi[2] = {a.im, a.re};
    VT o;
    o.re = dot<2>(reh, rel, xr);
    o.im = dot<2>(imh, iml, xi);
    return o;
  }
  __device__ static __forceinline__ VT row4(const SweepEntry* m, const VT* v) {
    float reh[8], rel[8], imh[8], iml[8];
    df64::DF xr[8], xi[8];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      reh[2 * c] = m[c].rh; rel[2 * c] = m[c].rl; reh[2 * c + 1] = -m[c].ih; rel[2 * c + 1] = -m[c].il;
      imh[2 * c] = m[c].rh; iml[2 * c] = m[c].rl; imh[2 * c + 1] = m[c].ih; iml[2 * c + 1] = m[c].il;
      xr[2 * c] = v[c].re; xr[2 * c + 1] = v[c].im;
      xi[2 * c] = v[c].im; xi[2 * c + 1] = v[c].re;
    }
    VT o;
    o.re = dot<8>(reh, rel, xr);
    o.im = dot<8>(imh, iml, xi);
    return o;
  }
};

// ---- exact operations common to both ----------------------------------------------------
__device__ __forceinline__ double cneg(double x) { return -x; }
__device__ __forceinline__ float cneg(float x) { return -x; }
__device__ __forceinline__ df64::DF cneg(df64::DF x) {
  x.h = -x.h;
  x.l = -x.l;
  return x;
}
template <typename VT>
__device__ __forceinline__ void vt_neg(VT& a) {
  a.re = cneg(a.re);
  a.im = cneg(a.im);
}
// Multiply by +i: (re, im) -> (-im, re); by -i: (re, im) -> (im, -re). Exact.
template <typename VT>
__device__ __forceinline__ void vt_mul_i(VT& a, bool plus) {
  const auto re = a.re;
  if (plus) {
    a.re = cneg(a.im);
    a.im = re;
  } else {
    a.re = a.im;
    a.im = cneg(re);
  }
}

// ---- the op interpreter -----------------------------------------------------------------

template <typename A, int K, int J>
__device__ __forceinline__ void op_u2(const SweepEntry* E, const SweepOp& op, typename A::VT* v, const uint64_t* idx,
                                      unsigned& tm) {
  constexpr int G = 1 << K, B = 1 << J;
  const SweepEntry* m = E + op.ent;
#pragma unroll
  for (int s = 0; s < G; ++s) {
    if (s & B) continue;
    if (op.mask && (idx[s] & op.mask) != op.mask) continue;
    typename A::VT a = v[s], b = v[s | B];
    tm |= (1u << s) | (1u << (s | B));
    if (op.flags & SF_X) {
      v[s] = b;
      v[s | B] = a;
    } else {
      v[s] = A::row(m[0], m[1], a, b);
      v[s | B] = A::row(m[2], m[3], a, b);
    }
  }
}

template <typename A, int K, int JH, int JL>
__device__ __forceinline__ void op_u4(const SweepEntry* E, const SweepOp& op, typename A::VT* v, const uint64_t* idx,
                                      unsigned& tm) {
  constexpr int G = 1 << K, BH = 1 << JH, BL = 1 << JL;
  const SweepEntry* m = E + op.ent;
#pragma unroll
  for (int s = 0; s < G; ++s) {
    if (s & (BH | BL)) continue;
    if (op.mask && (idx[s] & op.mask) != op.mask) continue;
    const typename A::VT q[4] = {v[s], v[s | BL], v[s | BH], v[s | BH | BL]};
    tm |= (1u << s) | (1u << (s | BL)) | (1u << (s | BH)) | (1u << (s | BH | BL));
    v[s] = A::row4(m, q);
    v[s | BL] = A::row4(m + 4, q);
    v[s | BH] = A::row4(m + 8, q);
    v[s | BH | BL] = A::row4(m + 12, q);
  }
}

template <typename A, int K, int JLO, int JHI>
__device__ __forceinline__ void op_swaplike(const SweepEntry* E, const SweepOp& op, typename A::VT* v,
                                            const uint64_t* idx, unsigned& tm) {
  constexpr int G = 1 << K, BL = 1 << JLO, BH = 1 << JHI;
  const SweepEntry* m = E + op.ent;
#pragma unroll
  for (int s = 0; s < G; ++s) {
    if (s & (BH | BL)) continue;
    if (op.mask && (idx[s] & op.mask) != op.mask) continue;
    typename A::VT a = v[s | BL], b = v[s | BH];
    tm |= (1u << (s | BL)) | (1u << (s | BH));
    if (op.flags & SF_X) {
      v[s | BL] = b;
      v[s | BH] = a;
    } else {
      v[s | BL] = A::row(m[0], m[1], a, b);
      v[s | BH] = A::row(m[2], m[3], a, b);
    }
  }
}

template <typename A, int K, int JLO, int JHI>
__device__ __forceinline__ void op_exc(const SweepEntry* E, const SweepOp& op, typename A::VT* v, const uint64_t* idx,
                                       unsigned& tm) {
  constexpr int G = 1 << K, BL = 1 << JLO, BH = 1 << JHI;
  const SweepEntry* m = E + op.ent;
#pragma unroll
  for (int s = 0; s < G; ++s) {
    if (s & (BH | BL)) continue;
    if (op.mask && (idx[s] & op.mask) != op.mask) continue;
    tm |= (1u << s) | (1u << (s | BL)) | (1u << (s | BH)) | (1u << (s | BH | BL));
    const typename A::VT a = v[s | BL], b = v[s | BH];
    v[s] = A::mul(m[0], v[s]);
    v[s | BL] = A::row(m[1], m[2], a, b);
    v[s | BH] = A::row(m[3], m[4], a, b);
    v[s | BH | BL] = A::mul(m[5], v[s | BH | BL]);
  }
}

template <typename A, int K>
__device__ __forceinline__ void op_phase(const SweepEntry* E, const SweepOp& op, typename A::VT* v, const uint64_t* idx,
                                         unsigned& tm) {
  constexpr int G = 1 << K;
  const SweepEntry& f = E[op.ent];
#pragma unroll
  for (int s = 0; s < G; ++s) {
    if ((idx[s] & op.mask) != op.value) continue;
    tm |= 1u << s;
    if (op.flags & SF_NEG) vt_neg(v[s]);
    else if (op.flags & SF_ONE_I) vt_mul_i(v[s], true);
    else if (op.flags & SF_NEG_I) vt_mul_i(v[s], false);
    else v[s] = A::mul(f, v[s]);
  }
}

template <typename A, int K>
__device__ __forceinline__ void op_czshift(const SweepOp& op, typename A::VT* v, const uint64_t* idx, unsigned& tm) {
  constexpr int G = 1 << K;
#pragma unroll
  for (int s = 0; s < G; ++s) {
    if (__popcll(idx[s] & (idx[s] >> op.j0) & op.mask) & 1) {
      vt_neg(v[s]);
      tm |= 1u << s;
    }
  }
}

// One operation on one group. A runtime active-bit index is dispatched to a compile-time
// one, so the group stays in registers (no dynamic register indexing).
template <typename A, int K>
__device__ __forceinline__ void apply_op(const SweepEntry* E, const SweepOp& op, typename A::VT* v,
                                         const uint64_t* idx, unsigned& tm) {
  switch (op.kind) {
    case SW_PHASE:
      op_phase<A, K>(E, op, v, idx, tm);
      break;
    case SW_CZSHIFT:
      op_czshift<A, K>(op, v, idx, tm);
      break;
    case SW_U2:
      if constexpr (K >= 1) {
        switch (op.j0) {
          case 0: op_u2<A, K, 0>(E, op, v, idx, tm); break;
          case 1: if constexpr (K >= 2) op_u2<A, K, (K >= 2 ? 1 : 0)>(E, op, v, idx, tm); break;
          case 2: if constexpr (K >= 3) op_u2<A, K, (K >= 3 ? 2 : 0)>(E, op, v, idx, tm); break;
          case 3: if constexpr (K >= 4) op_u2<A, K, (K >= 4 ? 3 : 0)>(E, op, v, idx, tm); break;
        }
      }
      break;
    case SW_U4:
    case SW_SWAPLIKE:
    case SW_EXC:
      if constexpr (K >= 2) {
        const int kind = op.kind;
        const int a = op.j0, b = op.j1;
#define IQSG_PAIR_CASE(X, Y)                                                               \
  if (a == X && b == Y) {                                                                  \
    if constexpr (K > (X > Y ? X : Y)) {                                                   \
      if (kind == SW_U4) op_u4<A, K, X, Y>(E, op, v, idx, tm);                             \
      else if (kind == SW_SWAPLIKE) op_swaplike<A, K, X, Y>(E, op, v, idx, tm);            \
      else op_exc<A, K, X, Y>(E, op, v, idx, tm);                                          \
    }                                                                                      \
  }
        IQSG_PAIR_CASE(0, 1) IQSG_PAIR_CASE(1, 0) IQSG_PAIR_CASE(0, 2) IQSG_PAIR_CASE(2, 0)
        IQSG_PAIR_CASE(1, 2) IQSG_PAIR_CASE(2, 1) IQSG_PAIR_CASE(0, 3) IQSG_PAIR_CASE(3, 0)
        IQSG_PAIR_CASE(1, 3) IQSG_PAIR_CASE(3, 1) IQSG_PAIR_CASE(2, 3) IQSG_PAIR_CASE(3, 2)
#undef IQSG_PAIR_CASE
      }
      break;
    default:
      break;
  }
}

// Apply every operation of the sweep to one group, in order. Bit s of tm records that slot s
// was written.
template <typename A, int K>
__device__ __forceinline__ void run_ops(const SweepParams& P, typename A::VT* v, const uint64_t* idx, unsigned& tm) {
#pragma unroll 1
  for (unsigned o = 0; o < P.nops; ++o) apply_op<A, K>(P.ent, P.ops[o], v, idx, tm);
}

// ---- adjoint (two-vector) sweeps --------------------------------------------------------
//
// The group of psi (v) and the group of lambda (w) are held together. Gate operations act
// on both; a gradient operation (SW_GRAD1: 2x2 M on active bit j0; SW_GRAD2: 4x4 M on
// active bits j0 = high, j1 = low; both where (idx & mask) == mask) adds
// Im sum_x conj(w_x) (M v)_x over the group to accumulator op.value.

template <typename R>
__device__ __forceinline__ R im_cdot(const typename NativeArith<R>::VT& l, const typename NativeArith<R>::VT& x) {
  return l.re * x.im - l.im * x.re;
}

template <typename R, int K, int J>
__device__ __forceinline__ R grad1(const SweepEntry* E, const SweepOp& op, const typename NativeArith<R>::VT* v,
                                   const typename NativeArith<R>::VT* w, const uint64_t* idx) {
  using A = NativeArith<R>;
  constexpr int G = 1 << K, B = 1 << J;
  const SweepEntry* m = E + op.ent;
  R c = 0;
#pragma unroll
  for (int s = 0; s < G; ++s) {
    if (s & B) continue;
    if (op.mask && (idx[s] & op.mask) != op.mask) continue;
    const typename A::VT a = v[s], b = v[s | B];
    c += im_cdot<R>(w[s], A::row(m[0], m[1], a, b)) + im_cdot<R>(w[s | B], A::row(m[2], m[3], a, b));
  }
  return c;
}

template <typename R, int K, int JH, int JL>
__device__ __forceinline__ R grad2(const SweepEntry* E, const SweepOp& op, const typename NativeArith<R>::VT* v,
                                   const typename NativeArith<R>::VT* w, const uint64_t* idx) {
  using A = NativeArith<R>;
  constexpr int G = 1 << K, BH = 1 << JH, BL = 1 << JL;
  const SweepEntry* m = E + op.ent;
  R c = 0;
#pragma unroll
  for (int s = 0; s < G; ++s) {
    if (s & (BH | BL)) continue;
    if (op.mask && (idx[s] & op.mask) != op.mask) continue;
    const typename A::VT q[4] = {v[s], v[s | BL], v[s | BH], v[s | BH | BL]};
    c += im_cdot<R>(w[s], A::row4(m, q)) + im_cdot<R>(w[s | BL], A::row4(m + 4, q)) +
         im_cdot<R>(w[s | BH], A::row4(m + 8, q)) + im_cdot<R>(w[s | BH | BL], A::row4(m + 12, q));
  }
  return c;
}

template <typename R, int K, int JLO, int JHI>
__device__ __forceinline__ R grad_exc(const SweepEntry* E, const SweepOp& op, const typename NativeArith<R>::VT* v,
                                      const typename NativeArith<R>::VT* w, const uint64_t* idx) {
  using A = NativeArith<R>;
  constexpr int G = 1 << K, BL = 1 << JLO, BH = 1 << JHI;
  const SweepEntry* m = E + op.ent;
  R c = 0;
#pragma unroll
  for (int s = 0; s < G; ++s) {
    if (s & (BH | BL)) continue;
    if (op.mask && (idx[s] & op.mask) != op.mask) continue;
    const typename A::VT a = v[s | BL], b = v[s | BH];
    c += im_cdot<R>(w[s], A::mul(m[0], v[s])) + im_cdot<R>(w[s | BL], A::row(m[1], m[2], a, b)) +
         im_cdot<R>(w[s | BH], A::row(m[3], m[4], a, b)) + im_cdot<R>(w[s | BH | BL], A::mul(m[5], v[s | BH | BL]));
  }
  return c;
}

template <typename R, int K, int JLO, int JHI>
__device__ __forceinline__ R excadj(const SweepEntry* E, const SweepOp& op, typename NativeArith<R>::VT* v,
                                    typename NativeArith<R>::VT* w, const uint64_t* idx, unsigned& tm) {
  using A = NativeArith<R>;
  constexpr int G = 1 << K, BL = 1 << JLO, BH = 1 << JHI;
  const SweepEntry* m = E + op.ent;
  const SweepEntry* g = m + 6;
  R c = 0;
#pragma unroll
  for (int s = 0; s < G; ++s) {
    if (s & (BH | BL)) continue;
    if (op.mask && (idx[s] & op.mask) != op.mask) continue;
    tm |= (1u << s) | (1u << (s | BL)) | (1u << (s | BH)) | (1u << (s | BH | BL));
    const typename A::VT a = v[s | BL], b = v[s | BH], la = w[s | BL], lb = w[s | BH];
    c += im_cdot<R>(w[s], A::mul(m[0], v[s])) + im_cdot<R>(la, A::row(m[1], m[2], a, b)) +
         im_cdot<R>(lb, A::row(m[3], m[4], a, b)) + im_cdot<R>(w[s | BH | BL], A::mul(m[5], v[s | BH | BL]));
    v[s] = A::mul(g[0], v[s]);
    v[s | BL] = A::row(g[1], g[2], a, b);
    v[s | BH] = A::row(g[3], g[4], a, b);
    v[s | BH | BL] = A::mul(g[5], v[s | BH | BL]);
    w[s] = A::mul(g[0], w[s]);
    w[s | BL] = A::row(g[1], g[2], la, lb);
    w[s | BH] = A::row(g[3], g[4], la, lb);
    w[s | BH | BL] = A::mul(g[5], w[s | BH | BL]);
  }
  return c;
}

template <typename R, int K>
__device__ __forceinline__ R excadj_op(const SweepEntry* E, const SweepOp& op, typename NativeArith<R>::VT* v,
                                       typename NativeArith<R>::VT* w, const uint64_t* idx, unsigned& tm) {
  if constexpr (K >= 2) {
    const int a = op.j0, b = op.j1;
#define IQSG_EXCADJ_CASE(X, Y)                                      \
  if (a == X && b == Y) {                                           \
    if constexpr (K > (X > Y ? X : Y)) return excadj<R, K, X, Y>(E, op, v, w, idx, tm); \
  }
    IQSG_EXCADJ_CASE(0, 1) IQSG_EXCADJ_CASE(1, 0) IQSG_EXCADJ_CASE(0, 2) IQSG_EXCADJ_CASE(2, 0)
    IQSG_EXCADJ_CASE(1, 2) IQSG_EXCADJ_CASE(2, 1) IQSG_EXCADJ_CASE(0, 3) IQSG_EXCADJ_CASE(3, 0)
    IQSG_EXCADJ_CASE(1, 3) IQSG_EXCADJ_CASE(3, 1) IQSG_EXCADJ_CASE(2, 3) IQSG_EXCADJ_CASE(3, 2)
#undef IQSG_EXCADJ_CASE
  }
  return R(0);
}

template <typename R, int K>
__device__ __forceinline__ R grad_op(const SweepEntry* E, const SweepOp& op, const typename NativeArith<R>::VT* v,
                                     const typename NativeArith<R>::VT* w, const uint64_t* idx) {
  if (op.kind == SW_GRAD1) {
    if constexpr (K >= 1) {
      switch (op.j0) {
        case 0: return grad1<R, K, 0>(E, op, v, w, idx);
        case 1: if constexpr (K >= 2) return grad1<R, K, (K >= 2 ? 1 : 0)>(E, op, v, w, idx); break;
        case 2: if constexpr (K >= 3) return grad1<R, K, (K >= 3 ? 2 : 0)>(E, op, v, w, idx); break;
        case 3: if constexpr (K >= 4) return grad1<R, K, (K >= 4 ? 3 : 0)>(E, op, v, w, idx); break;
      }
    }
    return R(0);
  }
  if constexpr (K >= 2) {
    const int a = op.j0, b = op.j1;
    const bool exc = op.kind == SW_GRADEXC;
#define IQSG_GRAD_CASE(X, Y)                                         \
  if (a == X && b == Y) {                                            \
    if constexpr (K > (X > Y ? X : Y)) return exc ? grad_exc<R, K, X, Y>(E, op, v, w, idx) : grad2<R, K, X, Y>(E, op, v, w, idx); \
  }
    IQSG_GRAD_CASE(0, 1) IQSG_GRAD_CASE(1, 0) IQSG_GRAD_CASE(0, 2) IQSG_GRAD_CASE(2, 0)
    IQSG_GRAD_CASE(1, 2) IQSG_GRAD_CASE(2, 1) IQSG_GRAD_CASE(0, 3) IQSG_GRAD_CASE(3, 0)
    IQSG_GRAD_CASE(1, 3) IQSG_GRAD_CASE(3, 1) IQSG_GRAD_CASE(2, 3) IQSG_GRAD_CASE(3, 2)
#undef IQSG_GRAD_CASE
  }
  return R(0);
}

template <typename R, int K>
__device__ __forceinline__ void run_ops_dual(const SweepParams& P, typename NativeArith<R>::VT* v,
                                             typename NativeArith<R>::VT* w, const uint64_t* idx, unsigned& tm,
                                             R* acc) {
  using A = NativeArith<R>;
#pragma unroll 1
  for (unsigned o = 0; o < P.nops; ++o) {
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
}

// Host side: launch one sweep on the register (k_sweep.cu).
void launch_sweep(iqsg_state* h, const SweepParams& P);
// Emulated-FP64 sweeps with the state held as double-float pairs between them (k_sweep.cu).
void launch_df_storage_run(iqsg_state* h, const std::vector<SweepParams>& progs);

// Host side: one adjoint sweep over psi and lam; gradient slot s adds into grad[param[s]]
// (a device array of doubles).
struct GradMap {
  unsigned nslots;
  unsigned param[kGradSlots];
};
void launch_sweep_adj(iqsg_state* psi, iqsg_state* lam, const SweepParams& P, const GradMap& map, double* grad);

}  // namespace iqsg
