// Host-side scheduling shared by the register sweeps (k_sweep.cu) and the shared-memory tile
// passes (k_tile.cu): op validation, and the builder that turns a gate stream into sweep
// programs (SweepParams) for a sink that launches them or collects them as tile phases.
#pragma once

#include <algorithm>
#include <cstring>
#include <vector>

#include "sweep.cuh"

namespace iqsg {

// Receives each finished sweep program instead of launching it (tile phases).
class SweepSink {
 public:
  virtual ~SweepSink() = default;
  virtual void take(const SweepParams& P, const GradMap& map) = 0;
};

// ---- greedy packing of a gate stream into sweeps ------------------------------------------
namespace {

bool is_one(double re, double im) { return re == 1.0 && im == 0.0; }
bool is_zero(double re, double im) { return re == 0.0 && im == 0.0; }

SweepEntry make_entry(double re, double im) {
  SweepEntry e;
  e.re = re;
  e.im = im;
  const df64::DF r = df64::split_host(re), i = df64::split_host(im);
  e.rh = r.h;
  e.rl = r.l;
  e.ih = i.h;
  e.il = i.l;
  return e;
}

uint8_t phase_flags(double re, double im) {
  if (re == -1.0 && im == 0.0) return SF_NEG;
  if (re == 0.0 && im == 1.0) return SF_ONE_I;
  if (re == 0.0 && im == -1.0) return SF_NEG_I;
  return SF_NONE;
}

bool is_x(const double* m) {
  return is_zero(m[0], m[1]) && is_one(m[2], m[3]) && is_one(m[4], m[5]) && is_zero(m[6], m[7]);
}

class SweepBuilder {
 public:
  SweepBuilder(iqsg_state* h, unsigned kmax) : h_(h), kmax_(kmax) { reset(); }
  // Adjoint mode: every gate acts on h and lam; gradient operations add into grad[param].
  SweepBuilder(iqsg_state* h, iqsg_state* lam, double* grad, unsigned kmax)
      : h_(h), lam_(lam), grad_(grad), kmax_(kmax) {
    reset();
  }
  // Collect mode: finished programs go to sink (positions stay data positions).
  SweepBuilder(SweepSink* sink, unsigned kmax) : h_(nullptr), sink_(sink), kmax_(kmax) { reset(); }

  // Slot of position p in the current sweep, or -1 when p is not active.
  int slot(unsigned p) {
    for (unsigned j = 0; j < P_.K; ++j)
      if (P_.pos[j] == p) return (int)j;
    return -1;
  }

  bool fits(const std::vector<unsigned>& targets, unsigned ops, unsigned entries, unsigned slots = 0) const {
    unsigned add = 0;
    for (unsigned t : targets) {
      bool have = false;
      for (unsigned j = 0; j < P_.K; ++j) have = have || P_.pos[j] == t;
      add += have ? 0u : 1u;
    }
    // A two-position operation opens a 2-wide sweep even when the width limit is 1.
    const unsigned kmax = std::max<unsigned>(kmax_, (unsigned)targets.size());
    return P_.K + add <= kmax && P_.nops + ops <= (unsigned)kSweepMaxOps &&
           nent_ + entries <= (unsigned)kSweepMaxEntries && map_.nslots + slots <= (unsigned)kGradSlots;
  }

  // Make room (flushing if necessary) and activate the target positions.
  void reserve(const std::vector<unsigned>& targets, unsigned ops, unsigned entries, unsigned slots = 0) {
    if (!fits(targets, ops, entries, slots)) flush();
    for (unsigned t : targets)
      if (slot(t) < 0) P_.pos[P_.K++] = t;
  }

  uint16_t add_entries(const double* m, unsigned count) {
    const uint16_t first = (uint16_t)nent_;
    for (unsigned k = 0; k < count; ++k) P_.ent[nent_++] = make_entry(m[2 * k], m[2 * k + 1]);
    return first;
  }

  void add_phase(uint64_t mask, uint64_t value, double re, double im) {
    if (is_one(re, im)) return;
    // A CZ (phase -1 where two bits are both set) joins the preceding CZ-run op of the same
    // bit distance: the product of CZ(a, a + d) over a set A of low bits is
    // (-1)^popcount(x & (x >> d) & A), and a repeated pair cancels (XOR into A).
    if (re == -1.0 && im == 0.0 && value == mask && __builtin_popcountll(mask) == 2) {
      const unsigned a = (unsigned)__builtin_ctzll(mask), b = 63u - (unsigned)__builtin_clzll(mask);
      const unsigned d = b - a;
      if (P_.nops && P_.ops[P_.nops - 1].kind == SW_CZSHIFT && P_.ops[P_.nops - 1].j0 == d) {
        P_.ops[P_.nops - 1].mask ^= uint64_t(1) << a;
        return;
      }
      reserve({}, 1, 0);
      SweepOp op{};
      op.kind = SW_CZSHIFT;
      op.j0 = (uint8_t)d;
      op.mask = uint64_t(1) << a;
      P_.ops[P_.nops++] = op;
      return;
    }
    reserve({}, 1, 1);
    SweepOp op{};
    op.kind = SW_PHASE;
    op.mask = mask;
    op.value = value;
    op.flags = phase_flags(re, im);
    const double e[2] = {re, im};
    op.ent = add_entries(e, 1);
    P_.ops[P_.nops++] = op;
  }

  // 2x2 on target t where all bits of cmask are 1 (cmask excludes t).
  void add_u2(unsigned t, uint64_t cmask, const double* m) {
    const uint64_t tb = uint64_t(1) << t;
    if (is_zero(m[2], m[3]) && is_zero(m[4], m[5])) {  // diagonal: phases only
      add_phase(cmask | tb, cmask, m[0], m[1]);
      add_phase(cmask | tb, cmask | tb, m[6], m[7]);
      return;
    }
    reserve({t}, 1, 4);
    SweepOp op{};
    op.kind = SW_U2;
    op.mask = cmask;
    op.j0 = (uint8_t)slot(t);
    op.flags = is_x(m) ? SF_X : SF_NONE;
    op.ent = add_entries(m, 4);
    P_.ops[P_.nops++] = op;
  }

  void add_u4(unsigned ph, unsigned pl, const double* m) {
    auto z = [&](int r, int c) { return is_zero(m[2 * (4 * r + c)], m[2 * (4 * r + c) + 1]); };
    bool diag = true, excitation = true;  // excitation: |00> and |11> only pick up phases
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) {
        if (r != c && !z(r, c)) diag = false;
        const bool inner = (r == 1 || r == 2) && (c == 1 || c == 2);
        if (r != c && !inner && !z(r, c)) excitation = false;
      }
    const uint64_t bh = uint64_t(1) << ph, bl = uint64_t(1) << pl;
    if (diag) {
      for (int k = 0; k < 4; ++k)
        add_phase(bh | bl, ((k & 2) ? bh : 0) | ((k & 1) ? bl : 0), m[2 * (5 * k)], m[2 * (5 * k) + 1]);
      return;
    }
    if (excitation) {
      double w[12];
      excitation_entries(ph, pl, m, w);
      const unsigned lo = std::min(ph, pl), hi = std::max(ph, pl);
      reserve({lo, hi}, 1, 6);
      SweepOp op{};
      op.kind = SW_EXC;
      op.j0 = (uint8_t)slot(lo);
      op.j1 = (uint8_t)slot(hi);
      op.ent = add_entries(w, 6);
      P_.ops[P_.nops++] = op;
      return;
    }
    reserve({ph, pl}, 1, 16);
    SweepOp op{};
    op.kind = SW_U4;
    op.j0 = (uint8_t)slot(ph);
    op.j1 = (uint8_t)slot(pl);
    op.ent = add_entries(m, 16);
    P_.ops[P_.nops++] = op;
  }

  // A 4x4 (rows 2*b(ph) + b(pl)) that maps |01> and |10> into each other and only scales
  // |00> and |11>, as the six SW_EXC entries (pair ordered lower position first).
  static bool is_excitation(const double* m) {
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) {
        const bool inner = (r == 1 || r == 2) && (c == 1 || c == 2);
        if (r != c && !inner && !is_zero(m[2 * (4 * r + c)], m[2 * (4 * r + c) + 1])) return false;
      }
    return true;
  }
  static void excitation_entries(unsigned ph, unsigned pl, const double* m, double* w) {
    auto e = [&](int r, int c, double* o) {
      o[0] = m[2 * (4 * r + c)];
      o[1] = m[2 * (4 * r + c) + 1];
    };
    const int a = pl < ph ? 1 : 2, b = pl < ph ? 2 : 1;  // row of (lower set), row of (higher set)
    e(0, 0, w);
    e(a, a, w + 2);
    e(a, b, w + 4);
    e(b, a, w + 6);
    e(b, b, w + 8);
    e(3, 3, w + 10);
  }

  void add_swaplike(unsigned p1, unsigned p2, const double* m) {
    const unsigned lo = std::min(p1, p2), hi = std::max(p1, p2);
    reserve({lo, hi}, 1, 4);
    SweepOp op{};
    op.kind = SW_SWAPLIKE;
    op.j0 = (uint8_t)slot(lo);
    op.j1 = (uint8_t)slot(hi);
    op.flags = is_x(m) ? SF_X : SF_NONE;
    op.ent = add_entries(m, 4);
    P_.ops[P_.nops++] = op;
  }

  // Adjoint mode: a parameterised excitation-preserving gate undone in one operation: the
  // gradient sum for M (4x4, rows 2*b(t0) + b(t1)), then the 4x4 gate g on both vectors.
  // Both matrices must have the excitation layout (is_excitation).
  void add_grad_and_excitation(unsigned t0, unsigned t1, const double* M, const double* g, unsigned param) {
    double w[24];
    excitation_entries(t0, t1, M, w);
    excitation_entries(t0, t1, g, w + 12);
    const unsigned lo = std::min(t0, t1), hi = std::max(t0, t1);
    reserve({lo, hi}, 1, 12, 1);
    SweepOp op{};
    op.kind = SW_EXCADJ;
    op.j0 = (uint8_t)slot(lo);
    op.j1 = (uint8_t)slot(hi);
    op.value = map_.nslots;
    map_.param[map_.nslots++] = param;
    op.ent = add_entries(w, 12);
    P_.ops[P_.nops++] = op;
  }

  // Adjoint mode: add Im <lam|M|psi> on the target positions into grad[param]; M is 2x2
  // (one target) or 4x4 (rows 2*b(t0) + b(t1)).
  void add_grad(unsigned ntargets, unsigned t0, unsigned t1, const double* m, unsigned param) {
    if (ntargets == 2 && is_excitation(m)) {
      double w[12];
      excitation_entries(t0, t1, m, w);
      const unsigned lo = std::min(t0, t1), hi = std::max(t0, t1);
      reserve({lo, hi}, 1, 6, 1);
      SweepOp op{};
      op.kind = SW_GRADEXC;
      op.j0 = (uint8_t)slot(lo);
      op.j1 = (uint8_t)slot(hi);
      op.value = map_.nslots;
      map_.param[map_.nslots++] = param;
      op.ent = add_entries(w, 6);
      P_.ops[P_.nops++] = op;
      return;
    }
    const unsigned ne = ntargets == 1 ? 4u : 16u;
    if (ntargets == 1) reserve({t0}, 1, ne, 1);
    else reserve({t0, t1}, 1, ne, 1);
    SweepOp op{};
    op.kind = ntargets == 1 ? SW_GRAD1 : SW_GRAD2;
    op.j0 = (uint8_t)slot(t0);
    op.j1 = ntargets == 1 ? 0 : (uint8_t)slot(t1);
    op.value = map_.nslots;
    map_.param[map_.nslots++] = param;
    op.ent = add_entries(m, ne);
    P_.ops[P_.nops++] = op;
  }

  void flush() {
    if (P_.nops) {
      std::copy(P_.pos, P_.pos + P_.K, P_.sorted);
      std::sort(P_.sorted, P_.sorted + P_.K);
      P_.native16 = h_ ? h_->native16 : 0u;
      if (sink_) sink_->take(P_, map_);
      else if (lam_) launch_sweep_adj(h_, lam_, P_, map_, grad_);
      else launch_sweep(h_, P_);
      ++launched_;
    }
    reset();
  }

  unsigned launched() const { return launched_; }

 private:
  void reset() {
    std::memset(&P_, 0, sizeof(P_));
    std::memset(&map_, 0, sizeof(map_));
    nent_ = 0;
  }
  iqsg_state* h_;
  iqsg_state* lam_ = nullptr;
  double* grad_ = nullptr;
  SweepSink* sink_ = nullptr;
  GradMap map_;
  unsigned kmax_;
  SweepParams P_;
  unsigned nent_ = 0;
  unsigned launched_ = 0;
};

}  // namespace

namespace {

// adjoint: the op list of iqsg_adjoint_ops (gradient ops allowed, parameter index < nparams).
int check_op(const iqsg_state* h, const iqsg_op& op, unsigned i, bool adjoint = false, unsigned nparams = 0) {
  auto bad = [&](const char* why) { return fail(IQSG_EINVAL, "iqsg_apply_ops: op %u: %s", i, why); };
  uint64_t seen = 0;
  auto use = [&](unsigned p) {
    if (p >= h->n) return false;
    if (seen & (uint64_t(1) << p)) return false;
    seen |= uint64_t(1) << p;
    return true;
  };
  switch (op.kind) {
    case IQSG_OP_1Q:
      if (!use(op.t0)) return bad("target out of range");
      break;
    case IQSG_OP_CTRL:
      if (op.nctrl > 4) return bad("more than 4 controls");
      for (unsigned c = 0; c < op.nctrl; ++c)
        if (!use(op.ctrl[c])) return bad("control out of range or repeated");
      if (!use(op.t0)) return bad("target out of range or equal to a control");
      break;
    case IQSG_OP_2Q:
    case IQSG_OP_SWAPLIKE:
    case IQSG_OP_DIAG2:
      if (!use(op.t0) || !use(op.t1)) return bad("positions out of range or equal");
      break;
    case IQSG_OP_PHASE:
      if (h->n < 64 && ((op.mask >> h->n) != 0)) return bad("phase mask beyond the register");
      if ((op.value & ~op.mask) != 0) return bad("phase value outside its mask");
      break;
    case IQSG_OP_GRAD1:
    case IQSG_OP_GRAD2:
      if (!adjoint) return bad("gradient ops belong to iqsg_adjoint_ops");
      if (op.value >= nparams) return bad("parameter index out of range");
      if (!use(op.t0)) return bad("target out of range");
      if (op.kind == IQSG_OP_GRAD2 && !use(op.t1)) return bad("positions out of range or equal");
      break;
    default:
      return bad("unknown kind");
  }
  return IQSG_OK;
}

// Queue one validated gate op on a builder.
void queue_op(SweepBuilder& b, const iqsg_op& op) {
  switch (op.kind) {
    case IQSG_OP_1Q:
      b.add_u2(op.t0, 0, op.m);
      break;
    case IQSG_OP_CTRL: {
      uint64_t cm = 0;
      for (unsigned c = 0; c < op.nctrl; ++c) cm |= uint64_t(1) << op.ctrl[c];
      b.add_u2(op.t0, cm, op.m);
      break;
    }
    case IQSG_OP_2Q:
      b.add_u4(op.t0, op.t1, op.m);
      break;
    case IQSG_OP_SWAPLIKE:
      b.add_swaplike(op.t0, op.t1, op.m);
      break;
    case IQSG_OP_DIAG2: {
      const uint64_t b1 = uint64_t(1) << op.t0, b2 = uint64_t(1) << op.t1;
      for (int k = 0; k < 4; ++k)
        b.add_phase(b1 | b2, ((k & 2) ? b1 : 0) | ((k & 1) ? b2 : 0), op.m[2 * k], op.m[2 * k + 1]);
      break;
    }
    case IQSG_OP_PHASE:
      b.add_phase(op.mask, op.value, op.m[0], op.m[1]);
      break;
    case IQSG_OP_GRAD1:
      b.add_grad(1, op.t0, 0, op.m, (unsigned)op.value);
      break;
    case IQSG_OP_GRAD2:
      b.add_grad(2, op.t0, op.t1, op.m, (unsigned)op.value);
      break;
  }
}

}  // namespace

}  // namespace iqsg
