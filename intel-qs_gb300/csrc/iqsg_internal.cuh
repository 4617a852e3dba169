// Internal declarations shared by the libiqsg translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "iqsg.h"

struct iqsg_state {
  unsigned n = 0;          // number of qubits
  int prec = IQSG_COMPLEX_DP;
  uint64_t N = 0;          // 2^n amplitudes
  void* amps = nullptr;    // device amplitudes (double2 or float2)
  bool owns = false;       // amps allocated by this register
  cudaStream_t stream = nullptr;
  bool owns_stream = false;
  int math = IQSG_MATH_NATIVE;
  bool df_storage = true;  // emulated FP64 runs of sweeps keep double-float pairs between sweeps
  uint64_t df_runs = 0;      // double-float storage runs started
  uint64_t df_launches = 0;  // kernels those runs launched
  int device = 0;
  double* scratch = nullptr;      // device: reduction partials + result slots
  double* host_result = nullptr;  // pinned host: reduction results
  void* tmp = nullptr;            // device: out-of-place permutation buffer (lazy)
  size_t tmp_bytes = 0;
  unsigned sweep_width = 0;       // fused-sweep width limit (0 = default for the precision)
  unsigned tile_qubits = 0;       // positions per shared-memory tile pass (0 = register sweeps only)
  bool bulk = false;              // fused passes through the bulk-copy pipeline (IQSG_OPT_SWEEP_PIPELINE)
  unsigned native16 = 0;          // emulated ComplexDP sweeps: share (in 16ths) of warps on the FP64 pipe
};

namespace iqsg {

constexpr int kThreads = 256;
// Reduction partials: one (or two) doubles per block of the first pass.
constexpr int kMaxPartials = 4096;
// scratch layout (doubles): [0, 2*kMaxPartials) partials, then 8 result slots.
constexpr int kResultSlot = 2 * kMaxPartials;
// scratch[kErrorSlot] (as unsigned long long): set by a kernel whose bounded wait ran out.
constexpr int kErrorSlot = 2 * kMaxPartials + 8;
// scratch[kRangeSlot] (as unsigned long long): set when a double-float storage run may not start.
constexpr int kRangeSlot = 2 * kMaxPartials + 9;
// scratch[kTableSlot ...]: small per-call tables (QAOA phases: 2 doubles per cut value).
constexpr int kTableSlot = 2 * kMaxPartials + 16;
constexpr int kTableDoubles = 2 * 1040;
constexpr int kScratchDoubles = kTableSlot + kTableDoubles;
// Registers from this size up use the bulk-copy pipelined sweep kernels.
constexpr unsigned kBulkMinQubits = 16;

// Records the error text for iqsg_last_error() and returns code.
int fail(int code, const char* fmt, ...);
// Maps a CUDA error to IQSG_EDEVICE (or IQSG_ENOMEM) with context; IQSG_OK on success.
int cuda_status(cudaError_t e, const char* what);
// Grid size for a grid-stride loop over `work` items, `per_thread` items per thread.
unsigned grid_for(uint64_t work, int per_thread);
// Launch facts cached per device (the device current at the call).
constexpr int kMaxDevices = 64;
int current_device();
int num_sms();
// Wait for the register's stream and report a device error word left by a bounded wait.
int sync_and_check(iqsg_state* h, const char* what);
int take_device_error(iqsg_state* h, unsigned long long word, const char* what);

template <typename R> struct V2;
template <> struct V2<double> { using type = double2; };
template <> struct V2<float> { using type = float2; };

template <typename R> struct M2 { R re[4], im[4]; };    // m00 m01 m10 m11
template <typename R> struct M4 { R re[16], im[16]; };  // row-major 4x4
template <typename R> struct C1 { R re, im; };

// Up to 9 sorted bit positions into which zeros are inserted to enumerate sub-blocks.
struct Positions {
  unsigned count;
  unsigned p[10];
};

__host__ __device__ __forceinline__ uint64_t insert_zero(uint64_t x, unsigned pos) {
  const uint64_t lo = x & ((uint64_t(1) << pos) - 1);
  return ((x ^ lo) << 1) | lo;
}

#if defined(__CUDACC__)
// (m0r + i m0i) a + (m1r + i m1i) b with an explicit FMA order, shared by the per-gate and
// the fused kernels so both produce bit-identical results.
template <typename R>
__device__ __forceinline__ void row2_fma(R m0r, R m0i, R m1r, R m1i, R ar, R ai, R br, R bi, R& orr, R& oi) {
  R t = m1i * bi;
  t = fma(m1r, br, -t);
  t = fma(-m0i, ai, t);
  orr = fma(m0r, ar, t);
  R u = m1i * br;
  u = fma(m1r, bi, u);
  u = fma(m0i, ar, u);
  oi = fma(m0r, ai, u);
}

// (fr + i fi) a, explicit FMA order (shared like row2_fma).
template <typename R>
__device__ __forceinline__ void cmul_fma(R fr, R fi, R ar, R ai, R& orr, R& oi) {
  orr = fma(fr, ar, -(fi * ai));
  oi = fma(fr, ai, fi * ar);
}

// Row of a 4x4 times (v0..v3): sum_c (mr_c + i mi_c) v_c, explicit FMA order.
template <typename R>
__device__ __forceinline__ void row4_fma(const R* mr, const R* mi, const R* vr, const R* vi, R& orr, R& oi) {
  R x = mr[0] * vr[0], y = mr[0] * vi[0];
  x = fma(-mi[0], vi[0], x);
  y = fma(mi[0], vr[0], y);
#pragma unroll
  for (int c = 1; c < 4; ++c) {
    x = fma(mr[c], vr[c], x);
    x = fma(-mi[c], vi[c], x);
    y = fma(mr[c], vi[c], y);
    y = fma(mi[c], vr[c], y);
  }
  orr = x;
  oi = y;
}
#endif

// ---- launchers (native kernels, k_gates.cu) ----
template <typename R> void launch_1q(iqsg_state* h, unsigned pos, const M2<R>& m);
template <typename R> void launch_1q_diag(iqsg_state* h, unsigned pos, C1<R> d0, C1<R> d1, bool touch0);
template <typename R> void launch_mc1q(iqsg_state* h, const Positions& zeros, uint64_t ctrl_mask, unsigned tpos, const M2<R>& m);
template <typename R> void launch_phase_mask(iqsg_state* h, const Positions& zeros, uint64_t ones, C1<R> d);
template <typename R> void launch_2q(iqsg_state* h, unsigned ph, unsigned pl, const M4<R>& m);
template <typename R> void launch_swaplike(iqsg_state* h, unsigned plo, unsigned phi, const M2<R>& m);
template <typename R> void launch_diag2(iqsg_state* h, unsigned p1, unsigned p2, const C1<R>* d);
template <typename R> void launch_cost_phase(iqsg_state* h, const void* diag, double gamma);
template <typename R> void launch_collapse(iqsg_state* h, unsigned pos, int value);
template <typename R> void launch_scale(iqsg_state* h, C1<R> f);
template <typename R> void launch_axpy(iqsg_state* h, const void* x, C1<R> f, bool unit);
template <typename R> void launch_fill(iqsg_state* h, C1<R> v);
template <typename R> void launch_permute(iqsg_state* h, const void* src, void* dst, const unsigned* src_bit_of_dst_bit);
template <typename R> void launch_maxcut_cost(iqsg_state* h, const int* edges_uv, unsigned num_edges, const unsigned* prog_pos);

// ---- reductions (k_reduce.cu); results land in h->scratch[kResultSlot + k] ----
template <typename R> void reduce_probability(iqsg_state* h, unsigned pos);
template <typename R> void reduce_pauli(iqsg_state* h, uint64_t xmask, uint64_t zmask, unsigned ny);
template <typename R> void reduce_norm2(iqsg_state* h);
template <typename R> void reduce_overlap(iqsg_state* h, const void* psi);
template <typename R> void reduce_max_abs_diff(iqsg_state* h, const void* x, C1<R> f);
template <typename R> void reduce_l2_diff(iqsg_state* h, const void* x);
template <typename R> void reduce_cost_expectation(iqsg_state* h, const void* diag, int power);
template <typename R> void reduce_max_real(iqsg_state* h);
// k_costfn.cu: weighted MaxCut cost vector (edge table of (u, v, w) doubles on the device) and
// cost histograms (out_dev: nbins device doubles; *bad counts values outside the histogram).
template <typename R> void launch_weighted_cost(iqsg_state* h, const double* edges, unsigned num_edges);
// k_costfn.cu: 11 state sums (-sum p ln p, -sum ln p over p > 0, sum p^k for k = 2..10) into out_dev.
template <typename R> void launch_state_stats(iqsg_state* h, double* out_dev);
template <typename R>
void launch_cost_hist(iqsg_state* psi, const void* diag, int mode, double max_value, double bin_width, int nbins,
                      double* out_dev, unsigned long long* bad);

// ---- emulated-FP64 gate kernels (k_emul.cu) ----
void launch_1q_emulated(iqsg_state* h, unsigned pos, const M2<double>& m);

// ---- fused sweeps (k_sweep.cu) ----
unsigned sweep_width(const iqsg_state* h);
// Tile passes (k_tile.cu): the tile size in positions for this register (0 = not used), and
// the scheduler that runs validated ops as tile passes (lam != NULL: adjoint passes).
unsigned tile_qubits(const iqsg_state* h, bool dual);
int tile_schedule(iqsg_state* h, iqsg_state* lam, const iqsg_op* ops, unsigned count, unsigned kt, unsigned kmax,
                  double* grad, unsigned* passes);

}  // namespace iqsg
