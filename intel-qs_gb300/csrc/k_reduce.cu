// Reductions over the state: FP64 accumulation, two passes in a fixed order so results
// are bit-reproducible run to run. Pass 1: a fixed-size grid of blocks, each summing a
// grid-strided slice and writing one partial per block to scratch. Pass 2: one block
// sums the partials in index order and writes the result slot.
#include "iqsg_internal.cuh"

namespace iqsg {

namespace {

constexpr int kFinishThreads = 1024;

__device__ __forceinline__ uint64_t gtid() { return (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ uint64_t gstride() { return (uint64_t)gridDim.x * blockDim.x; }

template <bool MAX>
__device__ __forceinline__ double combine(double a, double b) {
  if constexpr (MAX) return a > b ? a : b;
  else return a + b;
}

// Block-wide reduction of NV doubles; thread 0 returns the totals.
template <int NV, bool MAX>
__device__ __forceinline__ void block_reduce(double (&v)[NV]) {
  __shared__ double sh[NV][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k)
    for (int o = 16; o > 0; o >>= 1) v[k] = combine<MAX>(v[k], __shfl_down_sync(0xffffffffu, v[k], o));
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k][warp] = v[k];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      v[k] = lane < nwarps ? sh[k][lane] : (MAX ? -1.0 : 0.0);
      for (int o = 16; o > 0; o >>= 1) v[k] = combine<MAX>(v[k], __shfl_down_sync(0xffffffffu, v[k], o));
    }
  }
}

// Pass 2: partials[k*stride + b] for b < nparts -> out[k].
template <int NV, bool MAX>
__global__ void __launch_bounds__(kFinishThreads) k_finish(const double* __restrict__ partials, int nparts,
                                                           double* __restrict__ out) {
  double v[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    v[k] = MAX ? -1.0 : 0.0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) v[k] = combine<MAX>(v[k], partials[k * kMaxPartials + b]);
  }
  block_reduce<NV, MAX>(v);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = v[k];
  }
}

// Pass 1 driver: F(i, acc[]) adds element i's contribution(s) into acc.
template <int NV, bool MAX, typename F>
__global__ void __launch_bounds__(kThreads) k_reduce(F f, uint64_t count, double* __restrict__ partials) {
  double acc[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) acc[k] = MAX ? -1.0 : 0.0;
  for (uint64_t i = gtid(); i < count; i += gstride()) f(i, acc);
  block_reduce<NV, MAX>(acc);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[k * kMaxPartials + blockIdx.x] = acc[k];
  }
}

template <typename V>
__device__ __forceinline__ double norm2(V a) {
  return (double)a.x * (double)a.x + (double)a.y * (double)a.y;
}

template <typename R>
struct ProbF {
  const typename V2<R>::type* s;
  unsigned pos;
  __device__ void operator()(uint64_t p, double (&acc)[1]) const {
    acc[0] += norm2(s[insert_zero(p, pos) | (uint64_t(1) << pos)]);
  }
};

// <psi|P|psi> for a Pauli string: P|j> = i^ny (-1)^popcount(j & zmask) |j ^ xmask>,
// zmask holding the Y and Z positions, xmask the X and Y positions. With xmask != 0 the
// pass visits pairs (j, j ^ xmask) with the top bit of xmask clear; each contributes
// 2 Re(i^ny (-1)^par(j) conj(psi_{j^x}) psi_j) (the two terms of the pair are equal).
template <typename R>
struct PauliF {
  const typename V2<R>::type* s;
  uint64_t xmask, zmask;
  unsigned top;  // highest bit of xmask (unused when xmask == 0)
  unsigned ny;   // number of Y factors, mod 4
  __device__ void operator()(uint64_t p, double (&acc)[2]) const {
    if (xmask == 0) {
      const double w = norm2(s[p]);
      acc[0] += (__popcll(p & zmask) & 1) ? -w : w;
      acc[1] += w;
      return;
    }
    const uint64_t j = insert_zero(p, top), k = j ^ xmask;
    const auto a = s[j], b = s[k];
    // c = conj(b) * a
    const double cr = (double)b.x * (double)a.x + (double)b.y * (double)a.y;
    const double ci = (double)b.x * (double)a.y - (double)b.y * (double)a.x;
    // Re(i^ny c): ny=0 -> cr, 1 -> -ci, 2 -> -cr, 3 -> ci
    double t = (ny & 1) ? ci : cr;
    if (((ny + 1) >> 1) & 1) t = -t;
    acc[0] += ((__popcll(j & zmask) & 1) ? -2.0 : 2.0) * t;
    acc[1] += norm2(a) + norm2(b);
  }
};

template <typename R>
struct Norm2F {
  const typename V2<R>::type* s;
  __device__ void operator()(uint64_t i, double (&acc)[1]) const { acc[0] += norm2(s[i]); }
};

template <typename R>
struct OverlapF {
  const typename V2<R>::type* a;  // self
  const typename V2<R>::type* b;  // psi
  __device__ void operator()(uint64_t i, double (&acc)[2]) const {
    const auto x = a[i], y = b[i];
    acc[0] += (double)y.x * (double)x.x + (double)y.y * (double)x.y;
    acc[1] += (double)y.x * (double)x.y - (double)y.y * (double)x.x;
  }
};

template <typename R>
struct MaxAbsDiffF {
  const typename V2<R>::type* a;
  const typename V2<R>::type* b;
  C1<R> f;
  __device__ void operator()(uint64_t i, double (&acc)[1]) const {
    const auto x = a[i], y = b[i];
    const R pr = f.re * y.x - f.im * y.y, pi = f.re * y.y + f.im * y.x;
    const double v = hypot((double)(x.x - pr), (double)(x.y - pi));
    acc[0] = v > acc[0] ? v : acc[0];
  }
};

template <typename R>
struct L2DiffF {
  const typename V2<R>::type* a;
  const typename V2<R>::type* b;
  __device__ void operator()(uint64_t i, double (&acc)[1]) const {
    const auto x = a[i], y = b[i];
    const double dr = (double)x.x - (double)y.x, di = (double)x.y - (double)y.y;
    acc[0] += dr * dr + di * di;
  }
};

template <typename R>
struct CostF {
  const typename V2<R>::type* s;
  const typename V2<R>::type* d;
  int power;
  __device__ void operator()(uint64_t i, double (&acc)[1]) const {
    const double c = (double)d[i].x;
    acc[0] += (power == 2 ? c * c : c) * norm2(s[i]);
  }
};

template <typename R>
struct MaxRealF {
  const typename V2<R>::type* s;
  __device__ void operator()(uint64_t i, double (&acc)[1]) const {
    const double v = (double)s[i].x;
    acc[0] = v > acc[0] ? v : acc[0];
  }
};

unsigned reduce_grid(uint64_t count) {
  unsigned g = grid_for(count, 4);
  return g > (unsigned)kMaxPartials ? (unsigned)kMaxPartials : g;
}

template <int NV, bool MAX, typename F>
void run(iqsg_state* h, const F& f, uint64_t count) {
  const unsigned g = reduce_grid(count);
  k_reduce<NV, MAX, F><<<g, kThreads, 0, h->stream>>>(f, count, h->scratch);
  k_finish<NV, MAX><<<1, kFinishThreads, 0, h->stream>>>(h->scratch, (int)g, h->scratch + kResultSlot);
}

}  // namespace

#define CAMPS(R, p) reinterpret_cast<const typename V2<R>::type*>(p)

template <typename R>
void reduce_probability(iqsg_state* h, unsigned pos) {
  run<1, false>(h, ProbF<R>{CAMPS(R, h->amps), pos}, h->N >> 1);
}

template <typename R>
void reduce_pauli(iqsg_state* h, uint64_t xmask, uint64_t zmask, unsigned ny) {
  unsigned top = 0;
  for (unsigned b = 0; b < 64; ++b)
    if ((xmask >> b) & 1u) top = b;
  const uint64_t count = xmask ? (h->N >> 1) : h->N;
  run<2, false>(h, PauliF<R>{CAMPS(R, h->amps), xmask, zmask, top, ny & 3u}, count);
}

template <typename R>
void reduce_norm2(iqsg_state* h) {
  run<1, false>(h, Norm2F<R>{CAMPS(R, h->amps)}, h->N);
}

template <typename R>
void reduce_overlap(iqsg_state* h, const void* psi) {
  run<2, false>(h, OverlapF<R>{CAMPS(R, h->amps), CAMPS(R, psi)}, h->N);
}

template <typename R>
void reduce_max_abs_diff(iqsg_state* h, const void* x, C1<R> f) {
  run<1, true>(h, MaxAbsDiffF<R>{CAMPS(R, h->amps), CAMPS(R, x), f}, h->N);
}

template <typename R>
void reduce_l2_diff(iqsg_state* h, const void* x) {
  run<1, false>(h, L2DiffF<R>{CAMPS(R, h->amps), CAMPS(R, x)}, h->N);
}

template <typename R>
void reduce_cost_expectation(iqsg_state* h, const void* diag, int power) {
  run<1, false>(h, CostF<R>{CAMPS(R, h->amps), CAMPS(R, diag), power}, h->N);
}

template <typename R>
void reduce_max_real(iqsg_state* h) {
  run<1, true>(h, MaxRealF<R>{CAMPS(R, h->amps)}, h->N);
}

#define INSTANTIATE_R(R)                                                         \
  template void reduce_probability<R>(iqsg_state*, unsigned);                    \
  template void reduce_pauli<R>(iqsg_state*, uint64_t, uint64_t, unsigned);      \
  template void reduce_norm2<R>(iqsg_state*);                                    \
  template void reduce_overlap<R>(iqsg_state*, const void*);                     \
  template void reduce_max_abs_diff<R>(iqsg_state*, const void*, C1<R>);         \
  template void reduce_l2_diff<R>(iqsg_state*, const void*);                     \
  template void reduce_cost_expectation<R>(iqsg_state*, const void*, int);       \
  template void reduce_max_real<R>(iqsg_state*);

INSTANTIATE_R(double)
INSTANTIATE_R(float)

}  // namespace iqsg
