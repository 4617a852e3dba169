// Cost-function helpers of QAOA on the GPU -- the weighted MaxCut cost vector and histograms of
// |psi|^2 over the cost values (src/qaoa_features.cpp:153-239, :335-540) -- and the state
// statistics of Entropy / GoogleStats (src/qureg_utils.cpp:303-450).
#include "iqsg_internal.cuh"

namespace iqsg {

namespace {

// diag[x] = sum_e w_e [bit u_e of x != bit v_e of x], in FP64 then rounded to R. The edge
// table (u, v, w as doubles) is staged in shared memory.
template <typename R>
__global__ void __launch_bounds__(kThreads) k_weighted_cost(typename V2<R>::type* __restrict__ diag, uint64_t N,
                                                            const double* __restrict__ edges, unsigned num_edges) {
  extern __shared__ double sh_e[];
  for (unsigned e = threadIdx.x; e < 3 * num_edges; e += blockDim.x) sh_e[e] = edges[e];
  __syncthreads();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
    double cut = 0.0;
    for (unsigned e = 0; e < num_edges; ++e) {
      const unsigned pu = (unsigned)sh_e[3 * e], pv = (unsigned)sh_e[3 * e + 1];
      if (((i >> pu) ^ (i >> pv)) & 1u) cut += sh_e[3 * e + 2];
    }
    typename V2<R>::type v;
    v.x = (R)cut;
    v.y = 0;
    diag[i] = v;
  }
}

// Bin of a cost value, as the reference computes it; -1 when the value is outside the
// histogram (the reference asserts there).
__device__ __forceinline__ int hist_bin(double cut, int mode, double max_value, double bin_width) {
  if (mode == IQSG_HIST_INTEGER) {
    const int c = (int)cut;  // truncation, as (int)(diag[i].real())
    return (c >= 0 && (double)c <= max_value) ? c : -1;
  }
  if (!(cut >= -1e-7 && cut <= max_value + 1e-7)) return -1;
  return mode == IQSG_HIST_ROUNDED ? (int)floor(cut + 1e-7) : (int)floor(cut / bin_width + 1e-7);
}

constexpr int kHistChunk = 16;  // bins per pass, kept in registers

// Bins [b0, b0 + 16) of the histogram: per-thread sums in registers (static indices), fixed-
// order block sums into partials[block * 16 + j]; out-of-range values counted into *bad.
template <typename R>
__global__ void __launch_bounds__(kThreads) k_cost_hist(const typename V2<R>::type* __restrict__ psi,
                                                        const typename V2<R>::type* __restrict__ diag, uint64_t N,
                                                        int mode, double max_value, double bin_width, int nbins, int b0,
                                                        double* __restrict__ partials,
                                                        unsigned long long* __restrict__ bad) {
  double acc[kHistChunk];
#pragma unroll
  for (int j = 0; j < kHistChunk; ++j) acc[j] = 0.0;
  unsigned long long nbad = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
    const int b = hist_bin((double)diag[i].x, mode, max_value, bin_width);
    if (b < 0 || b >= nbins) {
      ++nbad;
      continue;
    }
    const typename V2<R>::type a = psi[i];
    const double p = (double)a.x * a.x + (double)a.y * a.y;
#pragma unroll
    for (int j = 0; j < kHistChunk; ++j)
      if (b - b0 == j) acc[j] += p;
  }
  if (b0 == 0 && nbad) atomicAdd(bad, nbad);
  __shared__ double red[kThreads / 32][kHistChunk];
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < kHistChunk; ++j) {
    double x = acc[j];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][j] = x;
  }
  __syncthreads();
  if (threadIdx.x < kHistChunk) {
    double t = 0.0;
    for (unsigned w = 0; w < kThreads / 32; ++w) t += red[w][threadIdx.x];
    partials[(uint64_t)blockIdx.x * kHistChunk + threadIdx.x] = t;
  }
}

__global__ void k_hist_finish(const double* __restrict__ partials, unsigned nblocks, int count,
                              double* __restrict__ out) {
  const int j = threadIdx.x;
  if (j >= count) return;
  double t = 0.0;
  for (unsigned b = 0; b < nblocks; ++b) t += partials[(uint64_t)b * kHistChunk + j];  // fixed order
  out[j] = t;
}

constexpr int kStats = 11;  // -sum p ln p, -sum ln p (p > 0), sum p^2 .. sum p^10

template <typename R>
__global__ void __launch_bounds__(kThreads) k_state_stats(const typename V2<R>::type* __restrict__ psi, uint64_t N,
                                                          double* __restrict__ partials) {
  double acc[kStats];
#pragma unroll
  for (int k = 0; k < kStats; ++k) acc[k] = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
    const typename V2<R>::type a = psi[i];
    const double p = (double)a.x * a.x + (double)a.y * a.y;
    if (p != 0.0) {
      const double l = log(p);
      acc[0] -= p * l;
      acc[1] -= l;
    }
    double pk = p;
#pragma unroll
    for (int k = 2; k < kStats; ++k) {
      pk *= p;
      acc[k] += pk;
    }
  }
  __shared__ double red[kThreads / 32][kStats];
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kStats; ++k) {
    double x = acc[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < kStats) {
    double t = 0.0;
    for (unsigned w = 0; w < kThreads / 32; ++w) t += red[w][threadIdx.x];
    partials[(uint64_t)blockIdx.x * kStats + threadIdx.x] = t;
  }
}

__global__ void k_stats_finish(const double* __restrict__ partials, unsigned nblocks, double* __restrict__ out) {
  const int k = threadIdx.x;
  if (k >= kStats) return;
  double t = 0.0;
  for (unsigned b = 0; b < nblocks; ++b) t += partials[(uint64_t)b * kStats + k];  // fixed order
  out[k] = t;
}

}  // namespace

template <typename R>
void launch_state_stats(iqsg_state* h, double* out_dev) {
  unsigned blocks = (unsigned)std::min<uint64_t>((h->N + kThreads - 1) / kThreads, (uint64_t)num_sms() * 2);
  if (blocks * kStats > 2u * kMaxPartials) blocks = 2u * kMaxPartials / kStats;
  k_state_stats<R><<<blocks, kThreads, 0, h->stream>>>(reinterpret_cast<const typename V2<R>::type*>(h->amps), h->N,
                                                       h->scratch);
  k_stats_finish<<<1, 32, 0, h->stream>>>(h->scratch, blocks, out_dev);
}

template <typename R>
void launch_weighted_cost(iqsg_state* h, const double* edges, unsigned num_edges) {
  const size_t shmem = (size_t)3 * num_edges * sizeof(double);
  k_weighted_cost<R><<<grid_for(h->N, 1), kThreads, shmem, h->stream>>>(
      reinterpret_cast<typename V2<R>::type*>(h->amps), h->N, edges, num_edges);
}

template <typename R>
void launch_cost_hist(iqsg_state* psi, const void* diag, int mode, double max_value, double bin_width, int nbins,
                      double* out_dev, unsigned long long* bad) {
  unsigned blocks = (unsigned)std::min<uint64_t>((psi->N + kThreads - 1) / kThreads, (uint64_t)num_sms() * 2);
  if (blocks * kHistChunk > 2u * kMaxPartials) blocks = 2u * kMaxPartials / kHistChunk;
  for (int b0 = 0; b0 < nbins; b0 += kHistChunk) {
    k_cost_hist<R><<<blocks, kThreads, 0, psi->stream>>>(
        reinterpret_cast<const typename V2<R>::type*>(psi->amps), reinterpret_cast<const typename V2<R>::type*>(diag),
        psi->N, mode, max_value, bin_width, nbins, b0, psi->scratch, bad);
    k_hist_finish<<<1, kHistChunk, 0, psi->stream>>>(psi->scratch, blocks, std::min(kHistChunk, nbins - b0),
                                                      out_dev + b0);
  }
}

template void launch_state_stats<double>(iqsg_state*, double*);
template void launch_state_stats<float>(iqsg_state*, double*);
template void launch_weighted_cost<double>(iqsg_state*, const double*, unsigned);
template void launch_weighted_cost<float>(iqsg_state*, const double*, unsigned);
template void launch_cost_hist<double>(iqsg_state*, const void*, int, double, double, int, double*, unsigned long long*);
template void launch_cost_hist<float>(iqsg_state*, const void*, int, double, double, int, double*, unsigned long long*);

}  // namespace iqsg
