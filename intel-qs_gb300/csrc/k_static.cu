// iqsg_probability_static: GetProbability for callers that cannot allocate device memory.
//
// Who needs it: code that must not call cudaMalloc/cudaFree at the moment it measures --
// an application whose registers already fill HBM (a 33-qubit ComplexDP state is 128 GiB,
// and its reorder buffer another 128 GiB), a host thread that must not take the implicit
// device-wide synchronisation cudaMalloc/cudaFree imply, or an embedding framework whose
// memory pool owns all device memory. Such a caller passes the amplitudes and a device slot
// for the result; this entry point then launches two kernels and allocates nothing.
//
// Its scratch (the per-block partial sums of the first pass) is the file-scope device array
// g_static_partials below, kStaticPartials doubles (16 KiB). Every GPU that loads libiqsg holds
// that array until the process exits. Host code cannot use the array's name as a device
// address, so the first call on each device (with that device current) looks the address up
// with cudaGetSymbolAddress and caches it; make that first call before any stream capture
// begins. Every call shares the one array per device: calls whose kernels overlap on the GPU
// (for example on two streams at once) race on it and must be ordered by the caller. No slot
// needs to start at zero: the first pass writes every partial the second pass reads.
#include <mutex>

#include "iqsg_internal.cuh"

namespace iqsg {
namespace {

constexpr int kStaticPartials = 2048;
constexpr int kStaticThreads = 256;
constexpr int kStaticFinishThreads = 1024;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_static_partials[kStaticPartials];

std::mutex g_static_mutex;
double* g_static_addr[kMaxDevices] = {};

// Device address of g_static_partials on the current device (looked up once per device).
int static_scratch(double** out) {
  int dev = 0;
  int st = cuda_status(cudaGetDevice(&dev), "iqsg_probability_static: cudaGetDevice");
  if (st) return st;
  if (dev < 0 || dev >= kMaxDevices) return fail(IQSG_EINVAL, "iqsg_probability_static: device %d not supported", dev);
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if (!g_static_addr[dev]) {
    void* p = nullptr;
    st = cuda_status(cudaGetSymbolAddress(&p, g_static_partials), "iqsg_probability_static: cudaGetSymbolAddress");
    if (st) return st;
    g_static_addr[dev] = static_cast<double*>(p);
  }
  *out = g_static_addr[dev];
  return IQSG_OK;
}

template <typename V>
__global__ void __launch_bounds__(kStaticThreads) k_prob_static(const V* __restrict__ s, uint64_t npairs, unsigned pos,
                                                                double* __restrict__ partials) {
  __shared__ double sh[kStaticThreads / 32];
  double acc = 0.0;
  const uint64_t bit = uint64_t(1) << pos;
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npairs; p += (uint64_t)gridDim.x * blockDim.x) {
    const V a = s[insert_zero(p, pos) | bit];
    acc += (double)a.x * (double)a.x + (double)a.y * (double)a.y;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < kStaticThreads / 32 ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
  }
}

__global__ void __launch_bounds__(kStaticFinishThreads) k_prob_static_finish(const double* __restrict__ partials,
                                                                             int nparts, double* __restrict__ out) {
  __shared__ double sh[kStaticFinishThreads / 32];
  double acc = 0.0;
  for (int b = threadIdx.x; b < nparts; b += blockDim.x) acc += partials[b];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = sh[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) *out = acc;
  }
}

}  // namespace
}  // namespace iqsg

using namespace iqsg;

extern "C" int iqsg_probability_static(const void* device_amps, unsigned num_qubits, int precision, unsigned pos,
                                       double* device_result, void* stream) {
  if (!device_amps || !device_result) return fail(IQSG_EINVAL, "iqsg_probability_static: null pointer");
  if ((uintptr_t)device_amps % 16 || (uintptr_t)device_result % 8)
    return fail(IQSG_EINVAL, "iqsg_probability_static: amplitudes must be 16-byte and the result 8-byte aligned");
  if (num_qubits < 1 || num_qubits > 40)
    return fail(IQSG_EINVAL, "iqsg_probability_static: num_qubits %u not in [1, 40]", num_qubits);
  if (pos >= num_qubits) return fail(IQSG_EINVAL, "iqsg_probability_static: position %u out of range", pos);
  if (precision != IQSG_COMPLEX_DP && precision != IQSG_COMPLEX_SP)
    return fail(IQSG_EINVAL, "iqsg_probability_static: unknown precision %d", precision);
  const uint64_t npairs = uint64_t(1) << (num_qubits - 1);
  const unsigned grid = grid_for(npairs, 4);
  if (grid > (unsigned)kStaticPartials)
    return fail(IQSG_EINVAL, "iqsg_probability_static: needs %u partial sums, the static scratch holds %d", grid,
                kStaticPartials);
  double* partials = nullptr;
  int st = static_scratch(&partials);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == IQSG_COMPLEX_DP)
    k_prob_static<double2><<<grid, kStaticThreads, 0, s>>>(static_cast<const double2*>(device_amps), npairs, pos, partials);
  else
    k_prob_static<float2><<<grid, kStaticThreads, 0, s>>>(static_cast<const float2*>(device_amps), npairs, pos, partials);
  k_prob_static_finish<<<1, kStaticFinishThreads, 0, s>>>(partials, (int)grid, device_result);
  return cuda_status(cudaGetLastError(), "iqsg_probability_static");
}
