// The C ABI (include/iqsg.h): argument validation, gate-class dispatch and stream handling.
// No arithmetic on amplitudes happens on the host; every path below launches a kernel.
#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "iqsg_internal.cuh"

namespace iqsg {

static thread_local std::string g_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_error = buf;
  return code;
}

int cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return IQSG_OK;
  const int code = (e == cudaErrorMemoryAllocation) ? IQSG_ENOMEM : IQSG_EDEVICE;
  return fail(code, "%s: %s", what, cudaGetErrorString(e));
}

int current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
  return dev;
}

int num_sms() {
  static int sms[kMaxDevices] = {};  // per device, filled on first use
  const int dev = current_device();
  if (!sms[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 1;
    sms[dev] = v;
  }
  return sms[dev];
}

unsigned grid_for(uint64_t work, int per_thread) {
  const uint64_t per_block = (uint64_t)kThreads * (uint64_t)per_thread;
  uint64_t g = (work + per_block - 1) / per_block;
  // Grid-stride loops: at most 8 resident 256-thread blocks per SM, in whole waves.
  const uint64_t cap = (uint64_t)num_sms() * 8;
  if (g > cap) g = cap;
  return g ? (unsigned)g : 1u;
}

}  // namespace iqsg

using namespace iqsg;

namespace {

constexpr unsigned kMaxQubits = 40;

int after_launch(const char* what) { return cuda_status(cudaGetLastError(), what); }

int check_h(const iqsg_state* h) {
  if (!h) return fail(IQSG_EINVAL, "null register handle");
  return IQSG_OK;
}

int check_pos(const iqsg_state* h, unsigned pos, const char* what) {
  if (pos >= h->n) return fail(IQSG_EINVAL, "%s: position %u out of range for %u qubits", what, pos, h->n);
  return IQSG_OK;
}

int check_pair(const iqsg_state* a, const iqsg_state* b, const char* what) {
  if (!a || !b) return fail(IQSG_EINVAL, "%s: null register handle", what);
  if (a->n != b->n || a->prec != b->prec)
    return fail(IQSG_EINVAL, "%s: registers differ in size or precision (%u/%d vs %u/%d)", what, a->n, a->prec, b->n,
                b->prec);
  return IQSG_OK;
}

size_t amp_bytes(int prec) { return prec == IQSG_COMPLEX_DP ? 16 : 8; }

template <typename R> M2<R> to_m2(const double* m) {
  M2<R> r;
  for (int k = 0; k < 4; ++k) { r.re[k] = (R)m[2 * k]; r.im[k] = (R)m[2 * k + 1]; }
  return r;
}
template <typename R> C1<R> to_c1(double re, double im) { return C1<R>{(R)re, (R)im}; }

bool is_one(double re, double im) { return re == 1.0 && im == 0.0; }

// Matrix entries the double-float kernels represent to full accuracy: zero or a normal
// magnitude in [2^-60, 2^60]. Other matrices take the native FP64 kernels.
bool emulation_safe(const double* m, int count) {
  for (int k = 0; k < count; ++k) {
    const double a = std::fabs(m[k]);
    if (a != 0.0 && !(a >= 0x1p-60 && a <= 0x1p60)) return false;
  }
  return true;
}

Positions sorted_positions(std::vector<unsigned> v) {
  Positions z{};
  std::sort(v.begin(), v.end());
  z.count = (unsigned)v.size();
  for (size_t k = 0; k < v.size(); ++k) z.p[k] = v[k];
  return z;
}

}  // namespace

namespace iqsg {

// A kernel whose bounded wait ran out leaves a nonzero word at scratch[kErrorSlot]; the
// next call that waits for the stream reports it (and clears it).
int take_device_error(iqsg_state* h, unsigned long long word, const char* what) {
  if (!word) return IQSG_OK;
  cudaMemsetAsync(h->scratch + kErrorSlot, 0, sizeof(unsigned long long), h->stream);
  return fail(IQSG_ETIMEOUT, "%s: a kernel gave up waiting for its data copies (device error word %llu)", what, word);
}

// Wait for a reduction and copy k result doubles to out (with the device error word).
int fetch_results(iqsg_state* h, int k, double* out, const char* what) {
  int st = after_launch(what);
  if (st) return st;
  st = cuda_status(cudaMemcpyAsync(h->host_result, h->scratch + kResultSlot, sizeof(double) * 9,
                                   cudaMemcpyDeviceToHost, h->stream), what);
  if (st) return st;
  st = cuda_status(cudaStreamSynchronize(h->stream), what);
  if (st) return st;
  unsigned long long word;
  std::memcpy(&word, h->host_result + (kErrorSlot - kResultSlot), sizeof word);
  if ((st = take_device_error(h, word, what))) return st;
  for (int i = 0; i < k; ++i) out[i] = h->host_result[i];
  return IQSG_OK;
}

// Wait for the stream, then check the device error word.
int sync_and_check(iqsg_state* h, const char* what) {
  int st = cuda_status(cudaMemcpyAsync(h->host_result + 8, h->scratch + kErrorSlot, sizeof(unsigned long long),
                                       cudaMemcpyDeviceToHost, h->stream), what);
  if (st) return st;
  st = cuda_status(cudaStreamSynchronize(h->stream), what);
  if (st) return st;
  unsigned long long word;
  std::memcpy(&word, h->host_result + 8, sizeof word);
  return take_device_error(h, word, what);
}

}  // namespace iqsg

namespace {

template <typename F>
int dispatch(const iqsg_state* h, F&& f) {
  if (h->prec == IQSG_COMPLEX_DP) f((double)0);
  else f((float)0);
  return IQSG_OK;
}

// ComplexDP gates other than the plain 2x2 run as one-gate sweeps: exchanges (X, CNOT,
// SWAP) and sign / +-i phases (Z, CZ, S) become exact data movement with no FP64
// instruction, and the emulated-FP64 mode covers every gate class.
int single_op(iqsg_state* h, const iqsg_op& op) { return iqsg_apply_ops(h, &op, 1, nullptr); }

iqsg_op make_op(int kind, unsigned t0, unsigned t1, const double* m, int nm) {
  iqsg_op op;
  std::memset(&op, 0, sizeof op);
  op.kind = kind;
  op.t0 = t0;
  op.t1 = t1;
  for (int k = 0; k < nm; ++k) op.m[k] = m[k];
  return op;
}

// Controlled / multi-controlled 2x2 with the diagonal shortcut: when m01 = m10 = 0 and
// m00 = 1 only the sub-block with every control and the target set changes.
int apply_controlled(iqsg_state* h, const std::vector<unsigned>& ctrl, unsigned tpos, const double* m,
                     const char* what) {
  if (h->prec == IQSG_COMPLEX_DP && ctrl.size() <= 4) {
    iqsg_op op = make_op(IQSG_OP_CTRL, tpos, 0, m, 8);
    op.nctrl = (uint32_t)ctrl.size();
    for (size_t k = 0; k < ctrl.size(); ++k) op.ctrl[k] = ctrl[k];
    return single_op(h, op);
  }
  uint64_t cmask = 0;
  std::vector<unsigned> all = ctrl;
  all.push_back(tpos);
  for (unsigned c : ctrl) cmask |= uint64_t(1) << c;
  const bool diag = m[2] == 0 && m[3] == 0 && m[4] == 0 && m[5] == 0;
  Positions z = sorted_positions(all);
  if (diag && is_one(m[0], m[1])) {
    if (is_one(m[6], m[7])) return IQSG_OK;
    const uint64_t ones = cmask | (uint64_t(1) << tpos);
    dispatch(h, [&](auto r) {
      using R = decltype(r);
      launch_phase_mask<R>(h, z, ones, to_c1<R>(m[6], m[7]));
    });
  } else {
    dispatch(h, [&](auto r) {
      using R = decltype(r);
      launch_mc1q<R>(h, z, cmask, tpos, to_m2<R>(m));
    });
  }
  return after_launch(what);
}

}  // namespace

extern "C" {

const char* iqsg_last_error(void) { return g_error.c_str(); }
int iqsg_version(void) { return 100; }

int iqsg_create(unsigned num_qubits, int precision, void* stream, iqsg_state** out) {
  if (!out) return fail(IQSG_EINVAL, "iqsg_create: null output pointer");
  *out = nullptr;
  if (num_qubits < 1 || num_qubits > kMaxQubits)
    return fail(IQSG_EINVAL, "iqsg_create: num_qubits %u not in [1, %u]", num_qubits, kMaxQubits);
  if (precision != IQSG_COMPLEX_DP && precision != IQSG_COMPLEX_SP)
    return fail(IQSG_EINVAL, "iqsg_create: unknown precision %d", precision);
  iqsg_state* h = new iqsg_state;
  h->n = num_qubits;
  h->prec = precision;
  h->N = uint64_t(1) << num_qubits;
  cudaGetDevice(&h->device);
  int st = IQSG_OK;
  if (stream) {
    h->stream = (cudaStream_t)stream;
  } else {
    st = cuda_status(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "iqsg_create: stream");
    h->owns_stream = (st == IQSG_OK);
  }
  if (!st) st = cuda_status(cudaMalloc(&h->amps, h->N * amp_bytes(precision)), "iqsg_create: state allocation");
  if (!st) h->owns = true;
  if (!st) st = cuda_status(cudaMalloc(&h->scratch, sizeof(double) * kScratchDoubles), "iqsg_create: scratch");
  if (!st) st = cuda_status(cudaMallocHost(&h->host_result, sizeof(double) * 16), "iqsg_create: pinned result");
  if (!st) st = cuda_status(cudaMemsetAsync(h->amps, 0, h->N * amp_bytes(precision), h->stream), "iqsg_create: zero");
  if (!st) st = cuda_status(cudaMemsetAsync(h->scratch, 0, sizeof(double) * kScratchDoubles, h->stream), "iqsg_create: scratch");
  if (st) {
    cudaGetLastError();
    iqsg_destroy(h);
    return st;
  }
  *out = h;
  return IQSG_OK;
}

int iqsg_create_from_device(unsigned num_qubits, int precision, void* device_amps, void* stream, iqsg_state** out) {
  if (!out) return fail(IQSG_EINVAL, "iqsg_create_from_device: null output pointer");
  *out = nullptr;
  if (!device_amps) return fail(IQSG_EINVAL, "iqsg_create_from_device: null device pointer");
  if ((uintptr_t)device_amps % 16)
    return fail(IQSG_EINVAL, "iqsg_create_from_device: device pointer must be 16-byte aligned");
  if (num_qubits < 1 || num_qubits > kMaxQubits)
    return fail(IQSG_EINVAL, "iqsg_create_from_device: num_qubits %u not in [1, %u]", num_qubits, kMaxQubits);
  if (precision != IQSG_COMPLEX_DP && precision != IQSG_COMPLEX_SP)
    return fail(IQSG_EINVAL, "iqsg_create_from_device: unknown precision %d", precision);
  iqsg_state* h = new iqsg_state;
  h->n = num_qubits;
  h->prec = precision;
  h->N = uint64_t(1) << num_qubits;
  h->amps = device_amps;
  h->owns = false;
  cudaGetDevice(&h->device);
  int st = IQSG_OK;
  if (stream) {
    h->stream = (cudaStream_t)stream;
  } else {
    st = cuda_status(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "iqsg_create_from_device: stream");
    h->owns_stream = (st == IQSG_OK);
  }
  if (!st) st = cuda_status(cudaMalloc(&h->scratch, sizeof(double) * kScratchDoubles), "iqsg_create_from_device: scratch");
  if (!st) st = cuda_status(cudaMallocHost(&h->host_result, sizeof(double) * 16), "iqsg_create_from_device: pinned");
  if (!st) st = cuda_status(cudaMemsetAsync(h->scratch, 0, sizeof(double) * kScratchDoubles, h->stream), "iqsg_create_from_device: scratch");
  if (st) {
    cudaGetLastError();
    iqsg_destroy(h);
    return st;
  }
  *out = h;
  return IQSG_OK;
}

int iqsg_clone(const iqsg_state* src, iqsg_state** out) {
  int st = check_h(src);
  if (st) return st;
  iqsg_state* h = nullptr;
  st = iqsg_create(src->n, src->prec, src->owns_stream ? nullptr : (void*)src->stream, &h);
  if (st) return st;
  h->math = src->math;
  // Order the copy after the source's queued work, then on the new register's stream.
  st = cuda_status(cudaStreamSynchronize(src->stream), "iqsg_clone: wait for source");
  if (!st)
    st = cuda_status(cudaMemcpyAsync(h->amps, src->amps, src->N * amp_bytes(src->prec), cudaMemcpyDeviceToDevice,
                                     h->stream), "iqsg_clone: copy");
  if (st) {
    iqsg_destroy(h);
    return st;
  }
  *out = h;
  return IQSG_OK;
}

int iqsg_destroy(iqsg_state* h) {
  if (!h) return IQSG_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->owns && h->amps) cudaFree(h->amps);
  if (h->tmp) cudaFree(h->tmp);
  if (h->scratch) cudaFree(h->scratch);
  if (h->host_result) cudaFreeHost(h->host_result);
  if (h->owns_stream && h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return IQSG_OK;
}

int iqsg_info(const iqsg_state* h, unsigned* num_qubits, int* precision, void** device_amps) {
  int st = check_h(h);
  if (st) return st;
  if (num_qubits) *num_qubits = h->n;
  if (precision) *precision = h->prec;
  if (device_amps) *device_amps = h->amps;
  return IQSG_OK;
}

int iqsg_set_math(iqsg_state* h, int math) {
  int st = check_h(h);
  if (st) return st;
  if (math != IQSG_MATH_NATIVE && math != IQSG_MATH_EMULATED)
    return fail(IQSG_EINVAL, "iqsg_set_math: unknown mode %d", math);
  h->math = math;
  return IQSG_OK;
}

int iqsg_synchronize(iqsg_state* h) {
  int st = check_h(h);
  if (st) return st;
  return sync_and_check(h, "iqsg_synchronize");
}

int iqsg_fill(iqsg_state* h, double re, double im) {
  int st = check_h(h);
  if (st) return st;
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    launch_fill<R>(h, to_c1<R>(re, im));
  });
  return after_launch("iqsg_fill");
}

int iqsg_init_basis(iqsg_state* h, uint64_t data_index) {
  int st = check_h(h);
  if (st) return st;
  if (data_index >= h->N) return fail(IQSG_EINVAL, "iqsg_init_basis: index %llu out of range", (unsigned long long)data_index);
  st = cuda_status(cudaMemsetAsync(h->amps, 0, h->N * amp_bytes(h->prec), h->stream), "iqsg_init_basis");
  if (st) return st;
  return iqsg_set_amplitude(h, data_index, 1.0, 0.0);
}

int iqsg_set_amplitude(iqsg_state* h, uint64_t data_index, double re, double im) {
  int st = check_h(h);
  if (st) return st;
  if (data_index >= h->N) return fail(IQSG_EINVAL, "iqsg_set_amplitude: index out of range");
  char* dst = (char*)h->amps + data_index * amp_bytes(h->prec);
  if (h->prec == IQSG_COMPLEX_DP) {
    h->host_result[0] = re;
    h->host_result[1] = im;
  } else {
    float v[2] = {(float)re, (float)im};
    std::memcpy(h->host_result, v, sizeof v);
  }
  // Pinned source + synchronize: the host slot is reused by the next call.
  st = cuda_status(cudaMemcpyAsync(dst, h->host_result, amp_bytes(h->prec), cudaMemcpyHostToDevice, h->stream),
                   "iqsg_set_amplitude");
  if (st) return st;
  return cuda_status(cudaStreamSynchronize(h->stream), "iqsg_set_amplitude");
}

int iqsg_get_amplitude(iqsg_state* h, uint64_t data_index, double* re_im) {
  int st = check_h(h);
  if (st) return st;
  if (!re_im) return fail(IQSG_EINVAL, "iqsg_get_amplitude: null output");
  if (data_index >= h->N) return fail(IQSG_EINVAL, "iqsg_get_amplitude: index out of range");
  const char* src = (const char*)h->amps + data_index * amp_bytes(h->prec);
  st = cuda_status(cudaMemcpyAsync(h->host_result, src, amp_bytes(h->prec), cudaMemcpyDeviceToHost, h->stream),
                   "iqsg_get_amplitude");
  if (st) return st;
  st = cuda_status(cudaStreamSynchronize(h->stream), "iqsg_get_amplitude");
  if (st) return st;
  if (h->prec == IQSG_COMPLEX_DP) {
    re_im[0] = h->host_result[0];
    re_im[1] = h->host_result[1];
  } else {
    float v[2];
    std::memcpy(v, h->host_result, sizeof v);
    re_im[0] = v[0];
    re_im[1] = v[1];
  }
  return IQSG_OK;
}

int iqsg_upload(iqsg_state* h, const void* host, uint64_t offset, uint64_t count) {
  int st = check_h(h);
  if (st) return st;
  if (!host && count) return fail(IQSG_EINVAL, "iqsg_upload: null host pointer");
  if (offset > h->N || count > h->N - offset) return fail(IQSG_EINVAL, "iqsg_upload: range out of bounds");
  const size_t b = amp_bytes(h->prec);
  st = cuda_status(cudaMemcpyAsync((char*)h->amps + offset * b, host, count * b, cudaMemcpyHostToDevice, h->stream),
                   "iqsg_upload");
  if (st) return st;
  return cuda_status(cudaStreamSynchronize(h->stream), "iqsg_upload");
}

int iqsg_download(iqsg_state* h, void* host, uint64_t offset, uint64_t count) {
  int st = check_h(h);
  if (st) return st;
  if (!host && count) return fail(IQSG_EINVAL, "iqsg_download: null host pointer");
  if (offset > h->N || count > h->N - offset) return fail(IQSG_EINVAL, "iqsg_download: range out of bounds");
  const size_t b = amp_bytes(h->prec);
  st = cuda_status(cudaMemcpyAsync(host, (const char*)h->amps + offset * b, count * b, cudaMemcpyDeviceToHost,
                                   h->stream), "iqsg_download");
  if (st) return st;
  return sync_and_check(h, "iqsg_download");
}

int iqsg_init_uniform_random(iqsg_state* h, uint64_t seed, uint64_t skip, double a, double b) {
  int st = check_h(h);
  if (st) return st;
  // Host generation in the register's precision with the standard library's std::mt19937 and
  // std::uniform_real_distribution, staged to HBM in chunks.
  constexpr uint64_t kChunk = uint64_t(1) << 22;  // amplitudes per copy
  std::mt19937 gen((std::mt19937::result_type)seed);
  auto fill = [&](auto r) -> int {
    using R = decltype(r);
    std::uniform_real_distribution<R> u((R)0.0, (R)1.0);
    for (uint64_t k = 0; k < skip; ++k) (void)u(gen);
    const R ra = (R)a, rb = (R)b;
    std::vector<R> buf(2 * std::min(kChunk, h->N));
    for (uint64_t off = 0; off < h->N; off += kChunk) {
      const uint64_t cnt = std::min(kChunk, h->N - off);
      for (uint64_t i = 0; i < 2 * cnt; ++i) buf[i] = ra + (rb - ra) * u(gen);
      int e = cuda_status(cudaMemcpyAsync(static_cast<char*>(h->amps) + off * 2 * sizeof(R), buf.data(),
                                          2 * cnt * sizeof(R), cudaMemcpyHostToDevice, h->stream),
                          "iqsg_init_uniform_random");
      if (!e) e = cuda_status(cudaStreamSynchronize(h->stream), "iqsg_init_uniform_random");
      if (e) return e;
    }
    return IQSG_OK;
  };
  return h->prec == IQSG_COMPLEX_DP ? fill((double)0) : fill((float)0);
}

int iqsg_upload_async(iqsg_state* h, const void* host, uint64_t offset, uint64_t count) {
  int st = check_h(h);
  if (st) return st;
  if (!host && count) return fail(IQSG_EINVAL, "iqsg_upload_async: null host pointer");
  if (offset > h->N || count > h->N - offset) return fail(IQSG_EINVAL, "iqsg_upload_async: range out of bounds");
  const size_t b = amp_bytes(h->prec);
  return cuda_status(cudaMemcpyAsync((char*)h->amps + offset * b, host, count * b, cudaMemcpyHostToDevice, h->stream),
                     "iqsg_upload_async");
}

int iqsg_download_async(iqsg_state* h, void* host, uint64_t offset, uint64_t count) {
  int st = check_h(h);
  if (st) return st;
  if (!host && count) return fail(IQSG_EINVAL, "iqsg_download_async: null host pointer");
  if (offset > h->N || count > h->N - offset) return fail(IQSG_EINVAL, "iqsg_download_async: range out of bounds");
  const size_t b = amp_bytes(h->prec);
  return cuda_status(cudaMemcpyAsync(host, (const char*)h->amps + offset * b, count * b, cudaMemcpyDeviceToHost,
                                     h->stream), "iqsg_download_async");
}

int iqsg_copy(iqsg_state* dst, const iqsg_state* src) {
  int st = check_pair(dst, src, "iqsg_copy");
  if (st) return st;
  if (dst == src) return IQSG_OK;
  if (src->stream != dst->stream) {
    st = cuda_status(cudaStreamSynchronize(src->stream), "iqsg_copy: wait for source");
    if (st) return st;
  }
  return cuda_status(cudaMemcpyAsync(dst->amps, src->amps, src->N * amp_bytes(src->prec), cudaMemcpyDeviceToDevice,
                                     dst->stream), "iqsg_copy");
}

// ---- gates ----

int iqsg_apply_1q(iqsg_state* h, unsigned pos, const double* m) {
  int st = check_h(h);
  if (st) return st;
  if (!m) return fail(IQSG_EINVAL, "iqsg_apply_1q: null matrix");
  if ((st = check_pos(h, pos, "iqsg_apply_1q"))) return st;
  const bool diag = m[2] == 0 && m[3] == 0 && m[4] == 0 && m[5] == 0;
  if (h->prec == IQSG_COMPLEX_DP && (diag || (m[0] == 0 && m[1] == 0 && m[6] == 0 && m[7] == 0)))
    return single_op(h, make_op(IQSG_OP_1Q, pos, 0, m, 8));
  if (diag) {
    const bool one0 = is_one(m[0], m[1]);
    if (one0 && is_one(m[6], m[7])) return IQSG_OK;  // identity
    if (one0) {
      Positions z = sorted_positions({pos});
      dispatch(h, [&](auto r) {
        using R = decltype(r);
        launch_phase_mask<R>(h, z, uint64_t(1) << pos, to_c1<R>(m[6], m[7]));
      });
    } else {
      dispatch(h, [&](auto r) {
        using R = decltype(r);
        launch_1q_diag<R>(h, pos, to_c1<R>(m[0], m[1]), to_c1<R>(m[6], m[7]), true);
      });
    }
    return after_launch("iqsg_apply_1q");
  }
  if (h->prec == IQSG_COMPLEX_DP && h->math == IQSG_MATH_EMULATED && emulation_safe(m, 8)) {
    launch_1q_emulated(h, pos, to_m2<double>(m));
  } else {
    dispatch(h, [&](auto r) {
      using R = decltype(r);
      launch_1q<R>(h, pos, to_m2<R>(m));
    });
  }
  return after_launch("iqsg_apply_1q");
}

int iqsg_apply_controlled_1q(iqsg_state* h, unsigned cpos, unsigned tpos, const double* m) {
  int st = check_h(h);
  if (st) return st;
  if (!m) return fail(IQSG_EINVAL, "iqsg_apply_controlled_1q: null matrix");
  if ((st = check_pos(h, cpos, "iqsg_apply_controlled_1q"))) return st;
  if ((st = check_pos(h, tpos, "iqsg_apply_controlled_1q"))) return st;
  if (cpos == tpos) return fail(IQSG_EINVAL, "iqsg_apply_controlled_1q: control and target are both %u", cpos);
  return apply_controlled(h, {cpos}, tpos, m, "iqsg_apply_controlled_1q");
}

int iqsg_apply_multi_controlled_1q(iqsg_state* h, unsigned num_ctrl, const unsigned* cpos, unsigned tpos,
                                   const double* m) {
  int st = check_h(h);
  if (st) return st;
  if (!m || (num_ctrl && !cpos)) return fail(IQSG_EINVAL, "iqsg_apply_multi_controlled_1q: null argument");
  if (num_ctrl > 8) return fail(IQSG_EINVAL, "iqsg_apply_multi_controlled_1q: at most 8 controls");
  if ((st = check_pos(h, tpos, "iqsg_apply_multi_controlled_1q"))) return st;
  uint64_t seen = uint64_t(1) << tpos;
  std::vector<unsigned> c;
  for (unsigned k = 0; k < num_ctrl; ++k) {
    if ((st = check_pos(h, cpos[k], "iqsg_apply_multi_controlled_1q"))) return st;
    if (seen & (uint64_t(1) << cpos[k])) return fail(IQSG_EINVAL, "iqsg_apply_multi_controlled_1q: repeated position %u", cpos[k]);
    seen |= uint64_t(1) << cpos[k];
    c.push_back(cpos[k]);
  }
  if (num_ctrl == 0) return iqsg_apply_1q(h, tpos, m);
  return apply_controlled(h, c, tpos, m, "iqsg_apply_multi_controlled_1q");
}

int iqsg_apply_2q(iqsg_state* h, unsigned pos_high, unsigned pos_low, const double* m) {
  int st = check_h(h);
  if (st) return st;
  if (!m) return fail(IQSG_EINVAL, "iqsg_apply_2q: null matrix");
  if ((st = check_pos(h, pos_high, "iqsg_apply_2q"))) return st;
  if ((st = check_pos(h, pos_low, "iqsg_apply_2q"))) return st;
  if (pos_high == pos_low) return fail(IQSG_EINVAL, "iqsg_apply_2q: positions coincide (%u)", pos_low);
  if (h->prec == IQSG_COMPLEX_DP) return single_op(h, make_op(IQSG_OP_2Q, pos_high, pos_low, m, 32));
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    M4<R> mm;
    for (int k = 0; k < 16; ++k) { mm.re[k] = (R)m[2 * k]; mm.im[k] = (R)m[2 * k + 1]; }
    launch_2q<R>(h, pos_high, pos_low, mm);
  });
  return after_launch("iqsg_apply_2q");
}

int iqsg_apply_swaplike(iqsg_state* h, unsigned p1, unsigned p2, const double* m) {
  int st = check_h(h);
  if (st) return st;
  if (!m) return fail(IQSG_EINVAL, "iqsg_apply_swaplike: null matrix");
  if ((st = check_pos(h, p1, "iqsg_apply_swaplike"))) return st;
  if ((st = check_pos(h, p2, "iqsg_apply_swaplike"))) return st;
  if (p1 == p2) return fail(IQSG_EINVAL, "iqsg_apply_swaplike: positions coincide (%u)", p1);
  if (h->prec == IQSG_COMPLEX_DP) return single_op(h, make_op(IQSG_OP_SWAPLIKE, p1, p2, m, 8));
  const unsigned lo = p1 < p2 ? p1 : p2, hi = p1 < p2 ? p2 : p1;
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    launch_swaplike<R>(h, lo, hi, to_m2<R>(m));
  });
  return after_launch("iqsg_apply_swaplike");
}

int iqsg_apply_diag_2q(iqsg_state* h, unsigned p1, unsigned p2, const double* d) {
  int st = check_h(h);
  if (st) return st;
  if (!d) return fail(IQSG_EINVAL, "iqsg_apply_diag_2q: null diagonal");
  if ((st = check_pos(h, p1, "iqsg_apply_diag_2q"))) return st;
  if ((st = check_pos(h, p2, "iqsg_apply_diag_2q"))) return st;
  if (p1 == p2) return fail(IQSG_EINVAL, "iqsg_apply_diag_2q: positions coincide (%u)", p1);
  if (h->prec == IQSG_COMPLEX_DP) return single_op(h, make_op(IQSG_OP_DIAG2, p1, p2, d, 8));
  if (is_one(d[0], d[1]) && is_one(d[2], d[3]) && is_one(d[4], d[5])) {
    if (is_one(d[6], d[7])) return IQSG_OK;
    Positions z = sorted_positions({p1, p2});
    const uint64_t ones = (uint64_t(1) << p1) | (uint64_t(1) << p2);
    dispatch(h, [&](auto r) {
      using R = decltype(r);
      launch_phase_mask<R>(h, z, ones, to_c1<R>(d[6], d[7]));
    });
  } else {
    dispatch(h, [&](auto r) {
      using R = decltype(r);
      C1<R> dd[4];
      for (int k = 0; k < 4; ++k) dd[k] = to_c1<R>(d[2 * k], d[2 * k + 1]);
      launch_diag2<R>(h, p1, p2, dd);
    });
  }
  return after_launch("iqsg_apply_diag_2q");
}

int iqsg_apply_cost_phase(iqsg_state* h, const iqsg_state* diag, double gamma) {
  int st = check_pair(h, diag, "iqsg_apply_cost_phase");
  if (st) return st;
  if (diag->stream != h->stream) {
    st = cuda_status(cudaStreamSynchronize(diag->stream), "iqsg_apply_cost_phase");
    if (st) return st;
  }
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    launch_cost_phase<R>(h, diag->amps, gamma);
  });
  return after_launch("iqsg_apply_cost_phase");
}

int iqsg_collapse(iqsg_state* h, unsigned pos, int value) {
  int st = check_h(h);
  if (st) return st;
  if ((st = check_pos(h, pos, "iqsg_collapse"))) return st;
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    launch_collapse<R>(h, pos, value ? 1 : 0);
  });
  return after_launch("iqsg_collapse");
}

int iqsg_scale(iqsg_state* h, double re, double im) {
  int st = check_h(h);
  if (st) return st;
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    launch_scale<R>(h, to_c1<R>(re, im));
  });
  return after_launch("iqsg_scale");
}

int iqsg_axpy(iqsg_state* h, const iqsg_state* x, double re, double im) {
  int st = check_pair(h, x, "iqsg_axpy");
  if (st) return st;
  if (x->stream != h->stream) {
    st = cuda_status(cudaStreamSynchronize(x->stream), "iqsg_axpy");
    if (st) return st;
  }
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    launch_axpy<R>(h, x->amps, to_c1<R>(re, im), is_one(re, im));
  });
  return after_launch("iqsg_axpy");
}

int iqsg_permute(iqsg_state* h, const unsigned* old_map, const unsigned* new_map) {
  int st = check_h(h);
  if (st) return st;
  if (!old_map || !new_map) return fail(IQSG_EINVAL, "iqsg_permute: null map");
  std::vector<unsigned> old_imap(h->n, ~0u), new_imap(h->n, ~0u);
  for (unsigned q = 0; q < h->n; ++q) {
    if (old_map[q] >= h->n || old_imap[old_map[q]] != ~0u) return fail(IQSG_EINVAL, "iqsg_permute: old_map is not a permutation");
    if (new_map[q] >= h->n || new_imap[new_map[q]] != ~0u) return fail(IQSG_EINVAL, "iqsg_permute: new_map is not a permutation");
    old_imap[old_map[q]] = q;
    new_imap[new_map[q]] = q;
  }
  // Destination bit p holds program qubit new_imap[p], which sat at source bit old_map[.].
  std::vector<unsigned> src_bit(h->n);
  bool same = true;
  for (unsigned p = 0; p < h->n; ++p) {
    src_bit[p] = old_map[new_imap[p]];
    same = same && src_bit[p] == p;
  }
  if (same) return IQSG_OK;
  const size_t bytes = h->N * amp_bytes(h->prec);
  if (!h->tmp || h->tmp_bytes < bytes) {
    if (h->tmp) cudaFree(h->tmp);
    h->tmp = nullptr;
    h->tmp_bytes = 0;
    st = cuda_status(cudaMalloc(&h->tmp, bytes), "iqsg_permute: reorder buffer");
    if (st) {
      cudaGetLastError();
      return st;
    }
    h->tmp_bytes = bytes;
  }
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    launch_permute<R>(h, h->amps, h->tmp, src_bit.data());
  });
  st = after_launch("iqsg_permute");
  if (st) return st;
  if (h->owns) {
    std::swap(h->amps, h->tmp);  // the register now lives in the other buffer
    return IQSG_OK;
  }
  return cuda_status(cudaMemcpyAsync(h->amps, h->tmp, bytes, cudaMemcpyDeviceToDevice, h->stream), "iqsg_permute: copy back");
}

// ---- reductions ----

int iqsg_probability(iqsg_state* h, unsigned pos, double* p) {
  int st = check_h(h);
  if (st) return st;
  if (!p) return fail(IQSG_EINVAL, "iqsg_probability: null output");
  if ((st = check_pos(h, pos, "iqsg_probability"))) return st;
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    reduce_probability<R>(h, pos);
  });
  return fetch_results(h, 1, p, "iqsg_probability");
}

int iqsg_expectation_pauli(iqsg_state* h, unsigned k, const unsigned* pos, const unsigned* obs, double* value,
                           double* norm2) {
  int st = check_h(h);
  if (st) return st;
  if (!value || (k && (!pos || !obs))) return fail(IQSG_EINVAL, "iqsg_expectation_pauli: null argument");
  uint64_t xmask = 0, zmask = 0, seen = 0;
  unsigned ny = 0;
  for (unsigned j = 0; j < k; ++j) {
    if ((st = check_pos(h, pos[j], "iqsg_expectation_pauli"))) return st;
    const uint64_t b = uint64_t(1) << pos[j];
    if (seen & b) return fail(IQSG_EINVAL, "iqsg_expectation_pauli: position %u repeated", pos[j]);
    seen |= b;
    switch (obs[j]) {
      case 1: xmask |= b; break;
      case 2: xmask |= b; zmask |= b; ++ny; break;
      case 3: zmask |= b; break;
      default: return fail(IQSG_EINVAL, "iqsg_expectation_pauli: observable %u not in {1,2,3}", obs[j]);
    }
  }
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    reduce_pauli<R>(h, xmask, zmask, ny);
  });
  double out[2];
  st = fetch_results(h, 2, out, "iqsg_expectation_pauli");
  if (st) return st;
  *value = out[0];
  if (norm2) *norm2 = out[1];
  return IQSG_OK;
}

int iqsg_norm2(iqsg_state* h, double* out) {
  int st = check_h(h);
  if (st) return st;
  if (!out) return fail(IQSG_EINVAL, "iqsg_norm2: null output");
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    reduce_norm2<R>(h);
  });
  return fetch_results(h, 1, out, "iqsg_norm2");
}

int iqsg_overlap(iqsg_state* h, const iqsg_state* psi, double* re_im) {
  int st = check_pair(h, psi, "iqsg_overlap");
  if (st) return st;
  if (!re_im) return fail(IQSG_EINVAL, "iqsg_overlap: null output");
  if (psi->stream != h->stream && (st = cuda_status(cudaStreamSynchronize(psi->stream), "iqsg_overlap"))) return st;
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    reduce_overlap<R>(h, psi->amps);
  });
  return fetch_results(h, 2, re_im, "iqsg_overlap");
}

int iqsg_max_abs_diff(iqsg_state* h, const iqsg_state* x, double re, double im, double* out) {
  int st = check_pair(h, x, "iqsg_max_abs_diff");
  if (st) return st;
  if (!out) return fail(IQSG_EINVAL, "iqsg_max_abs_diff: null output");
  if (x->stream != h->stream && (st = cuda_status(cudaStreamSynchronize(x->stream), "iqsg_max_abs_diff"))) return st;
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    reduce_max_abs_diff<R>(h, x->amps, to_c1<R>(re, im));
  });
  return fetch_results(h, 1, out, "iqsg_max_abs_diff");
}

int iqsg_l2_diff(iqsg_state* h, const iqsg_state* x, double* out) {
  int st = check_pair(h, x, "iqsg_l2_diff");
  if (st) return st;
  if (!out) return fail(IQSG_EINVAL, "iqsg_l2_diff: null output");
  if (x->stream != h->stream && (st = cuda_status(cudaStreamSynchronize(x->stream), "iqsg_l2_diff"))) return st;
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    reduce_l2_diff<R>(h, x->amps);
  });
  return fetch_results(h, 1, out, "iqsg_l2_diff");
}

int iqsg_cost_expectation(iqsg_state* psi, const iqsg_state* diag, int power, double* out) {
  int st = check_pair(psi, diag, "iqsg_cost_expectation");
  if (st) return st;
  if (!out) return fail(IQSG_EINVAL, "iqsg_cost_expectation: null output");
  if (power != 1 && power != 2) return fail(IQSG_EINVAL, "iqsg_cost_expectation: power must be 1 or 2");
  if (diag->stream != psi->stream && (st = cuda_status(cudaStreamSynchronize(diag->stream), "iqsg_cost_expectation")))
    return st;
  dispatch(psi, [&](auto r) {
    using R = decltype(r);
    reduce_cost_expectation<R>(psi, diag->amps, power);
  });
  return fetch_results(psi, 1, out, "iqsg_cost_expectation");
}

int iqsg_maxcut_cost(iqsg_state* diag, const int* adj, const unsigned* map, int* max_cut) {
  int st = check_h(diag);
  if (st) return st;
  if (!adj) return fail(IQSG_EINVAL, "iqsg_maxcut_cost: null adjacency");
  const unsigned n = diag->n;
  std::vector<unsigned> pmap(n);
  std::vector<unsigned char> seen(n, 0);
  for (unsigned q = 0; q < n; ++q) {
    pmap[q] = map ? map[q] : q;
    if (pmap[q] >= n || seen[pmap[q]]) return fail(IQSG_EINVAL, "iqsg_maxcut_cost: map is not a permutation");
    seen[pmap[q]] = 1;
  }
  std::vector<int> edges;
  for (unsigned v = 0; v < n; ++v) {
    if (adj[v * n + v] != 0) return fail(IQSG_EINVAL, "iqsg_maxcut_cost: adjacency diagonal must be zero");
    for (unsigned u = v + 1; u < n; ++u) {
      if (adj[v * n + u] != adj[u * n + v]) return fail(IQSG_EINVAL, "iqsg_maxcut_cost: adjacency must be symmetric");
      if (adj[v * n + u] != 0) {
        edges.push_back((int)pmap[v]);
        edges.push_back((int)pmap[u]);
        edges.push_back(adj[v * n + u]);
      }
    }
  }
  const unsigned ne = (unsigned)(edges.size() / 3);
  if (edges.size() > (size_t)2 * kMaxPartials * 2) return fail(IQSG_EINVAL, "iqsg_maxcut_cost: too many edges");
  if (ne) {
    st = cuda_status(cudaMemcpyAsync(diag->scratch, edges.data(), edges.size() * sizeof(int), cudaMemcpyHostToDevice,
                                     diag->stream), "iqsg_maxcut_cost: edges");
    if (st) return st;
    // The edge list must stay valid until the kernel has read it.
    st = cuda_status(cudaStreamSynchronize(diag->stream), "iqsg_maxcut_cost");
    if (st) return st;
  }
  dispatch(diag, [&](auto r) {
    using R = decltype(r);
    launch_maxcut_cost<R>(diag, reinterpret_cast<const int*>(diag->scratch), ne, pmap.data());
  });
  st = after_launch("iqsg_maxcut_cost");
  if (st) return st;
  if (!max_cut) return IQSG_OK;
  dispatch(diag, [&](auto r) {
    using R = decltype(r);
    reduce_max_real<R>(diag);
  });
  double mx = 0;
  st = fetch_results(diag, 1, &mx, "iqsg_maxcut_cost");
  if (st) return st;
  *max_cut = (int)mx;
  return IQSG_OK;
}

int iqsg_weighted_maxcut_cost(iqsg_state* diag, const double* adj, const unsigned* map, double* max_cut) {
  int st = check_h(diag);
  if (st) return st;
  if (!adj) return fail(IQSG_EINVAL, "iqsg_weighted_maxcut_cost: null adjacency");
  const unsigned n = diag->n;
  std::vector<unsigned> pmap(n);
  std::vector<unsigned char> seen(n, 0);
  for (unsigned q = 0; q < n; ++q) {
    pmap[q] = map ? map[q] : q;
    if (pmap[q] >= n || seen[pmap[q]]) return fail(IQSG_EINVAL, "iqsg_weighted_maxcut_cost: map is not a permutation");
    seen[pmap[q]] = 1;
  }
  std::vector<double> edges;
  for (unsigned v = 0; v < n; ++v) {
    if (adj[v * n + v] != 0) return fail(IQSG_EINVAL, "iqsg_weighted_maxcut_cost: adjacency diagonal must be zero");
    for (unsigned u = v + 1; u < n; ++u) {
      if (adj[v * n + u] != adj[u * n + v])
        return fail(IQSG_EINVAL, "iqsg_weighted_maxcut_cost: adjacency must be symmetric");
      if (adj[v * n + u] != 0) {
        edges.push_back((double)pmap[v]);
        edges.push_back((double)pmap[u]);
        edges.push_back(adj[v * n + u]);
      }
    }
  }
  const unsigned ne = (unsigned)(edges.size() / 3);
  if (edges.size() > (size_t)2 * kMaxPartials) return fail(IQSG_EINVAL, "iqsg_weighted_maxcut_cost: too many edges");
  if (ne) {
    st = cuda_status(cudaMemcpyAsync(diag->scratch, edges.data(), edges.size() * sizeof(double), cudaMemcpyHostToDevice,
                                     diag->stream), "iqsg_weighted_maxcut_cost: edges");
    if (st) return st;
    st = cuda_status(cudaStreamSynchronize(diag->stream), "iqsg_weighted_maxcut_cost");  // edges outlive the copy
    if (st) return st;
  }
  dispatch(diag, [&](auto r) {
    using R = decltype(r);
    launch_weighted_cost<R>(diag, diag->scratch, ne);
  });
  if ((st = after_launch("iqsg_weighted_maxcut_cost"))) return st;
  if (!max_cut) return IQSG_OK;
  dispatch(diag, [&](auto r) {
    using R = decltype(r);
    reduce_max_real<R>(diag);
  });
  return fetch_results(diag, 1, max_cut, "iqsg_weighted_maxcut_cost");
}

int iqsg_state_stats(iqsg_state* h, double* stats) {
  int st = check_h(h);
  if (st) return st;
  if (!stats) return fail(IQSG_EINVAL, "iqsg_state_stats: null output");
  double* out_dev = h->scratch + kTableSlot;
  dispatch(h, [&](auto r) {
    using R = decltype(r);
    launch_state_stats<R>(h, out_dev);
  });
  if ((st = after_launch("iqsg_state_stats"))) return st;
  double raw[11];
  if ((st = cuda_status(cudaMemcpyAsync(raw, out_dev, sizeof raw, cudaMemcpyDeviceToHost, h->stream),
                        "iqsg_state_stats")))
    return st;
  if ((st = sync_and_check(h, "iqsg_state_stats"))) return st;
  // The reference's normalisation (src/qureg_utils.cpp:418-437).
  const double two2n = (double)h->N, ln2 = std::log(2.0);
  stats[0] = raw[0] / ln2;
  stats[1] = raw[1] / ln2 / two2n;
  double factorial = 1.0;
  for (int i = 0; i < 9; ++i) {
    const int k = i + 2;
    factorial *= (double)k;
    stats[2 + i] = raw[2 + i] * (std::pow(two2n, (double)(k - 1)) / factorial);
  }
  return IQSG_OK;
}

int iqsg_cost_histogram(iqsg_state* psi, const iqsg_state* diag, int mode, double max_value, double bin_width,
                        double* hist, unsigned num_bins) {
  int st = check_pair(psi, diag, "iqsg_cost_histogram");
  if (st) return st;
  if (!hist) return fail(IQSG_EINVAL, "iqsg_cost_histogram: null output");
  if (!(max_value > 0)) return fail(IQSG_EINVAL, "iqsg_cost_histogram: max_value must be positive");
  long long want;
  if (mode == IQSG_HIST_INTEGER) {
    if (max_value != std::floor(max_value)) return fail(IQSG_EINVAL, "iqsg_cost_histogram: max_value must be an integer");
    want = (long long)max_value + 1;
  } else if (mode == IQSG_HIST_ROUNDED) {
    want = (long long)std::floor(max_value) + 1;
  } else if (mode == IQSG_HIST_BINNED) {
    if (!(bin_width > 0)) return fail(IQSG_EINVAL, "iqsg_cost_histogram: bin_width must be positive");
    want = (long long)std::ceil(max_value / bin_width) + 1;
  } else {
    return fail(IQSG_EINVAL, "iqsg_cost_histogram: unknown mode %d", mode);
  }
  if (want > (long long)kTableDoubles) return fail(IQSG_EINVAL, "iqsg_cost_histogram: more than %d bins", kTableDoubles);
  if ((long long)num_bins != want)
    return fail(IQSG_EINVAL, "iqsg_cost_histogram: num_bins %u, this histogram has %lld", num_bins, want);
  if (diag->stream != psi->stream && (st = cuda_status(cudaStreamSynchronize(diag->stream), "iqsg_cost_histogram")))
    return st;
  double* out_dev = psi->scratch + kTableSlot;
  auto* bad = reinterpret_cast<unsigned long long*>(psi->scratch + kResultSlot + 7);
  if ((st = cuda_status(cudaMemsetAsync(bad, 0, sizeof(unsigned long long), psi->stream), "iqsg_cost_histogram")))
    return st;
  dispatch(psi, [&](auto r) {
    using R = decltype(r);
    launch_cost_hist<R>(psi, diag->amps, mode, max_value, bin_width, (int)num_bins, out_dev, bad);
  });
  if ((st = after_launch("iqsg_cost_histogram"))) return st;
  std::vector<double> h(num_bins);
  unsigned long long nbad = 0;
  if ((st = cuda_status(cudaMemcpyAsync(h.data(), out_dev, sizeof(double) * num_bins, cudaMemcpyDeviceToHost,
                                        psi->stream), "iqsg_cost_histogram")))
    return st;
  if ((st = cuda_status(cudaMemcpyAsync(&nbad, bad, sizeof nbad, cudaMemcpyDeviceToHost, psi->stream),
                        "iqsg_cost_histogram")))
    return st;
  if ((st = sync_and_check(psi, "iqsg_cost_histogram"))) return st;
  if (nbad) return fail(IQSG_EINVAL, "iqsg_cost_histogram: %llu cost values outside the histogram range", nbad);
  for (unsigned b = 0; b < num_bins; ++b) hist[b] = h[b];
  return IQSG_OK;
}

}  // extern "C"
