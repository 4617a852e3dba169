// Double-float ("df64") arithmetic for ComplexDP gates on GPUs whose FP64 pipe is narrow.
//
// On GB300 the FP64 pipe issues about 0.5 T instructions/s against about 35 T/s for FP32,
// so a native FP64 2x2 gate (16 FP64 FMAs per amplitude pair) is compute-bound at roughly
// 30 % of HBM bandwidth. Here the amplitudes stay IEEE FP64 in HBM; each kernel
//   1. splits every loaded double x into floats (h, l) with x = h + l + O(2^-49 |x|)
//      using integer instructions only (h = x truncated to 24 bits, l = the remaining
//      29 bits rounded to nearest float),
//   2. forms products with the exact FMA error term and sums them with error-free
//      TwoSum steps (relative error about 2^-47 of the largest term),
//   3. rounds the double-float result back to the nearest FP64 with integer
//      instructions (bit pattern of h as a double plus the rounded ulp count of l).
// No FP64 instruction is issued on the fast path. Values outside the fast range
// (|x| < 2^-73 except exact zero, |x| >= 2^77, Inf, NaN), and results that would land
// outside it, are reported to the caller, which recomputes that group in native FP64.
//
// The functions are __host__ __device__ so the CPU test suite checks them against
// native double arithmetic; the device path uses the CUDA intrinsics of the same meaning.
#pragma once

#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD static inline
#endif

namespace df64 {

struct DF {
  float h, l;
};

DF_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}
DF_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}
DF_HD uint64_t d2u(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u;
  memcpy(&u, &d, 8);
  return u;
#endif
}
DF_HD double u2d(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double d;
  memcpy(&d, &u, 8);
  return d;
#endif
}
DF_HD float fmaf_(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}
DF_HD float mul_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);  // never contracted into an FMA
#else
  return a * b;
#endif
}
DF_HD float add_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
DF_HD float sub_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
DF_HD float u32_to_f_rn(uint32_t v) {
#if defined(__CUDA_ARCH__)
  return __uint2float_rn(v);
#else
  return (float)v;  // round to nearest under the default rounding mode
#endif
}
DF_HD int32_t f_to_i32_rn(float v) {
#if defined(__CUDA_ARCH__)
  return __float2int_rn(v);
#else
  return (int32_t)lrintf(v);
#endif
}

// Fast range in terms of the biased FP64 exponent e: [kEmin, kEmax].
constexpr uint32_t kEmin = 950;   // 2^-73: keeps the scale of l a normal float
constexpr uint32_t kEmax = 1100;  // 2^77: leaves head room for gate sums and products

// Split x into (h, l). Returns false when x is outside the fast range.
DF_HD bool split(double x, DF& r) {
  const uint64_t u = d2u(x);
  const uint32_t H = (uint32_t)(u >> 32), L = (uint32_t)u;
  const uint32_t a = H & 0x7FFFFFFFu, sign = H & 0x80000000u;
  const uint32_t e = a >> 20;
  if ((a | L) == 0u) {  // +-0
    r.h = 0.f;
    r.l = 0.f;
    return true;
  }
  // Top 32 bits of (H:L) << 3: the low 9 exponent bits and the top 23 mantissa bits.
  const uint32_t F = (H << 3) | (L >> 29);
  // Rebias 1023 -> 127: subtract 0x180 from the 9-bit field; in range the result fits 8 bits.
  const uint32_t hb = (F - 0xC0000000u) | sign;
  r.h = u2f(hb);
  // Remaining 29 mantissa bits, weight 2^(e - 1075) = 2^((ef - 52) - 127), ef = e - 896.
  const float rem = u32_to_f_rn(L & 0x1FFFFFFFu);
  r.l = mul_rn(rem, u2f((hb & 0xFF800000u) - (52u << 23)));
  return (e - kEmin) <= (kEmax - kEmin);
}

// Nearest FP64 to h + l, for |l| <= ulp_float(h)/2 (a normalised pair).
// Returns false when h is outside the fast range (the result is then unusable).
DF_HD bool merge(float h, float l, double& out) {
  const uint32_t F = f2u(h);
  const uint32_t a = F & 0x7FFFFFFFu, sign = F & 0x80000000u;
  const uint32_t ef = a >> 23;
  if (a == 0u) {
    out = 0.0;
    return l == 0.f;
  }
  // Bits of |h| as a double: exponent + 896, mantissa shifted up by 29.
  const uint64_t habs = ((uint64_t)((a >> 3) + (896u << 20)) << 32) | (uint64_t)(a << 29);
  // l in units of ulp_double(h) = 2^(ef - 179), with the sign of h folded in so the
  // count adds to |h|'s bit pattern. When |h| is a power of two and the count is negative
  // the result falls into the binade below, whose ulp is half as large.
  float q = mul_rn(l, u2f(((306u - ef) << 23) | sign));
  if ((a & 0x7FFFFFu) == 0u && q < 0.f) q = add_rn(q, q);
  const int64_t k = (int64_t)f_to_i32_rn(q);
  out = u2d((habs + (uint64_t)k) | ((uint64_t)sign << 32));
  // |h| in [2^-74, 2^101): the ulp scale above stays a normal float.
  return (ef - 53u) <= 175u;
}

// Error-free sum: s + e = a + b exactly.
DF_HD void two_sum(float a, float b, float& s, float& e) {
  s = add_rn(a, b);
  const float bb = sub_rn(s, a);
  e = add_rn(sub_rn(a, sub_rn(s, bb)), sub_rn(b, bb));
}

// Product of a constant (mh, ml) with (ah, al): ph exact high part, pl the rest.
DF_HD void prod(float mh, float ml, float ah, float al, float& ph, float& pl) {
  ph = mul_rn(mh, ah);
  const float pe = fmaf_(mh, ah, -ph);  // exact: mh*ah = ph + pe
  pl = fmaf_(ml, ah, fmaf_(mh, al, pe));
}

// Accumulator of double-float terms: hi sum kept error-free, low parts summed plainly.
struct Acc {
  float h, l;
};
DF_HD void acc_init(Acc& s, float ph, float pl) {
  s.h = ph;
  s.l = pl;
}
DF_HD void acc_add(Acc& s, float ph, float pl) {
  float e;
  two_sum(s.h, ph, s.h, e);
  s.l = add_rn(s.l, add_rn(e, pl));
}
// Normalised (h, l) with |l| <= ulp(h)/2.
DF_HD void acc_norm(const Acc& s, float& h, float& l) { two_sum(s.h, s.l, h, l); }

// Split a host double into (h, l) with h = nearest float, l = nearest float of the rest.
inline DF split_host(double x) {
  DF r;
  r.h = (float)x;
  r.l = (float)(x - (double)r.h);
  return r;
}

}  // namespace df64
