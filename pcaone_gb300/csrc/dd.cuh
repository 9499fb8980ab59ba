// Double-float arithmetic: a value held as an unevaluated sum hi + lo of two
// FP32 numbers (|lo| <= ulp(hi)/2), about 48 significand bits.  FP64 runs at a
// small fraction of the FP32 rate on this GPU, so the small (k+p)^2 factor
// kernels compute in this form.  The operations are the error-free
// transformations of Dekker (1971) and Knuth (TAOCP vol. 2, 4.2.2), combined
// as in the double-double algorithms of Hida, Li and Bailey ("Algorithms for
// quad-double precision floating point arithmetic", ARITH-15, 2001), with
// single precision in place of double: TwoSum, QuickTwoSum, TwoProd via FMA,
// the accurate addition, the multiplication, the division by long division
// with three quotient digits, and the square root by one Newton step on the
// FP32 root.  Host and device share the code (host builds must not contract
// a*b+c, i.e. compile with -ffp-contract=off).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDA_ARCH__
#define PCAONE_DD_ADD(a, b) __fadd_rn((a), (b))
#define PCAONE_DD_SUB(a, b) __fsub_rn((a), (b))
#define PCAONE_DD_MUL(a, b) __fmul_rn((a), (b))
#else
#define PCAONE_DD_ADD(a, b) ((a) + (b))
#define PCAONE_DD_SUB(a, b) ((a) - (b))
#define PCAONE_DD_MUL(a, b) ((a) * (b))
#endif

namespace pcaone {

struct dd {
  float hi, lo;
};

// Bit casts usable on host and device.
__host__ __device__ inline uint64_t dd_bits(double v) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(v);
#else
  uint64_t b;
  std::memcpy(&b, &v, 8);
  return b;
#endif
}
__host__ __device__ inline double dd_double_of(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double v;
  std::memcpy(&v, &b, 8);
  return v;
#endif
}
__host__ __device__ inline float dd_float_of(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float v;
  std::memcpy(&v, &b, 4);
  return v;
#endif
}
__host__ __device__ inline uint32_t dd_fbits(float v) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(v);
#else
  uint32_t b;
  std::memcpy(&b, &v, 4);
  return b;
#endif
}
__host__ __device__ inline int dd_clz32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __clz((int)x);
#else
  return x ? __builtin_clz(x) : 32;
#endif
}

// hi + lo = v with integer operations only: this GPU runs FP64 arithmetic and
// the FP64 <-> FP32 conversions at a small fraction of its FP32 rate, and the
// tall products of CholeskyQR split every element they read.  hi is v with its
// 52-bit mantissa cut to the top 23 bits (exact as a float), lo the remaining
// 29 bits cut to a float's 24 (lo rounds toward zero), so |hi + lo - v| <
// 2^-46 |v| for 2^-74 <= |v| < 2^128.  Below 2^-74 lo underflows (24 bits
// remain), below 2^-126 both are zero, and 2^128 is out of range; the tall
// matrices of CholeskyQR (sketch columns, their Q factors, inverse Cholesky
// factors) lie far inside.
__host__ __device__ inline void dd_split_bits(double v, float& hi, float& lo) {
  const uint64_t b = dd_bits(v);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7FFu) - 1023;
  if (e < -126) {
    hi = lo = 0.f;
    return;
  }
  hi = dd_float_of(sign | ((uint32_t)(e + 127) << 23) | ((uint32_t)(b >> 29) & 0x7FFFFFu));
  const uint32_t m = (uint32_t)b & 0x1FFFFFFFu;  // value m * 2^(e - 52)
  const int k = 31 - dd_clz32(m);                // leading bit of m (m > 0)
  const int el = e - 52 + k;                     // exponent of lo
  if (m == 0u || el < -126) {
    lo = 0.f;
    return;
  }
  const uint32_t mant = k >= 23 ? (m >> (k - 23)) : (m << (23 - k));
  lo = dd_float_of(sign | ((uint32_t)(el + 127) << 23) | (mant & 0x7FFFFFu));
}

// (double)hi + (double)lo with the two conversions done on the bits (exact
// for normal floats; zero and subnormal floats count as zero), leaving one FP64
// addition.
__host__ __device__ inline double dd_double_of_float(float f) {
  const uint32_t b = dd_fbits(f);
  const uint32_t e = (b >> 23) & 0xFFu;
  if (e == 0u) return 0.0;
  return dd_double_of(((uint64_t)(b & 0x80000000u) << 32) | ((uint64_t)(e - 127 + 1023) << 52) |
                      ((uint64_t)(b & 0x7FFFFFu) << 29));
}
__host__ __device__ inline double dd_merge_bits(float hi, float lo) { return dd_double_of_float(hi) + dd_double_of_float(lo); }

__host__ __device__ inline dd dd_from_double(double v) {
  const float h = (float)v;
  return dd{h, (float)(v - (double)h)};
}
__host__ __device__ inline double dd_to_double(dd a) { return (double)a.hi + (double)a.lo; }

// s + e = a + b exactly
__host__ __device__ inline dd two_sum(float a, float b) {
  const float s = PCAONE_DD_ADD(a, b);
  const float bb = PCAONE_DD_SUB(s, a);
  const float e = PCAONE_DD_ADD(PCAONE_DD_SUB(a, PCAONE_DD_SUB(s, bb)), PCAONE_DD_SUB(b, bb));
  return dd{s, e};
}
// s + e = a + b exactly, given |a| >= |b| (or a == 0)
__host__ __device__ inline dd quick_two_sum(float a, float b) {
  const float s = PCAONE_DD_ADD(a, b);
  return dd{s, PCAONE_DD_SUB(b, PCAONE_DD_SUB(s, a))};
}
// p + e = a * b exactly
__host__ __device__ inline dd two_prod(float a, float b) {
  const float p = PCAONE_DD_MUL(a, b);
  return dd{p, fmaf(a, b, -p)};
}

__host__ __device__ inline dd dd_neg(dd a) { return dd{-a.hi, -a.lo}; }

__host__ __device__ inline dd dd_add(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  const dd t = two_sum(a.lo, b.lo);
  s.lo = PCAONE_DD_ADD(s.lo, t.hi);
  s = quick_two_sum(s.hi, s.lo);
  s.lo = PCAONE_DD_ADD(s.lo, t.lo);
  return quick_two_sum(s.hi, s.lo);
}
__host__ __device__ inline dd dd_sub(dd a, dd b) { return dd_add(a, dd_neg(b)); }

__host__ __device__ inline dd dd_mul(dd a, dd b) {
  dd p = two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, p.lo);
  p.lo = fmaf(a.lo, b.hi, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
__host__ __device__ inline dd dd_mul_f(dd a, float b) {
  dd p = two_prod(a.hi, b);
  p.lo = fmaf(a.lo, b, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
// c - a * b
__host__ __device__ inline dd dd_fms(dd c, dd a, dd b) { return dd_sub(c, dd_mul(a, b)); }
// c + a * b
__host__ __device__ inline dd dd_fma(dd c, dd a, dd b) { return dd_add(c, dd_mul(a, b)); }

// a / b: three quotient digits, each from the FP32 quotient of the running
// remainder's leading part
__host__ __device__ inline dd dd_div(dd a, dd b) {
  const float q1 = a.hi / b.hi;
  dd r = dd_sub(a, dd_mul_f(b, q1));
  const float q2 = r.hi / b.hi;
  r = dd_sub(r, dd_mul_f(b, q2));
  const float q3 = r.hi / b.hi;
  const dd q = quick_two_sum(q1, q2);
  return dd_add(q, dd{q3, 0.f});
}

// sqrt(a) for a > 0: s = sqrt(a.hi) in FP32, corrected by (a - s^2) / (2 s)
__host__ __device__ inline dd dd_sqrt(dd a) {
  const float s = sqrtf(a.hi);
  const dd r = dd_sub(a, two_prod(s, s));
  const float c = r.hi / PCAONE_DD_ADD(s, s);
  return quick_two_sum(s, c);
}

}  // namespace pcaone
