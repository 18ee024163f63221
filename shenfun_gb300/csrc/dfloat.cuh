// Double-float ("df") arithmetic: a value is hi + lo with two FP32 numbers,
// |lo| <= ulp(hi)/2, about 48 significant bits.  It runs on the FP32 pipes,
// which on GB300 are ~65x faster than the FP64 pipe, and is the arithmetic of
// the library's mixed ("chosen") form.
//
// Algorithms: Knuth's TwoSum and Dekker/FMA TwoProd error-free
// transformations with a fast renormalisation (Dekker 1971; Hida, Li & Bailey,
// "Library for double-double and quad-double arithmetic", 2000), restated for
// FP32 pairs.  Every FP32 operation uses an explicit round-to-nearest
// intrinsic on the device so the compiler cannot contract or reassociate the
// error terms.
//
// Conversions to and from FP64 avoid the FP64/F2F pipes: the FP64 bit
// pattern is split with integer operations (hi = the top 24 significand
// bits, lo = the next 29 bits rounded to 24), and the way back assembles the
// FP64 bits of hi with integer operations and adds lo with one FP64 add.
// Inputs with |x| < 2^-120 flush to zero, |x| > FLT_MAX becomes +-inf.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#include "sgpu_common.cuh"

namespace sgpu {

#ifdef __CUDA_ARCH__
#define DF_ADD(a, b) __fadd_rn(a, b)
#define DF_SUB(a, b) __fsub_rn(a, b)
#define DF_MUL(a, b) __fmul_rn(a, b)
#define DF_FMA(a, b, c) __fmaf_rn(a, b, c)
#else
#define DF_ADD(a, b) ((float)((float)(a) + (float)(b)))
#define DF_SUB(a, b) ((float)((float)(a) - (float)(b)))
#define DF_MUL(a, b) ((float)((float)(a) * (float)(b)))
#define DF_FMA(a, b, c) fmaf(a, b, c)
#endif

SGPU_HD uint32_t f2u(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}
SGPU_HD float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}
SGPU_HD uint64_t d2u(double d) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u;
  memcpy(&u, &d, 8);
  return u;
#endif
}
SGPU_HD double u2d(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double d;
  memcpy(&d, &u, 8);
  return d;
#endif
}

struct df {
  float hi, lo;
  SGPU_HD constexpr df() : hi(0.0f), lo(0.0f) {}
  SGPU_HD constexpr df(float h, float l) : hi(h), lo(l) {}
  // compile-time constants (and rare runtime scalars): FP64 -> pair
  SGPU_HD constexpr explicit df(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
  SGPU_HD constexpr explicit df(int x) : hi((float)x), lo(0.0f) {}
};

// hi = s + e, lo = error, assuming |s| >= |e| (Dekker's Fast2Sum)
SGPU_HD df fast_two_sum(float s, float e) {
  float h = DF_ADD(s, e);
  float l = DF_SUB(e, DF_SUB(h, s));
  return df(h, l);
}

SGPU_HD df operator+(df a, df b) {
  float s = DF_ADD(a.hi, b.hi);
  float v = DF_SUB(s, a.hi);
  float e = DF_ADD(DF_SUB(a.hi, DF_SUB(s, v)), DF_SUB(b.hi, v));
  e = DF_ADD(e, DF_ADD(a.lo, b.lo));
  return fast_two_sum(s, e);
}

SGPU_HD df operator-(df a) { return df(-a.hi, -a.lo); }
SGPU_HD df operator-(df a, df b) { return a + (-b); }

SGPU_HD df operator*(df a, df b) {
  float p = DF_MUL(a.hi, b.hi);
  float e = DF_FMA(a.hi, b.hi, -p);
  e = DF_FMA(a.hi, b.lo, e);
  e = DF_FMA(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

// 2^(e - 127) as a float for a biased exponent e, gradual underflow below 1
SGPU_HD float pow2_biased(int e) {
  if (e >= 1) return u2f((uint32_t)e << 23);
  if (e >= -22) return u2f(1u << (e + 22));
  return 0.0f;
}

// FP64 -> df with integer operations only.
SGPU_HD df df_from_double(double x) {
  const uint64_t b = d2u(x);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff);
  const uint64_t m = b & 0xFFFFFFFFFFFFFull;  // 52 fraction bits
  if (e == 0x7ff) return df(u2f(sign | 0x7f800000u | (m ? 0x400000u : 0u)), 0.0f);
  const int ef = e - 1023 + 127;  // FP32 biased exponent of hi
  if (ef <= 6) return df(u2f(sign), 0.0f);   // |x| < 2^-120: flush
  if (ef >= 255) return df(u2f(sign | 0x7f800000u), 0.0f);
  const float hi = u2f(sign | ((uint32_t)ef << 23) | (uint32_t)(m >> 29));
  // remainder: 29 fraction bits, value r * 2^(e-1075); r = a*2^16 + c
  const uint32_t r = (uint32_t)(m & 0x1FFFFFFFu);
  if (r == 0) return df(hi, 0.0f);
  const uint32_t a = r >> 16, c = r & 0xFFFFu;
  // exact small-integer -> float via the 2^23 magic number
  const float fa = DF_SUB(u2f(0x4B000000u | a), 8388608.0f);
  const float fc = DF_SUB(u2f(0x4B000000u | c), 8388608.0f);
  // 2^(e-1075+16) and 2^(e-1075) as floats: biased exponents ef-23-29+16 and ef-52
  const int e1 = ef - 36, e0 = ef - 52;
  const float s1 = pow2_biased(e1);
  const float s0 = pow2_biased(e0);
  float lo = DF_FMA(fa, s1, DF_MUL(fc, s0));
  if (sign) lo = -lo;
  return df(hi, lo);
}

// df -> FP64: FP64 bits of hi assembled with integer operations, plus lo.
SGPU_HD double df_to_double(df a) {
  const uint32_t u = f2u(a.hi);
  const uint32_t sign = u & 0x80000000u;
  const uint32_t ef = (u >> 23) & 0xff;
  double dh;
  if (ef == 0) {
    dh = u2d((uint64_t)sign << 32);  // zero (FP32 denormals are not produced)
  } else if (ef == 0xff) {
    dh = u2d(((uint64_t)sign << 32) | 0x7ff0000000000000ull | ((uint64_t)(u & 0x7fffff) << 29));
  } else {
    dh = u2d(((uint64_t)sign << 32) | ((uint64_t)(ef - 127 + 1023) << 52) |
             ((uint64_t)(u & 0x7fffff) << 29));
  }
  const uint32_t v = f2u(a.lo);
  const uint32_t sl = v & 0x80000000u;
  const uint32_t el = (v >> 23) & 0xff;
  if (el == 0 || el == 0xff) return dh;
  const double dl = u2d(((uint64_t)sl << 32) | ((uint64_t)(el - 127 + 1023) << 52) |
                        ((uint64_t)(v & 0x7fffff) << 29));
  return dh + dl;
}

// ---------------------------------------------------------------------------
// Generic helpers so that templated kernels work for R = double and R = df.
template <class R>
SGPU_HD R from_f64(double x);
template <>
SGPU_HD double from_f64<double>(double x) { return x; }
template <>
SGPU_HD df from_f64<df>(double x) { return df_from_double(x); }

SGPU_HD double to_f64(double x) { return x; }
SGPU_HD double to_f64(df x) { return df_to_double(x); }

// FP64 <-> FP32 with integer operations (the F2F conversions run on the
// FP64 pipe): the FP32 value is the FP64 significand truncated to 24 bits
// (|x| < 2^-120 flushes to zero, beyond FP32 range becomes +-inf), and the
// widening is exact.  The refined solves use them around their FP32 sweeps.
SGPU_HD float f32_from_f64(double x) {
  const uint64_t b = d2u(x);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff);
  const int ef = e - 1023 + 127;
  if (e == 0x7ff || ef >= 255) return u2f(sign | 0x7f800000u);
  if (ef <= 6) return u2f(sign);
  return u2f(sign | ((uint32_t)ef << 23) | (uint32_t)((b & 0xFFFFFFFFFFFFFull) >> 29));
}
SGPU_HD double f64_from_f32(float x) {
  const uint32_t u = f2u(x);
  const uint32_t sign = u & 0x80000000u;
  const uint32_t ef = (u >> 23) & 0xff;
  if (ef == 0) return u2d((uint64_t)sign << 32);
  if (ef == 0xff) return u2d(((uint64_t)sign << 32) | 0x7ff0000000000000ull | ((uint64_t)(u & 0x7fffff) << 29));
  return u2d(((uint64_t)sign << 32) | ((uint64_t)(ef - 127 + 1023) << 52) | ((uint64_t)(u & 0x7fffff) << 29));
}
template <>
SGPU_HD float from_f64<float>(double x) { return f32_from_f64(x); }
SGPU_HD double to_f64(float x) { return f64_from_f32(x); }

// complex product specialisation for df (4 products, 2 sums)
SGPU_HD Cx<df> operator*(Cx<df> a, Cx<df> b) {
  Cx<df> z;
  z.re = a.re * b.re - a.im * b.im;
  z.im = a.re * b.im + a.im * b.re;
  return z;
}

}  // namespace sgpu
