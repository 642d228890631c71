// Conversions between binary32 and binary64 done on the integer pipe, and
// FP32-pair arithmetic.
//
// On GB300 every FP64 instruction, the float<->double conversions included,
// runs on the narrow FP64 unit (about 2 operations per clock per SM), so an
// element-wise pass that converts each of millions of values spends more time
// there than in memory.  Widening a normal float is exact and is only a
// rebiasing of the exponent and a shift of the mantissa (IEEE 754 binary32 and
// binary64 layouts); narrowing by truncation is the inverse with the low 29
// mantissa bits dropped.  Zeros, subnormals, infinities and NaNs take the
// regular conversion.
#pragma once
#include <cuda_runtime.h>

namespace pecs {

// exact float -> double
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  if (e == 0u || e == 0xFFu) return (double)f;
  const unsigned long long bits = ((unsigned long long)(u >> 31) << 63) |
                                  ((unsigned long long)(e + (1023u - 127u)) << 52) |
                                  ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)bits);
}

// double -> float rounded toward zero (relative error < 2^-23); for sums of
// squares, where the rounding mode does not matter
__device__ __forceinline__ float d2f_trunc(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FFull) - 1023 + 127;
  if (e <= 0 || e >= 0xFF) return (float)x;  // zero, tiny, huge, inf, nan
  const unsigned u = ((unsigned)(b >> 63) << 31) | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7FFFFFull);
  return __uint_as_float(u);
}

// ---- FP32-pair ("double-float") arithmetic --------------------------------
// A value is an unevaluated sum hi + lo of two floats with |lo| <= ulp(hi):
// about 47 significant bits, on the FP32 pipe.  The algorithms are the
// classic error-free transformations: TwoSum (Knuth), FastTwoSum (Dekker;
// |a| >= |b|) and the product error through a fused multiply-add.

// binary64 -> pair: hi = x truncated to 24 bits (integer pipe), lo = the next
// 24 bits of x (truncated), both built from x's bit fields; values whose
// exponent puts lo outside the normal float range (and zeros, infinities,
// NaNs) take the regular conversion
__device__ __forceinline__ float2 d2ff(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FFull) - 1023;
  if (e < -70 || e > 126) {
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
  }
  const float hi = d2f_trunc(x);
  const unsigned m = (unsigned)(b & 0x1FFFFFFFull);  // the 29 bits below hi's mantissa
  if (m == 0u) return make_float2(hi, 0.f);
  const int lead = 31 - __clz(m);                     // m = 1.f * 2^lead
  const unsigned mant = lead > 23 ? (m >> (lead - 23)) : (m << (23 - lead));
  const unsigned ex = (unsigned)(e - 52 + lead + 127);  // lo = m * 2^(e - 52)
  const float lo = __uint_as_float(((unsigned)(b >> 63) << 31) | (ex << 23) | (mant & 0x7FFFFFu));
  return make_float2(hi, lo);
}

// pair -> binary64 (the two exact widenings and one FP64 addition)
__device__ __forceinline__ double ff2d(float2 a) { return f2d_exact(a.x) + f2d_exact(a.y); }

__device__ __forceinline__ float2 ff_fast_two_sum(float a, float b) {
  const float s = a + b;
  return make_float2(s, b - (s - a));
}

__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
  const float s = a.x + b.x;
  const float z = s - a.x;
  const float e = (a.x - (s - z)) + (b.x - z);
  return ff_fast_two_sum(s, e + a.y + b.y);
}

__device__ __forceinline__ float2 ff_add(float2 a, float b) {
  const float s = a.x + b;
  const float z = s - a.x;
  const float e = (a.x - (s - z)) + (b - z);
  return ff_fast_two_sum(s, e + a.y);
}

__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
  const float p = a.x * b.x;
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  return ff_fast_two_sum(p, e);
}

// acc + a * b
__device__ __forceinline__ float2 ff_fma(float2 a, float2 b, float2 acc) { return ff_add(acc, ff_mul(a, b)); }

}  // namespace pecs
