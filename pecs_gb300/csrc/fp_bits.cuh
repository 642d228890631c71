// Conversions between binary32 and binary64 done on the integer pipe.
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

}  // namespace pecs
