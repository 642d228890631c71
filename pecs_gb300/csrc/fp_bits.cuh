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

// The bit fields are handled in 32-bit halves (__double2hiint /
// __double2loint / __hiloint2double): 64-bit integer shifts and bit counts
// also occupy the narrow FP64 unit on GB300 (measured with ncu: FP64-pipe
// activity followed them), 32-bit integer operations do not.

// exact float -> double
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  if ((u << 1) == 0u) return __hiloint2double((int)u, 0);  // +-0
  if (e == 0u || e == 0xFFu) return (double)f;
  const unsigned m = u & 0x7FFFFFu;
  const unsigned hi = (u & 0x80000000u) | ((e + (1023u - 127u)) << 20) | (m >> 3);
  return __hiloint2double((int)hi, (int)(m << 29));
}

// double -> float rounded toward zero (relative error < 2^-23); for sums of
// squares, where the rounding mode does not matter
__device__ __forceinline__ float d2f_trunc(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const int e = (int)((hi >> 20) & 0x7FFu) - 1023 + 127;
  if (e <= 0 || e >= 0xFF) return (float)x;  // zero, tiny, huge, inf, nan
  return __uint_as_float((hi & 0x80000000u) | ((unsigned)e << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
}

// ---- FP32-pair ("double-float") arithmetic --------------------------------
// A value is an unevaluated sum hi + lo of two floats with |lo| <= ulp(hi):
// about 47 significant bits, on the FP32 pipe.  The algorithms are the
// classic error-free transformations: TwoSum (Knuth), FastTwoSum (Dekker;
// |a| >= |b|) and the product error through a fused multiply-add.

// binary64 -> pair: hi = x truncated to 24 bits, lo = the next 24 bits of x
// (truncated), both built from x's bit fields on the integer pipe; |x| below
// 2^-126 becomes 0 and a lo below the normal float range is dropped (absolute
// errors under 2^-126), values above 2^127 take the regular conversion
__device__ __forceinline__ float2 d2ff(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7FFu) - 1023;
  if (e < -126) return make_float2(__uint_as_float(sign), 0.f);  // zero, or below 2^-126: 0
  if (e > 126) {  // huge, infinity, NaN
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
  }
  const float fh = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
  const unsigned m = lo & 0x1FFFFFFFu;  // the 29 bits below hi's mantissa
  if (m == 0u) return make_float2(fh, 0.f);
  const int lead = 31 - __clz(m);       // m = 1.f * 2^lead
  const int ex = e - 52 + lead + 127;   // lo = m * 2^(e - 52)
  if (ex <= 0) return make_float2(fh, 0.f);  // lo below the normal range: dropped
  const unsigned mant = lead > 23 ? (m >> (lead - 23)) : (m << (23 - lead));
  return make_float2(fh, __uint_as_float(sign | ((unsigned)ex << 23) | (mant & 0x7FFFFFu)));
}

// pair -> binary64 (the two exact widenings and one FP64 addition)
__device__ __forceinline__ double ff2d(float2 a) { return f2d_exact(a.x) + f2d_exact(a.y); }

// pair -> binary64 with 32-bit integer operations only: hi's 24-bit
// significand is placed at bits 52..29 of a 53-bit integer held in two
// words, lo's significand aligned to it (bits below 2^(e_hi - 52) dropped) is
// added or subtracted with carry, and one shift renormalises (|lo| <= ulp(hi),
// so the sum moves by less than a factor of two).  Within one unit in the
// last place of the exact sum; subnormal, infinite and NaN halves take ff2d.
__device__ __forceinline__ double ff2d_i32(float2 a) {
  const unsigned uh = __float_as_uint(a.x), ul = __float_as_uint(a.y);
  const int eh = (int)((uh >> 23) & 0xFFu), el = (int)((ul >> 23) & 0xFFu);
  if ((ul << 1) == 0u) return f2d_exact(a.x);
  if (eh == 0 || eh == 0xFF || el == 0xFF) return ff2d(a);
  if (el == 0) return f2d_exact(a.x);  // subnormal lo: below hi's last place
  const int sh = 29 - (eh - el);       // lo's significand in units of 2^(eh - 179)
  if (sh < -24) return f2d_exact(a.x);
  const unsigned ml = (ul & 0x7FFFFFu) | 0x800000u;
  const unsigned L = sh >= 0 ? (ml << sh) : (ml >> -sh);
  const unsigned mh = (uh & 0x7FFFFFu) | 0x800000u;
  unsigned AH = mh >> 3, AL = mh << 29;  // mh * 2^29
  if ((uh ^ ul) >> 31) {
    AH -= (AL < L) ? 1u : 0u;
    AL -= L;
  } else {
    const unsigned t = AL + L;
    AH += (t < AL) ? 1u : 0u;
    AL = t;
  }
  int e = eh - 127;
  if (AH >= (1u << 21)) {  // carried into bit 53
    AL = (AL >> 1) | (AH << 31);
    AH >>= 1;
    ++e;
  } else if (AH < (1u << 20)) {  // borrowed below bit 52
    AH = (AH << 1) | (AL >> 31);
    AL <<= 1;
    --e;
  }
  return __hiloint2double((int)((uh & 0x80000000u) | ((unsigned)(e + 1023) << 20) | (AH & 0xFFFFFu)), (int)AL);
}

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
