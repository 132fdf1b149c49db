// Conversions between FP32 and FP64 with integer operations on the bit
// patterns.  GB300 issues FP64 at 1/64 of its FP32 rate, and the cvt
// instructions between the two formats use the FP64 pipe; these keep the
// conversions of the mixed-precision and paired-FP32 kernels off it.
#pragma once

// FP32 -> FP64, exact, with integer operations.  Zero and FP32 subnormals
// give a signed zero (slopes that small are below every tolerance here);
// infinities and NaNs map to infinities and NaNs.
__device__ __forceinline__ double f2d(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned sign = u & 0x80000000u;
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0u) return __hiloint2double((int)sign, 0);
  const unsigned ed = (e == 255u) ? 2047u : e + 896u;  // rebias 127 -> 1023
  const unsigned m = u & 0x7fffffu;
  return __hiloint2double((int)(sign | (ed << 20) | (m >> 3)), (int)(m << 29));
}

// FP64 -> FP32 rounded to nearest (ties away from zero) with integer
// operations; magnitudes below FP32's normal range give a signed zero and
// above it an infinity.
__device__ __forceinline__ float d2f_rn(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu) - 896;
  if (e <= 0) return __uint_as_float(sign);
  if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
  const unsigned mag = ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  return __uint_as_float(sign | (mag + ((lo >> 28) & 1u)));  // a carry rounds into the exponent
}
