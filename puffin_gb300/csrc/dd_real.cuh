// Paired-FP32 ("double-float") real numbers for the FP64 path's FFTs.
//
// GB300 issues FP64 at 1/64 of its FP32 rate, and the FP64 diffraction is
// bound by that pipe (the 43-point butterflies of the 129-point transforms).
// A value held as an unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2)
// carries 48 significand bits; sums and products are formed with FP32
// operations only, using the error-free transformations TwoSum (Knuth) and
// TwoProd through the fused multiply-add, the classical double-float
// arithmetic (Dekker 1971; the "sloppy" addition of Hida, Li and Bailey's
// double-double library, applied to floats).  Each operation is exact to
// about 2^-46 relative, so a 129-point transform keeps about 1e-13 of the
// field scale, where the reference's FFTW keeps about 1e-16: far inside the
// 1e-10 at which the reference's own tests compare runs.  The results do not
// depend on the order of anything (every butterfly's operations are fixed),
// so runs stay bit-reproducible.
//
// Conversions to and from FP64 happen once per element and pass (loads of
// the split FP64 field, stores of the result); the float halves are taken
// with integer operations on the bit patterns and one FP64 subtraction.
#pragma once

#include <stdint.h>

#include "fp_convert.cuh"

struct pf_dd {
  float hi, lo;
  pf_dd() = default;
  __host__ __device__ constexpr pf_dd(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr pf_dd(int v) : hi((float)v), lo(0.f) {}
  __host__ __device__ constexpr pf_dd(double v)
      : hi((float)v), lo((float)(v - (double)(float)v)) {}
};

__device__ __forceinline__ pf_dd dd_fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return pf_dd(s, b - (s - a));
}

__device__ __forceinline__ pf_dd operator+(pf_dd a, pf_dd b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);  // TwoSum error of the high parts
  e += a.lo + b.lo;
  return dd_fast_two_sum(s, e);
}
__device__ __forceinline__ pf_dd operator-(pf_dd a) { return pf_dd(-a.hi, -a.lo); }
__device__ __forceinline__ pf_dd operator-(pf_dd a, pf_dd b) { return a + (-b); }

__device__ __forceinline__ pf_dd operator*(pf_dd a, pf_dd b) {
  const float p = a.hi * b.hi;
  float e = __fmaf_rn(a.hi, b.hi, -p);  // TwoProd error
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return dd_fast_two_sum(p, e);
}

// a * b + c with one normalisation
__device__ __forceinline__ pf_dd fma(pf_dd a, pf_dd b, pf_dd c) {
  const float p = a.hi * b.hi;
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const float s = p + c.hi;
  const float bb = s - p;
  float t = (p - (s - bb)) + (c.hi - bb);
  t += e + c.lo;
  return dd_fast_two_sum(s, t);
}

__device__ __forceinline__ pf_dd operator/(pf_dd a, pf_dd b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const pf_dd r = a - b * pf_dd(q1, 0.f);
  const float q2 = __fdiv_rn(r.hi, b.hi);
  return dd_fast_two_sum(q1, q2);
}

// FP64 <-> pair, with integer operations for the float halves
__device__ __forceinline__ pf_dd dd_from_double(double v) {
  const float h = d2f_rn(v);
  return pf_dd(h, d2f_rn(v - f2d(h)));
}
__device__ __forceinline__ double dd_to_double(pf_dd v) { return f2d(v.hi) + f2d(v.lo); }

// Sums x0 + sum_j a_j c_j of the FFTs' odd-prime butterflies.  For pairs the
// sum is kept unnormalised: one float s takes the high parts of the products
// (TwoSum on every addition) and a second float l gathers x0's low part, the
// TwoSum errors and the TwoProd and cross-term errors of the products; one
// TwoSum at the end normalises.  12 float operations per term against 15 for
// a normalised pair multiply-add (Ogita, Rump and Oishi's cascaded summation,
// applied to the dot product); l's own roundings are 2^-24 of the errors it
// holds, about 2^-48 of the terms.  For float and double the accumulator is
// the value with a fused multiply-add.
struct pf_dd_acc {
  float s, l;
};
__device__ __forceinline__ pf_dd_acc acc_start(pf_dd x) { return pf_dd_acc{x.hi, x.lo}; }
__device__ __forceinline__ void acc_fma(pf_dd_acc &c, pf_dd a, pf_dd b) {
  const float p = a.hi * b.hi;
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const float s = c.s + p;
  const float bb = s - c.s;
  const float err = (c.s - (s - bb)) + (p - bb);
  c.s = s;
  c.l += err + e;
}
__device__ __forceinline__ pf_dd acc_end(pf_dd_acc c) {
  const float s = c.s + c.l;
  const float bb = s - c.s;
  return pf_dd(s, (c.s - (s - bb)) + (c.l - bb));
}
__device__ __forceinline__ float acc_start(float x) { return x; }
__device__ __forceinline__ void acc_fma(float &c, float a, float b) { c = __fmaf_rn(a, b, c); }
__device__ __forceinline__ float acc_end(float c) { return c; }
__device__ __forceinline__ double acc_start(double x) { return x; }
__device__ __forceinline__ void acc_fma(double &c, double a, double b) { c = __fma_rn(a, b, c); }
__device__ __forceinline__ double acc_end(double c) { return c; }
template <class T>
struct pf_acc_of {
  using type = T;
};
template <>
struct pf_acc_of<pf_dd> {
  using type = pf_dd_acc;
};
