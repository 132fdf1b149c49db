// Device helpers shared by the mixed-precision stage kernel (rk4_mixed.cu)
// and its adjoint (adjoint.cu): the FP32 b-field coefficients and b-field,
// the p2 series and the z2 cell split.
#pragma once

#include <math.h>

#include "fp_convert.cuh"
#include "pf_internal.h"

struct BFieldF {
  int type, place, one_d, focusing, tcase;
  float bx0, by0, focx, focy, S, C, c1, ux, uy, u3, fx, fy, kx, ky, kxky, czs, cze, szt;
};

__device__ __forceinline__ void bfield_f(const BFieldF &b, float x, float y, float &bx, float &by,
                                         float &bz) {
  const float pi = (float)PF_PUFFIN_PI;
  bx = b.bx0;
  by = b.by0;
  bz = 0.f;
  if (b.type == PF_UND_CURVED) {
    const float shx = sinhf(b.kx * x), shy = sinhf(b.ky * y);
    const float chx = coshf(b.kx * x), chy = coshf(b.ky * y);
    if (b.place == 0) {
      bx = b.kxky * shx * shy * b.szt / 4.f / pi * b.S;
      by = chx * chy * b.szt / 4.f / pi * b.S;
      bz = b.czs * chx * shy * b.u3 * b.C;
    } else if (b.place == 2) {
      bx = b.kxky * shx * shy * b.u3 * b.S;
      by = chx * chy * b.u3 * b.S;
      bz = b.cze * chx * shy * b.u3 * b.C;
    } else {
      bx = b.kxky * shx * shy * b.S;
      by = chx * chy * b.S;
      bz = b.cze * chx * shy * b.C;
    }
    if (b.one_d) bz = 0.f;
  } else if (b.type == PF_UND_PLANEPOLE) {
    if (!b.one_d) {
      const float sh = sinhf(b.c1 * y);
      bz = (b.place == 1) ? sh * b.C : sh * b.u3 * b.C;
    }
  } else if (!b.one_d) {
    const bool hel = (b.type == PF_UND_HELICAL);
    if (b.place == 1) {
      bz = hel ? b.c1 * (-(x * b.S) + y * b.C) : b.c1 * (-(b.fx * x * b.S) + b.fy * y * b.C);
    } else {
      const float t = (b.tcase == 0) ? 0.f : -(b.ux * x * b.S);
      bz = t + b.uy * y * b.C;
    }
  }
  if (b.focusing) {
    bx = b.focx * y + bx;
    by = -(b.focy * x) + by;
  }
}

// p2 = (1/sqrt(1 - u) - 1) / eta from the binomial series with the 1/eta
// folded into the coefficients c[k] = C(2k+2, k+1) / 4^(k+1) / eta:
// three terms for u < 2e-6, five for u < 1e-4, seven for u < 1e-3 (the
// truncation stays below 1e-17 of the result), the closed form above
__device__ __forceinline__ double p2_series(double u, const double *c, double inv_eta, float r1,
                                            float r2) {
  if (u < 2.0e-6) {
    // u c0 (1 + (c1/c0) u + (c2/c0) u^2) with the correction (below 2e-6) in
    // FP32: its rounding is below 1e-13 of p2; two FP64 operations
    const float uf = d2f_rn(u);
    const float corr = uf * fmaf(r2, uf, r1);
    const double uc = u * c[0];
    return fma(uc, f2d(corr), uc);
  }
  if (u < 1.0e-4) {
    double s = c[4];
    s = fma(s, u, c[3]);
    s = fma(s, u, c[2]);
    s = fma(s, u, c[1]);
    s = fma(s, u, c[0]);
    return u * s;
  }
  if (u < 1.0e-3) {
    double s = c[6];
#pragma unroll
    for (int k = 5; k >= 0; --k) s = fma(s, u, c[k]);
    return u * s;
  }
  return (1.0 / sqrt(1.0 - u) - 1.0) * inv_eta;
}

// Cell index and FP32 fraction of t >= 0 taken from the bits of t (integer
// operations only); false for t < 0 or t >= 2^30, which the caller handles
// in FP64.
__device__ __forceinline__ bool cell_split(double t, int &ip, float &fr) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(t);
  const int e = (int)((b >> 52) & 0x7ffull) - 1023;
  if ((b >> 63) || e > 29) return false;
  if (e < 0) {
    ip = 0;
    fr = d2f_rn(t);
    return true;
  }
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int sh = 52 - e;
  ip = (int)(m >> sh);
  const unsigned long long fb = m & ((1ull << sh) - 1ull);  // fraction * 2^sh
  if (fb == 0ull) {
    fr = 0.f;
    return true;
  }
  const int lz = __clzll((long long)fb);
  const int ex = (63 - lz) - sh;  // fraction = 1.xxx * 2^ex, ex < 0
  const unsigned mant = (unsigned)((fb << (lz + 1)) >> 41);  // 23 bits below the leading one
  fr = __uint_as_float((unsigned)(ex + 127) << 23 | mant);
  return true;
}

// FP32 form of the stage's b-field coefficients
inline BFieldF to_float(const BFieldCoef &b) {
  BFieldF f;
  f.type = b.type;
  f.place = b.place;
  f.one_d = b.one_d;
  f.focusing = b.focusing;
  f.tcase = b.tcase;
  f.bx0 = (float)b.bx0;
  f.by0 = (float)b.by0;
  f.focx = (float)b.focx;
  f.focy = (float)b.focy;
  f.S = (float)b.S;
  f.C = (float)b.C;
  f.c1 = (float)b.c1;
  f.ux = (float)b.ux;
  f.uy = (float)b.uy;
  f.u3 = (float)b.u3;
  f.fx = (float)b.fx;
  f.fy = (float)b.fy;
  f.kx = (float)b.kx;
  f.ky = (float)b.ky;
  f.kxky = (float)b.kxky;
  f.czs = (float)b.czs;
  f.cze = (float)b.cze;
  f.szt = (float)b.szt;
  return f;
}
