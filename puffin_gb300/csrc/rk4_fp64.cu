// FP64 RK4 macroparticle push: one fused kernel per RK4 stage (state
// update + p2 + trilinear weights + gather + deposit + b-fields + equations)
// and one node kernel per stage over the inner-window field.
//
// Reference: rk4par (puffin/lib/interaction/puffin_mpi_RK4.f90:142-328),
// getrhs (rhs.f90:60-330), getInterps_3D / getFFelecs_3D / getSource_3D
// (system_interpolation.f90:25-248) and their 1D forms
// (system_interpolation_1D.f90:24-179), getP2 (gamma_to_p2.f90:84-85),
// the six equations (puffin_equations.f90:17-176), bfields.f90.
//
// Deposit: every contribution w_c * s is converted exactly (truncation at
// 2^-E) to a 128-bit fixed-point integer and added with two 64-bit integer
// atomics (low word, then high word plus the low word's carry).  Integer
// addition is associative, so dA/dz is bit-identical run to run whatever the
// order in which the atomics land; the reference's OpenMP atomics
// (system_interpolation.f90:174-241) are not.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>

#include <climits>

#include "pf_internal.h"

namespace {

typedef unsigned long long u64;

__device__ __forceinline__ void bfield(const BFieldCoef &b, double x, double y,
                                       double &bx, double &by, double &bz) {
  const double pi = PF_PUFFIN_PI;
  bx = b.bx0;
  by = b.by0;
  bz = 0.0;
  if (b.type == PF_UND_CURVED) {
    double shx = sinh(b.kx * x), shy = sinh(b.ky * y);
    double chx = cosh(b.kx * x), chy = cosh(b.ky * y);
    if (b.place == 0) {
      bx = b.kxky * shx * shy * b.szt / 4.0 / pi * b.S;
      by = chx * chy * b.szt / 4.0 / pi * b.S;
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
    if (b.one_d) bz = 0.0;
  } else if (b.type == PF_UND_PLANEPOLE) {
    if (!b.one_d) {
      double sh = sinh(b.c1 * y);
      bz = (b.place == 1) ? sh * b.C : sh * b.u3 * b.C;
    }
  } else if (!b.one_d) {
    const bool hel = (b.type == PF_UND_HELICAL);
    if (b.place == 1) {
      bz = hel ? b.c1 * (-(x * b.S) + y * b.C)
               : b.c1 * (-(b.fx * x * b.S) + b.fy * y * b.C);
    } else {
      double t = (b.tcase == 0) ? 0.0 : -(b.ux * x * b.S);
      bz = t + b.uy * y * b.C;
    }
  }
  if (b.focusing) {
    bx = b.focx * y + bx;
    by = -(b.focy * x) + by;
  }
}

// Integer part and fraction of t (0 <= t < 2^52, or a zero of either sign)
// from the bits of t, with integer operations only: the same values as
// floor(t) and t - floor(t) (both exact), without the FP64 pipe the stage
// kernel is bound by.  False for negative, non-finite or larger t.
__device__ __forceinline__ bool split_cell(double t, int64_t &ip, double &fr) {
  const u64 b = (u64)__double_as_longlong(t);
  if ((b << 1) == 0ull) {  // +0 or -0: floor is 0 (-0), t - floor(t) is +0
    ip = 0;
    fr = 0.0;
    return true;
  }
  if (b >> 63) return false;
  const int e = (int)((b >> 52) & 0x7ffull) - 1023;
  if (e > 51) return false;  // >= 2^52, infinity, NaN
  if (e < 0) {
    ip = 0;
    fr = t;
    return true;
  }
  const u64 m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int sh = 52 - e;  // 1 .. 52
  ip = (int64_t)(m >> sh);
  const u64 fb = m & ((1ull << sh) - 1ull);  // fraction * 2^sh
  if (fb == 0ull) {
    fr = 0.0;
    return true;
  }
  const int lz = __clzll((long long)fb);  // >= 12
  const int ex = (63 - lz) - sh;         // fraction = 1.xxx * 2^ex
  const u64 mant = (fb << (lz + 1)) >> 12;
  fr = __longlong_as_double((long long)(((u64)(ex + 1023) << 52) | mant));
  return true;
}

// A deposit factor unpacked once for mul_to_fix: significand with its hidden
// bit, biased exponent (0: zero or subnormal, 0x7ff: not finite) and sign.
struct FixOperand {
  u64 m;
  int e;
  unsigned neg;
};
__device__ __forceinline__ FixOperand fix_operand(double v) {
  const u64 b = (u64)__double_as_longlong(v);
  return FixOperand{(b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull, (int)((b >> 52) & 0x7ffull),
                    (unsigned)(b >> 63)};
}

// Exact product x * y * 2^E truncated toward zero as a two's-complement
// 128-bit integer (hi:lo), with integer operations only: the 106-bit
// product of the significands shifted onto the fixed-point grid, so the
// product is never rounded to FP64 first and no FP64 operation is spent on
// it.  Returns false when |x y 2^E| >= 2^maxexp (maxexp <= 126) or an
// operand is not finite; a zero or subnormal operand gives 0.
__device__ __forceinline__ bool mul_to_fix(const FixOperand &x, const FixOperand &y, int E,
                                           int maxexp, u64 &lo, u64 &hi) {
  lo = 0;
  hi = 0;
  if (x.e == 0x7ff || y.e == 0x7ff) return false;
  if (x.e == 0 || y.e == 0) return true;
  const u64 plo = x.m * y.m, phi = __umul64hi(x.m, y.m);  // P < 2^106
  const int sh = x.e + y.e - 2150 + E;                     // |x y| 2^E = P 2^sh
  const int top = (phi >> 41) ? 106 : 105;                 // bit length of P
  if (top + sh > maxexp) return false;
  if (sh >= 0) {  // sh <= maxexp - 105 < 64
    hi = sh ? (phi << sh) | (plo >> (64 - sh)) : phi;
    lo = plo << sh;
  } else {
    const int r = -sh;
    if (r >= 106) return true;  // below the grid
    if (r < 64) {
      lo = (plo >> r) | (phi << (64 - r));
      hi = phi >> r;
    } else {
      lo = phi >> (r - 64);
    }
  }
  if (x.neg ^ y.neg) {  // negate
    const u64 nlo = ~lo + 1ull;
    hi = ~hi + (lo == 0 ? 1ull : 0ull);
    lo = nlo;
  }
  return true;
}

__device__ __forceinline__ void fix_add(u64 *lo_arr, u64 *hi_arr, int64_t n, u64 lo, u64 hi) {
  if (lo == 0 && hi == 0) return;
  u64 old = atomicAdd(lo_arr + n, lo);
  u64 carry = (old + lo < old) ? 1ull : 0ull;
  u64 add = hi + carry;
  if (add != 0) atomicAdd(hi_arr + n, add);
}

// The 128-bit fixed-point sum (hi:lo) times 2^-E as the nearest double (ties
// to even), with integer operations only: the leading 53 bits of the
// magnitude, rounded on the bits below them, with the scale 2^-E folded into
// the exponent.  Results outside the normal range (not reached by the scales
// the beam sets) take the FP64 route.
__device__ __forceinline__ double fix_to_double(u64 lo, u64 hi, int E) {
  const bool neg = (long long)hi < 0;
  if (neg) {
    u64 nlo = ~lo + 1ull;
    hi = ~hi + (lo == 0 ? 1ull : 0ull);
    lo = nlo;
  }
  if ((hi | lo) == 0ull) return 0.0;
  const int lz = hi ? __clzll((long long)hi) : 64 + __clzll((long long)lo);
  u64 nh, nl;  // the magnitude shifted so that its leading one is bit 127
  if (lz >= 64) {
    nh = lo << (lz - 64);
    nl = 0ull;
  } else if (lz > 0) {
    nh = (hi << lz) | (lo >> (64 - lz));
    nl = lo << lz;
  } else {
    nh = hi;
    nl = lo;
  }
  int msb = 127 - lz;
  u64 m = nh >> 11;  // 53 bits, the leading one at bit 52
  const bool rb = (nh >> 10) & 1ull, sticky = ((nh & 0x3FFull) | nl) != 0ull;
  if (rb && (sticky || (m & 1ull))) ++m;
  if (m >> 53) {  // the rounding carried into a new leading bit
    m >>= 1;
    ++msb;
  }
  const int be = msb - E + 1023;
  double v;
  if (be > 0 && be < 2047) {
    v = __longlong_as_double((long long)(((u64)be << 52) | (m & 0xFFFFFFFFFFFFFull)));
  } else {
    v = (__ull2double_rn(hi) * 18446744073709551616.0 + __ull2double_rn(lo)) * ldexp(1.0, -E);
  }
  return neg ? -v : v;
}

// Shared-memory deposit tile of the dense mode: the 128-bit fixed-point sums
// (lo and hi words, re and im) of FT_PLANES window planes starting at pzlo.
// Integer addition is associative, so the tile and its flush to HBM give the
// same bits as the direct atomics, whatever the order.
constexpr int FT_PLANES = 3;
constexpr int FT_PPB = PF_FT_PPB;  // macroparticles per block in the dense mode
constexpr int FT_THREADS = 256;

struct FixTile {
  u64 *lo_r, *hi_r, *lo_i, *hi_i;
  int pzlo, ntr;
};

// tc: this step's coefficients of a replayed step block (read once per
// thread or staged once per block by the caller), null outside graphs
template <int STAGE, bool ONED, bool TILE>
__device__ __forceinline__ void stage_particle(const StageArgs &a, const int64_t i,
                                               const FixTile &t, const StageCoef *tc) {
  const double y0[6] = {a.x[i], a.y[i], a.z2[i], a.px[i], a.py[i], a.gam[i]};
  double s[6];
  double kin[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    if (STAGE > 1) {
      kin[j] = a.kin[j][i];
      s[j] = y0[j] + a.cstate * kin[j];
    } else {
      kin[j] = 0.0;
      s[j] = y0[j];
    }
  }
  const double X = s[0], Y = s[1], Z2 = s[2], PX = s[3], PY = s[4], G = s[5];
  const double chi = a.chi[i];
  // a NaN or infinity in the stage state stops the step (PF_NOT_FINITE)
  if (!(pf_finite(X) && pf_finite(Y) && pf_finite(Z2) && pf_finite(PX) && pf_finite(PY) &&
        pf_finite(G)))
    atomicOr(a.status, ST_NOT_FINITE);

  // getP2 (gamma_to_p2.f90:84-85).  1 - u loses ~7 digits, so u and the
  // square root and reciprocal that follow keep IEEE division/sqrt and the
  // reference's operation order; after the cancellation (r - 1) a reciprocal
  // multiply is exact to an ulp.
  const double aa = 1.0 / (a.gamma_r * (G * G));   // a.gamma_r holds gamma0**2
  const double bb = 1.0 + a.aw * ((PX * PX) + (PY * PY));  // a.aw holds aw**2
  const double p2 = ((1.0 / sqrt(1.0 - aa * bb)) - 1.0) * a.inv_eta;
  const double q = 1.0 + a.eta * p2;
  // 1/Gamma from aa = 1/(gamma0^2 Gamma^2): two products instead of a
  // division, within 3 ulp (1/Gamma only scales well-conditioned terms)
  const double rG = G * (a.gamma_r * aa);
  const double qrG = q * rG;

  // interpolation (getInterps_3D / getInterps_1D): cell index and fraction
  // from one scaled coordinate t = position / cell size
  double w[8];
  int64_t node[8];
  bool ok = true;
  int64_t pz0 = 0, pz1 = 0;
  {
    // the cell index and fraction from the bits (integer operations, the
    // same values as floor and subtraction); FP64 floor where the bits
    // cannot give them (negative or very large z2)
    const double tz = Z2 * a.inv_dz2;
    int64_t izc;
    double zw2;
    if (split_cell(tz, izc, zw2)) {
      if (a.periodic) {
        int64_t m = izc;  // z2n - 1
        if ((uint64_t)m >= (uint64_t)a.npl) m %= a.npl;
        pz0 = m;
        pz1 = (m + 1 == a.npl) ? 0 : m + 1;
      } else if (!(izc + 1 < a.nz2)) {
        ok = false;
        atomicOr(a.status, ST_OUT_OF_Z2);
      } else {
        pz0 = izc;
        pz1 = pz0 + 1;
      }
    } else {
      const double fz = floor(tz);
      const double z2n = fz + 1.0;
      zw2 = tz - fz;
      if (a.periodic) {
        if (!(fabs(z2n) < 9.0e15)) {
          ok = false;
          atomicOr(a.status, ST_OUT_OF_Z2);
        } else {
          int64_t m = ((int64_t)z2n - 1) % a.npl;
          if (m < 0) m += a.npl;
          pz0 = m;
          pz1 = (m + 1 == a.npl) ? 0 : m + 1;
        }
      } else {
        if (!(z2n >= 1.0 && z2n < (double)a.nz2)) {
          ok = false;
          atomicOr(a.status, ST_OUT_OF_Z2);
        } else {
          pz0 = (int64_t)z2n - 1;
          pz1 = pz0 + 1;
        }
      }
    }
    if (ONED) {
      const double w1 = 1.0 - zw2;
      w[0] = w1;
      w[1] = 1.0 - w1;
      node[0] = pz0;
      node[1] = pz1;
    } else {
      // a coordinate whose bits give no cell (negative, non-finite, huge)
      // is outside the window, as floor + 1 < 1 or >= nix would say
      const double tx = (X + a.halfx) * a.inv_dx;
      const double ty = (Y + a.halfy) * a.inv_dy;
      int64_t ixc = -1, iyc = -1;
      double x2 = 0.0, y2 = 0.0;
      const bool okx = split_cell(tx, ixc, x2) && ixc + 1 < a.nix;
      const bool oky = split_cell(ty, iyc, y2) && iyc + 1 < a.niy;
      const double x1 = 1.0 - x2, y1 = 1.0 - y2;
      const double zw1 = 1.0 - zw2;
      if (!(okx && oky)) {
        ok = false;
        atomicOr(a.status, ST_OUT_OF_WINDOW);
      }
      const int64_t ntr = a.nix * a.niy;
      const int64_t ix = ok ? ixc : 0, iy = ok ? iyc : 0;
      const int64_t b0 = ix + iy * a.nix + pz0 * ntr, b1 = ix + iy * a.nix + pz1 * ntr;
      const double x1y1 = x1 * y1, x2y1 = x2 * y1, x1y2 = x1 * y2, x2y2 = x2 * y2;
      w[0] = x1y1 * zw1;
      w[1] = x2y1 * zw1;
      w[2] = x1y2 * zw1;
      w[3] = x2y2 * zw1;
      w[4] = x1y1 * zw2;
      w[5] = x2y1 * zw2;
      w[6] = x1y2 * zw2;
      w[7] = x2y2 * zw2;
      node[0] = b0;
      node[1] = b0 + 1;
      node[2] = b0 + a.nix;
      node[3] = b0 + a.nix + 1;
      node[4] = b1;
      node[5] = b1 + 1;
      node[6] = b1 + a.nix;
      node[7] = b1 + a.nix + 1;
    }
  }
  constexpr int NC = ONED ? 2 : 8;

  // gather (getFFelecs)
  double fr = 0.0, fi = 0.0;
  if (ok) {
    fr = w[0] * __ldg(a.ar + node[0]);
    fi = w[0] * __ldg(a.ai + node[0]);
#pragma unroll
    for (int c = 1; c < NC; ++c) {
      fr = w[c] * __ldg(a.ar + node[c]) + fr;
      fi = w[c] * __ldg(a.ai + node[c]) + fi;
    }
    if (!(pf_finite(fr) && pf_finite(fi))) atomicOr(a.status, ST_NOT_FINITE);
    // deposit (getSource)
    if (a.field_evolve) {
      // (chi/dV3) (1 + eta p2) p / Gamma
      const double dw = chi * a.inv_dV3 * qrG;
      const FixOperand osr = fix_operand(dw * PX), osi = fix_operand(dw * PY);
      bool fits = true;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        int ti = -1;  // tile slot of the node, -1: outside the tile
        if constexpr (TILE) {
          const int64_t plane = (ONED ? c == 0 : c < 4) ? pz0 : pz1;
          const int tp = (int)plane - t.pzlo;
          if (tp >= 0 && tp < FT_PLANES) ti = tp * t.ntr + (int)(node[c] - plane * t.ntr);
        }
        u64 lo, hi;
        const FixOperand ow = fix_operand(w[c]);
        fits &= mul_to_fix(ow, osr, a.fix_e, a.fix_maxexp, lo, hi);
        if (TILE && ti >= 0) fix_add(t.lo_r, t.hi_r, ti, lo, hi);
        else fix_add(a.acc_lo_r, a.acc_hi_r, node[c], lo, hi);
        fits &= mul_to_fix(ow, osi, a.fix_e, a.fix_maxexp, lo, hi);
        if (TILE && ti >= 0) fix_add(t.lo_i, t.hi_i, ti, lo, hi);
        else fix_add(a.acc_lo_i, a.acc_hi_i, node[c], lo, hi);
      }
      if (!fits) atomicOr(a.status, ST_OVERFLOW);
    }
  }
  if (!a.coupling) {
    fr = 0.0;
    fi = 0.0;
  }

  double k[6];
  if (a.electrons_evolve) {
    double bx, by, bz;
    bfield(tc ? tc->bf : a.bf, X, Y, bx, by, bz);
    const double n2col = tc ? tc->n2col : a.n2col, kn2col = tc ? tc->kn2col : a.kn2col;
    const double ep = p2 * a.eta_k2;           // eta p2 / kappa^2
    const double cz = kn2col * qrG * bz;       // kappa (1 + eta p2) / Gamma alpha bz
    k[2] = p2;
    k[0] = a.dxc * qrG * PX;
    k[1] = -(a.dxc * qrG * PY);
    k[3] = a.sInv2rho * (n2col * by - ep * fr) + cz * PY;
    k[4] = a.sInv2rho * (n2col * bx - ep * fi) - cz * PX;
    k[5] = -(a.rho2 * qrG * (PX * fr + PY * fi));
  } else {
#pragma unroll
    for (int j = 0; j < 6; ++j) k[j] = 0.0;
  }

#pragma unroll
  for (int j = 0; j < 6; ++j) {
    if (STAGE == 1) {
      a.kout[j][i] = k[j];
    } else if (STAGE == 2) {
      a.kacc[j][i] = k[j];
    } else if (STAGE == 3) {
      // k2 and (stage 4) the state are read again here rather than held
      // live through the body: the same values, fewer registers
      a.kout[j][i] = k[j];
      a.kacc[j][i] = a.kin[j][i] + k[j];
    } else {
      const double k1 = a.k1[j][i];
      const double k23 = a.kacc[j][i];
      const double yj = (j == 0) ? a.x[i] : (j == 1) ? a.y[i] : (j == 2) ? a.z2[i]
                      : (j == 3) ? a.px[i] : (j == 4) ? a.py[i] : a.gam[i];
      a.ynext[j][i] = yj + a.h6 * (k1 + k[j] + 2.0 * k23);
    }
  }
}

// Dense mode of one block: macroparticles i0..i1-1 deposit into a shared
// tile of FT_PLANES planes from the lowest plane they start from (z2 only
// moves forward within a step, p2 > 0); the tile is then added to the window
// accumulators, one pair of atomics per node.  Every thread of the block
// calls it (it holds block barriers).
template <int STAGE, bool ONED>
__device__ __forceinline__ void stage_tile_block(const StageArgs &a, const int64_t i0,
                                                 const int64_t i1, u64 *ftile, int &s_pzlo) {
  const int ntr = (int)(a.nix * a.niy);
  const int tn = FT_PLANES * ntr;
  __shared__ StageCoef s_coef;  // a replayed block's coefficients, staged once
  for (int k = threadIdx.x; k < 4 * tn; k += blockDim.x) ftile[k] = 0ull;
  if (threadIdx.x == 0) {
    s_pzlo = INT_MAX;
    if (a.coef_tab) s_coef = a.coef_tab[(*a.step_ctr) * 4 + (STAGE - 1)];
  }
  __syncthreads();
  const StageCoef *tc = a.coef_tab ? &s_coef : nullptr;
  const bool halted = (*((volatile unsigned int *)a.status) != 0u);
  int my = INT_MAX;
  if (!halted) {
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      const double fz = floor(a.z2[i] * a.inv_dz2);
      if (!(fabs(fz) < 2.0e9)) continue;
      int m = (int)fz;
      if (a.periodic) {
        m %= (int)a.npl;
        if (m < 0) m += (int)a.npl;
      }
      my = min(my, m);
    }
  }
  for (int o = 16; o > 0; o >>= 1) my = min(my, __shfl_xor_sync(0xffffffffu, my, o));
  if ((threadIdx.x & 31) == 0 && my != INT_MAX) atomicMin(&s_pzlo, my);
  __syncthreads();
  const FixTile t{ftile, ftile + tn, ftile + 2 * tn, ftile + 3 * tn, s_pzlo, ntr};
  if (!halted)
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x)
      stage_particle<STAGE, ONED, true>(a, i, t, tc);
  __syncthreads();
  if (t.pzlo == INT_MAX) return;
  for (int k = threadIdx.x; k < tn; k += blockDim.x) {
    const int64_t plane = (int64_t)t.pzlo + k / ntr;
    if (plane >= a.npl) break;
    const int64_t node = plane * ntr + (k % ntr);
    fix_add(a.acc_lo_r, a.acc_hi_r, node, t.lo_r[k], t.hi_r[k]);
    fix_add(a.acc_lo_i, a.acc_hi_i, node, t.lo_i[k], t.hi_i[k]);
  }
}

template <int STAGE, bool ONED, bool TILE = false>
__global__ void __launch_bounds__(256, TILE ? 3 : 4) k_stage(const StageArgs a) {
  if constexpr (!TILE) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.np) return;
    if (*((volatile unsigned int *)a.status) != 0u) return;
    const StageCoef *tc = a.coef_tab ? a.coef_tab + (*a.step_ctr) * 4 + (STAGE - 1) : nullptr;
    stage_particle<STAGE, ONED, false>(a, i, FixTile{}, tc);
  } else {
    extern __shared__ u64 ftile[];
    __shared__ int s_pzlo;
    const int64_t i0 = (int64_t)blockIdx.x * a.tile_ppb;
    stage_tile_block<STAGE, ONED>(a, i0, min(a.np, i0 + (int64_t)a.tile_ppb), ftile, s_pzlo);
  }
}

// Batched stage: the tiles (instance, macroparticle range) of many
// independent instances in one launch; a block walks the tiles
// blockIdx.x, blockIdx.x + gridDim.x, ... and stages the arguments of each
// tile's instance in shared memory.  TILE: the dense-mode deposit.
template <int STAGE, bool TILE>
__global__ void __launch_bounds__(256, 4) k_stage_batch(const StageArgs *__restrict__ args,
                                                     const BatchTile *__restrict__ tiles,
                                                     const int ntiles) {
  __shared__ __align__(16) u64 sa_raw[sizeof(StageArgs) / 8];
  __shared__ int s_pzlo;
  extern __shared__ u64 ftile[];
  static_assert(sizeof(StageArgs) % 8 == 0, "StageArgs is copied as 64-bit words");
  const StageArgs &sa = *reinterpret_cast<const StageArgs *>(sa_raw);
  __shared__ StageCoef s_coef;  // the tile's instance's coefficients (replayed blocks)
  int cur = -1;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BatchTile tl = tiles[t];
    if (tl.inst != cur) {
      __syncthreads();  // the previous tile is done with the arguments
      const u64 *src = reinterpret_cast<const u64 *>(args + tl.inst);
      for (int k = threadIdx.x; k < (int)(sizeof(StageArgs) / 8); k += blockDim.x) sa_raw[k] = src[k];
      if (threadIdx.x == 0) {
        const StageArgs &g = args[tl.inst];
        if (g.coef_tab) s_coef = g.coef_tab[(*g.step_ctr) * 4 + (STAGE - 1)];
      }
      cur = tl.inst;
      __syncthreads();
    }
    if constexpr (TILE) {
      stage_tile_block<STAGE, false>(sa, tl.begin, tl.end, ftile, s_pzlo);
      __syncthreads();  // the tile is reused by the next range
    } else {
      if (*((volatile unsigned int *)sa.status) != 0u) continue;
      const StageCoef *tc = sa.coef_tab ? &s_coef : nullptr;
      for (int64_t i = tl.begin + threadIdx.x; i < tl.end; i += blockDim.x)
        stage_particle<STAGE, false, false>(sa, i, FixTile{}, tc);
    }
  }
}

// Every input of the node is loaded before the first store (the arrays
// could alias as far as the compiler knows), so a thread waits for HBM once.
template <int STAGE>
__device__ __forceinline__ void node_update(const NodeArgs &a, const int64_t n) {
  const u64 lr = a.acc_lo_r[n], hr = a.acc_hi_r[n], li = a.acc_lo_i[n], hi = a.acc_hi_i[n];
  const double wr = a.wr[n], wi = a.wi[n];
  double e0r = 0.0, e0i = 0.0, e12r = 0.0, e12i = 0.0;
  if (STAGE == 3 || STAGE == 4) {
    e12r = a.d12r[n];
    e12i = a.d12i[n];
  }
  if (STAGE == 4) {
    e0r = a.d0r[n];
    e0i = a.d0i[n];
  }
  const unsigned st = (STAGE == 4) ? *a.status : 0u;
  // a non-finite field value stops the step before stage 4 commits
  if (STAGE == 1 && !(pf_finite(wr) && pf_finite(wi)))
    atomicOr(const_cast<unsigned int *>(a.status), ST_NOT_FINITE);
  const double dr = fix_to_double(lr, hr, a.fix_e);
  const double di = fix_to_double(li, hi, a.fix_e);
  // the four accumulator words of a node are cleared right after their
  // conversion (measured faster here than clearing them after the other
  // stores)
  a.acc_lo_r[n] = 0ull;
  a.acc_hi_r[n] = 0ull;
  a.acc_lo_i[n] = 0ull;
  a.acc_hi_i[n] = 0ull;
  if (STAGE == 1) {
    a.d0r[n] = dr;
    a.d0i[n] = di;
    a.asr[n] = wr + a.coef * dr;
    a.asi[n] = wi + a.coef * di;
  } else if (STAGE == 2) {
    a.d12r[n] = dr;
    a.d12i[n] = di;
    a.asr[n] = wr + a.coef * dr;
    a.asi[n] = wi + a.coef * di;
  } else if (STAGE == 3) {
    a.asr[n] = wr + a.coef * dr;
    a.asi[n] = wi + a.coef * di;
    a.d12r[n] = e12r + dr;
    a.d12i[n] = e12i + di;
  } else {
    if (st == 0u) {
      a.wr[n] = wr + a.h6 * (e0r + dr + 2.0 * e12r);
      a.wi[n] = wi + a.h6 * (e0i + di + 2.0 * e12i);
    }
  }
}

template <int STAGE>
__global__ void __launch_bounds__(256) k_nodes(const NodeArgs a) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.n) return;
  node_update<STAGE>(a, n);
  if (STAGE == 4 && a.step_ctr && n == 0) *a.step_ctr += 1;
}

// Batched node update over (instance, node range) tiles; the last stage
// advances the batch's step counter once.
template <int STAGE>
__global__ void __launch_bounds__(256) k_nodes_batch(const NodeArgs *__restrict__ args,
                                                     const BatchTile *__restrict__ tiles,
                                                     const int ntiles, int *step_ctr) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BatchTile tl = tiles[t];
    const NodeArgs a = args[tl.inst];
    for (int64_t n = tl.begin + threadIdx.x; n < tl.end; n += blockDim.x)
      node_update<STAGE>(a, n);
  }
  if (STAGE == 4 && step_ctr && blockIdx.x == 0 && threadIdx.x == 0) *step_ctr += 1;
}

// Batched periodic z2 wrap after a step of a block: instance i wraps when
// its cumulative step count (csteps0 + steps done in the block) is a
// multiple of its cadence; the current buffer after k steps is cur0 ^ (k & 1).
__global__ void __launch_bounds__(256) k_wrap_batch(const WrapArgs *__restrict__ args,
                                                    const BatchTile *__restrict__ tiles,
                                                    const int ntiles, const int *step_ctr) {
  const int k = *step_ctr;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BatchTile tl = tiles[t];
    const WrapArgs a = args[tl.inst];
    if (!a.periodic || (a.csteps0 + k) % a.redist != 0) continue;
    double *z2 = ((a.cur0 ^ (k & 1)) != 0) ? a.z2[1] : a.z2[0];
    for (int64_t i = tl.begin + threadIdx.x; i < tl.end; i += blockDim.x)
      z2[i] = z2[i] - (floor(z2[i] / a.lenz2) * a.lenz2);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

// getAlpha (wiggler_taper.f90:39-47) + adjUndPlace (puffin_equations.f90:218-254)
// alpha(z) of a piecewise-linear profile, constant beyond its end points
double pf_taper_profile_at(const std::vector<double> &z, const std::vector<double> &a, double sz) {
  const size_t n = z.size();
  if (sz <= z[0]) return a[0];
  if (sz >= z[n - 1]) return a[n - 1];
  const size_t k = (size_t)(std::upper_bound(z.begin(), z.end(), sz) - z.begin()) - 1;
  const double t = (sz - z[k]) / (z[k + 1] - z[k]);
  return a[k] + t * (a[k + 1] - a[k]);
}

void pf_taper_stage(pf_handle *h, double sz, double *n2col, int *place) {
  const pf_params &p = h->p;
  if (!h->prof_z.empty()) {
    h->n2col = pf_taper_profile_at(h->prof_z, h->prof_a, sz);
  } else if ((sz >= p.szfs) && (sz <= p.szfe)) {
    h->n2col = h->n2col0 + h->undgrad * (sz - p.szfs);
  } else if (sz > p.szfe) {
    h->n2col0 = h->n2col;
  }
  *n2col = h->n2col;
  if (p.und_ends) {
    if (sz <= p.szfs) *place = 0;
    else if (sz >= p.szfe) *place = 2;
    else *place = 1;
  } else {
    *place = 1;
  }
}

// Stage-uniform parts of bfields.f90, evaluated left to right.
void pf_stage_coefficients(const pf_params &p, double sz, double n2col, int place,
                           BFieldCoef *b) {
  (void)n2col;
  const double pi = PF_PUFFIN_PI, rho = p.rho;
  const double seta = sqrt(p.eta);
  *b = BFieldCoef();
  b->type = p.und_type;
  b->place = place;
  b->one_d = p.one_d;
  b->focusing = p.focusing;
  b->focx = seta * (p.kbysf * p.kbysf) / p.kappa;
  b->focy = seta * (p.kbxsf * p.kbxsf) / p.kappa;
  b->c1 = seta / 2.0 / rho;
  b->fx = p.fx;
  b->fy = p.fy;
  double szt = sz / 2.0 / rho;
  if (p.und_type == PF_UND_CURVED) {
    b->kx = p.kx_und;
    b->ky = p.ky_und;
    b->kxky = p.kx_und / p.ky_und;
    b->czs = seta / 2.0 / rho / p.ky_und;
    b->cze = seta / 2.0 / rho / p.kx_und;
    if (place == 0) {
      b->szt = szt;
      b->S = sin(szt);
      b->C = cos(szt);
      b->u3 = (szt / 4.0 / pi);
    } else if (place == 2) {
      double s = (sz - p.szfe) / 2.0 / rho;
      b->S = sin(s);
      b->C = cos(s);
      b->u3 = (-s / 4.0 / pi + 1.0);
    } else {
      b->S = sin(szt);
      b->C = cos(szt);
    }
  } else if (p.und_type == PF_UND_PLANEPOLE) {
    b->bx0 = 0.0;
    if (place == 0) {
      b->by0 = szt / 4.0 / pi * sin(szt);
      b->u3 = (szt / 4.0 / pi);
      b->C = cos(szt);
    } else if (place == 2) {
      double s = (sz - p.szfe) / 2.0 / rho;
      b->by0 = (-s / 4.0 / pi + 1.0) * sin(s);
      b->u3 = (-s / 4.0 / pi + 1.0);
      b->C = cos(s);
    } else {
      b->by0 = sin(szt);
      b->C = cos(szt);
    }
  } else {
    const bool hel = (p.und_type == PF_UND_HELICAL);
    const double f = hel ? 1.0 : p.fx;
    // bx
    if (place == 0) {
      b->bx0 = hel ? (sz - pi * rho) / (6.0 * pi * rho) * cos(szt)
                   : f * (sz - pi * rho) / (6.0 * pi * rho) * cos(szt);
      if (sz < pi * rho) b->bx0 = 0.0;
      else if (sz > 7.0 * pi * rho) b->bx0 = hel ? cos(szt) : f * cos(szt);
    } else if (place == 2) {
      double s2 = sz - p.szfe;
      b->bx0 = hel ? -((s2 - 7.0 * pi * rho) / (6.0 * pi * rho) * cos(s2 / 2.0 / rho))
                   : -(f * (s2 - 7.0 * pi * rho) / (6.0 * pi * rho) * cos(s2 / 2.0 / rho));
      if (s2 < pi * rho) b->bx0 = hel ? cos(s2 / 2.0 / rho) : f * cos(s2 / 2.0 / rho);
      else if (s2 > 7.0 * pi * rho) b->bx0 = 0.0;
    } else {
      b->bx0 = hel ? cos(szt) : f * cos(szt);
    }
    // by
    if (place == 0) {
      b->by0 = hel ? szt / 4.0 / pi * sin(szt) : p.fy * szt / 4.0 / pi * sin(szt);
    } else if (place == 2) {
      double s = (sz - p.szfe) / 2.0 / rho;
      b->by0 = hel ? (-s / 4.0 / pi + 1.0) * sin(s) : p.fy * (-s / 4.0 / pi + 1.0) * sin(s);
    } else {
      b->by0 = hel ? sin(szt) : p.fy * sin(szt);
    }
    // bz
    const double c1 = b->c1;
    if (place == 1) {
      b->S = sin(szt);
      b->C = cos(szt);
    } else if (place == 0) {
      b->S = sin(szt);
      b->C = cos(szt);
      if (sz < pi * rho) {
        b->tcase = 0;
      } else if (sz > 7.0 * pi * rho) {
        b->tcase = 2;
        b->ux = hel ? c1 : c1 * p.fx;
      } else {
        b->tcase = 1;
        double u = c1 * (sz - pi * rho) / (6.0 * pi * rho);
        b->ux = hel ? u : u * p.fx;
      }
      double uy = szt / 4.0 / pi * seta / 2.0 / rho;
      b->uy = hel ? uy : uy * p.fy;
    } else {
      double s2 = sz - p.szfe;
      b->S = sin(s2 / 2.0 / rho);
      b->C = cos(s2 / 2.0 / rho);
      if (s2 < pi * rho) {
        b->tcase = 2;
        b->ux = hel ? c1 : c1 * p.fx;
      } else if (s2 > 7.0 * pi * rho) {
        b->tcase = 0;
      } else {
        b->tcase = 1;
        double u = c1 * (s2 - 7.0 * pi * rho) / (6.0 * pi * rho);
        b->ux = hel ? u : u * p.fx;
      }
      double uy = (-(s2 / 8.0 / pi / rho) + 1.0) * seta / 2.0 / rho;
      b->uy = hel ? uy : uy * p.fy;
    }
  }
}

// Dense beams (many macroparticles per window cell) deposit through the
// shared tile: direct atomics would pile onto few addresses.
static bool dense_mode(const pf_handle *h, size_t *smem) {
  const int64_t ntr = (int64_t)h->nix * h->niy;
  const size_t bytes = (size_t)4 * FT_PLANES * ntr * sizeof(u64);
  *smem = bytes;
  return h->np >= (int64_t)8 * h->npl * ntr && bytes <= 96 * 1024;
}

// Macroparticles per block of the dense mode: FT_PPB, unless that grid's
// waves of resident blocks are less than 85 % full, then a multiple of
// FT_THREADS sized so that the grid fills whole waves (2^22 macroparticles
// in blocks of 8192 made a grid of 1.12 waves, which left the SMs idle for
// 29 % of the launch: 4608 per block made it 2.0 waves and the saturated
// config-1-mesh run 25 % faster; at 2^24, 4.49 waves, smaller blocks
// measured no faster).
static int64_t dense_ppb(int64_t np, int64_t slots) {
  slots = std::max<int64_t>(1, slots);
  const int64_t nb = (np + FT_PPB - 1) / FT_PPB;
  const int64_t waves = std::max<int64_t>(1, (nb + slots - 1) / slots);
  if (nb >= (int64_t)(0.85 * (double)(waves * slots))) return FT_PPB;
  int64_t ppb = (np + waves * slots - 1) / (waves * slots);
  ppb = (ppb + FT_THREADS - 1) / FT_THREADS * FT_THREADS;
  return std::min<int64_t>(std::max<int64_t>(ppb, FT_THREADS), FT_PPB);
}

// k_stage<stage> over the a.np macroparticles a points to (the handle's
// beam, or a range of it), in the deposit mode the handle's beam takes
static int launch_stage(pf_handle *h, int stage, StageArgs &a) {
  // direct mode: blocks of 256 threads, halved down to 64 while the grid
  // has fewer than eight blocks per SM, so that a small beam's warps spread
  // over all SMs evenly (2^16 macroparticles: 256 blocks of 256 left 48 of
  // 152 SMs one block and the others two)
  const int nsm = pf_sm_count();
  int threads = 256;
  while (threads > 64 && (a.np + threads - 1) / threads < (int64_t)8 * nsm) threads /= 2;
  const int64_t blocks = (a.np + threads - 1) / threads;
  if (blocks == 0) return PF_OK;
  const bool oned = h->p.one_d != 0;
  size_t smem = 0;
  const bool dense = dense_mode(h, &smem);
  a.tile_ppb = FT_PPB;
  static PfDeviceOnce attr_once;  // the attribute is per device
  if (dense) {
    PF_CUDA(pf_device_once(attr_once, [] {
      const void *fns[] = {(const void *)k_stage<1, false, true>, (const void *)k_stage<2, false, true>,
                           (const void *)k_stage<3, false, true>, (const void *)k_stage<4, false, true>,
                           (const void *)k_stage<1, true, true>,  (const void *)k_stage<2, true, true>,
                           (const void *)k_stage<3, true, true>,  (const void *)k_stage<4, true, true>};
      for (const void *f : fns) {
        const cudaError_t e =
            cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
        if (e != cudaSuccess) return e;
      }
      return cudaSuccess;
    }));
    const void *kf = oned ? (const void *)k_stage<1, true, true> : (const void *)k_stage<1, false, true>;
    a.tile_ppb = (int)dense_ppb(a.np, pf_resident_blocks(kf, FT_THREADS, smem));
  }
  const int64_t dblocks = (a.np + a.tile_ppb - 1) / a.tile_ppb;
  pf_prof_begin(h, PROF_STAGE);
#define PF_STAGE_CASE(S)                                                                   \
  case S:                                                                                  \
    if (dense) {                                                                           \
      if (oned) k_stage<S, true, true><<<(unsigned)dblocks, FT_THREADS, smem, h->stream>>>(a); \
      else k_stage<S, false, true><<<(unsigned)dblocks, FT_THREADS, smem, h->stream>>>(a);     \
    } else {                                                                               \
      if (oned) k_stage<S, true><<<(unsigned)blocks, threads, 0, h->stream>>>(a);          \
      else k_stage<S, false><<<(unsigned)blocks, threads, 0, h->stream>>>(a);              \
    }                                                                                      \
    break;
  switch (stage) {
    PF_STAGE_CASE(1)
    PF_STAGE_CASE(2)
    PF_STAGE_CASE(3)
    PF_STAGE_CASE(4)
  }
#undef PF_STAGE_CASE
  pf_prof_end(h);
  PF_LAUNCHED(h);
  return PF_OK;
}

static int launch_nodes(pf_handle *h, int stage, NodeArgs &n) {
  const int threads = 256;
  const int64_t blocks = (n.n + threads - 1) / threads;
  if (blocks == 0) return PF_OK;
  pf_prof_begin(h, PROF_NODES);
  switch (stage) {
    case 1: k_nodes<1><<<(unsigned)blocks, threads, 0, h->stream>>>(n); break;
    case 2: k_nodes<2><<<(unsigned)blocks, threads, 0, h->stream>>>(n); break;
    case 3: k_nodes<3><<<(unsigned)blocks, threads, 0, h->stream>>>(n); break;
    case 4: k_nodes<4><<<(unsigned)blocks, threads, 0, h->stream>>>(n); break;
  }
  pf_prof_end(h);
  PF_LAUNCHED(h);
  return PF_OK;
}

// Particle, window and physics arguments of the stage kernels for the
// handle's current state (the per-stage fields are set by the caller).
void pf_fill_stage_args(pf_handle *h, StageArgs &a, double h6) {
  const pf_params &p = h->p;
  memset(&a, 0, sizeof(a));
  a.x = h->y[h->cur][0];
  a.y = h->y[h->cur][1];
  a.z2 = h->y[h->cur][2];
  a.px = h->y[h->cur][3];
  a.py = h->y[h->cur][4];
  a.gam = h->y[h->cur][5];
  a.chi = h->chi;
  a.np = h->np;
  a.h6 = h6;
  a.acc_lo_r = h->acc;
  a.acc_hi_r = h->acc + h->wcap;
  a.acc_lo_i = h->acc + 2 * h->wcap;
  a.acc_hi_i = h->acc + 3 * h->wcap;
  a.nix = h->nix;
  a.niy = h->niy;
  a.npl = h->npl;
  a.nz2 = p.nz2;
  a.periodic = (p.mesh_type == PF_MESH_PERIODIC);
  a.one_d = p.one_d;
  a.dx = p.dx;
  a.dy = p.dy;
  a.dz2 = p.dz2;
  a.dV3 = p.dx * p.dy * p.dz2;
  a.halfx = ((double)(h->nix - 1) / 2.0) * p.dx;
  a.halfy = ((double)(h->niy - 1) / 2.0) * p.dy;
  a.eta = p.eta;
  a.kappa = p.kappa;
  a.rho = p.rho;
  a.gamma_r = p.gamma_r * p.gamma_r;  // gamma0**2, as used by getP2
  a.aw = p.aw * p.aw;                 // aw**2
  a.sInv2rho = 1.0 / (2.0 * p.rho);
  a.dxc = 2.0 * p.rho * p.kappa / sqrt(p.eta);
  a.k2 = p.kappa * p.kappa;
  a.inv_eta = 1.0 / p.eta;
  a.eta_k2 = p.eta / a.k2;
  a.rho2 = 2.0 * p.rho;
  a.inv_dx = 1.0 / p.dx;
  a.inv_dy = 1.0 / p.dy;
  a.inv_dz2 = 1.0 / p.dz2;
  a.inv_dV3 = 1.0 / a.dV3;
  a.field_evolve = p.field_evolve;
  a.electrons_evolve = p.electrons_evolve;
  a.coupling = p.coupling;
  a.fix_e = h->fix_e;
  a.fix_maxexp = h->fix_maxexp;
  a.status = h->d_status;
}

int pf_launch_stage(pf_handle *h, int stage, StageArgs &a) { return launch_stage(h, stage, a); }

void pf_stage_pointers(pf_handle *h, StageArgs &a, int s, int cur) {
  const int nxt = cur ^ 1;
  a.x = h->y[cur][0];
  a.y = h->y[cur][1];
  a.z2 = h->y[cur][2];
  a.px = h->y[cur][3];
  a.py = h->y[cur][4];
  a.gam = h->y[cur][5];
  a.ar = (s == 1) ? h->wr : h->asr;
  a.ai = (s == 1) ? h->wi : h->asi;
  for (int j = 0; j < 6; ++j) {
    a.kin[j] = (s == 2) ? h->k1[j] : (s == 3) ? h->ka[j] : (s == 4) ? h->kb[j] : nullptr;
    a.kout[j] = (s == 1) ? h->k1[j] : (s == 3) ? h->kb[j] : nullptr;
    a.kacc[j] = (s >= 2) ? h->ka[j] : nullptr;
    a.k1[j] = h->k1[j];
    a.ynext[j] = h->y[nxt][j];
  }
}

void pf_fill_node_args(pf_handle *h, NodeArgs &n, double hstep) {
  memset(&n, 0, sizeof(n));
  n.n = h->nwin;
  n.acc_lo_r = h->acc;
  n.acc_hi_r = h->acc + h->wcap;
  n.acc_lo_i = h->acc + 2 * h->wcap;
  n.acc_hi_i = h->acc + 3 * h->wcap;
  n.wr = h->wr;
  n.wi = h->wi;
  n.asr = h->asr;
  n.asi = h->asi;
  n.d0r = h->d0r;
  n.d0i = h->d0i;
  n.d12r = h->d12r;
  n.d12i = h->d12i;
  n.h6 = hstep / 6.0;
  n.fix_e = h->fix_e;
  n.status = h->d_status;
}

int pf_sm_count() {
  static std::atomic<int> cache[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  int n = cache[dev].load(std::memory_order_relaxed);
  if (n == 0) {
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    n = std::max(1, n);
    cache[dev].store(n, std::memory_order_relaxed);
  }
  return n;
}

int pf_resident_blocks(const void *kernel, int threads, size_t smem) {
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
  return std::max(1, nsm * std::max(1, per_sm));
}

size_t pf_stage_tile_smem(const pf_handle *h) {
  const size_t bytes = (size_t)4 * FT_PLANES * h->nix * h->niy * sizeof(u64);
  return bytes <= 96 * 1024 ? bytes : 0;
}

cudaError_t pf_stage_batch(cudaStream_t st, int stage, bool tile, const StageArgs *args,
                           const BatchTile *tiles, int ntiles, int grid, int threads, size_t smem) {
  static PfDeviceOnce attr_once;  // the attribute is per device
  const cudaError_t attr = pf_device_once(attr_once, [] {
    const void *fns[] = {(const void *)k_stage_batch<1, true>, (const void *)k_stage_batch<2, true>,
                         (const void *)k_stage_batch<3, true>, (const void *)k_stage_batch<4, true>};
    cudaError_t err = cudaSuccess;
    for (const void *f : fns) {
      const cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
      if (e != cudaSuccess) err = e;
    }
    return err;
  });
  if (attr != cudaSuccess) return attr;
  if (ntiles <= 0) return cudaSuccess;
  if (grid < 0) {  // persistent: the blocks that fit on the device at once
    const void *f = tile ? (const void *)k_stage_batch<1, true> : (const void *)k_stage_batch<1, false>;
    grid = pf_resident_blocks(f, threads, tile ? smem : 0);
  }
  const unsigned g = (unsigned)(grid == 0 ? ntiles : std::max(1, std::min(grid, ntiles)));
#define PF_BATCH_CASE(S)                                                                   \
  case S:                                                                                  \
    if (tile) k_stage_batch<S, true><<<g, threads, smem, st>>>(args, tiles, ntiles);       \
    else k_stage_batch<S, false><<<g, threads, 0, st>>>(args, tiles, ntiles);              \
    break;
  switch (stage) {
    PF_BATCH_CASE(1)
    PF_BATCH_CASE(2)
    PF_BATCH_CASE(3)
    PF_BATCH_CASE(4)
  }
#undef PF_BATCH_CASE
  return cudaGetLastError();
}

cudaError_t pf_nodes_batch(cudaStream_t st, int stage, const NodeArgs *args,
                           const BatchTile *tiles, int ntiles, int grid, int threads,
                           int *step_ctr) {
  if (ntiles <= 0) return cudaSuccess;
  if (grid < 0) grid = pf_resident_blocks((const void *)k_nodes_batch<1>, threads, 0);
  const unsigned g = (unsigned)(grid == 0 ? ntiles : std::max(1, std::min(grid, ntiles)));
  switch (stage) {
    case 1: k_nodes_batch<1><<<g, threads, 0, st>>>(args, tiles, ntiles, nullptr); break;
    case 2: k_nodes_batch<2><<<g, threads, 0, st>>>(args, tiles, ntiles, nullptr); break;
    case 3: k_nodes_batch<3><<<g, threads, 0, st>>>(args, tiles, ntiles, nullptr); break;
    default: k_nodes_batch<4><<<g, threads, 0, st>>>(args, tiles, ntiles, step_ctr); break;
  }
  return cudaGetLastError();
}

cudaError_t pf_wrap_batch(cudaStream_t st, const WrapArgs *args, const BatchTile *tiles,
                          int ntiles, int grid, const int *step_ctr) {
  if (ntiles <= 0) return cudaSuccess;
  if (grid < 0) grid = pf_resident_blocks((const void *)k_wrap_batch, 256, 0);
  const unsigned g = (unsigned)(grid == 0 ? ntiles : std::max(1, std::min(grid, ntiles)));
  k_wrap_batch<<<g, 256, 0, st>>>(args, tiles, ntiles, step_ctr);
  return cudaGetLastError();
}

// The four stage-coefficient entries of one step at local zbar szl
// (advances the taper state as the step itself does).
void pf_step_coefficients(pf_handle *h, double szl, double hstep, StageCoef *out) {
  const double hh = hstep * 0.5, szh = szl + hh;
  const double stage_sz[4] = {szl, szh, szh, szl + hstep};
  for (int s = 0; s < 4; ++s) {
    double n2col;
    int place;
    pf_taper_stage(h, stage_sz[s], &n2col, &place);
    out[s].n2col = n2col;
    out[s].kn2col = h->p.kappa * n2col;
    pf_stage_coefficients(h->p, stage_sz[s], n2col, place, &out[s].bf);
  }
}
int pf_launch_nodes(pf_handle *h, int stage, NodeArgs &n) { return launch_nodes(h, stage, n); }

int pf_rk4_fp64(pf_handle *h, double szl, double hstep, unsigned int *status_out) {
  const pf_params &p = h->p;
  const double hh = hstep * 0.5, h6 = hstep / 6.0, szh = szl + hh;
  const double stage_sz[4] = {szl, szh, szh, szl + hstep};
  const double stage_c[4] = {0.0, hh, hh, hstep};
  const int nxt = h->cur ^ 1;

  // status_out == nullptr: enqueue only (a step of an asynchronous block;
  // the caller clears the status word once per block and reads it after)
  if (status_out) PF_CUDA(cudaMemsetAsync(h->d_status, 0, sizeof(unsigned int), h->stream));

  StageArgs a;
  pf_fill_stage_args(h, a, h6);
  if (h->capturing) {
    a.coef_tab = (const StageCoef *)h->coef_dev;
    a.step_ctr = h->step_ctr;
  }

  NodeArgs n;
  pf_fill_node_args(h, n, hstep);
  if (h->capturing) n.step_ctr = h->step_ctr;

  for (int s = 1; s <= 4; ++s) {
    double n2col;
    int place;
    pf_taper_stage(h, stage_sz[s - 1], &n2col, &place);
    a.n2col = n2col;
    a.kn2col = p.kappa * n2col;
    pf_stage_coefficients(p, stage_sz[s - 1], n2col, place, &a.bf);
    a.cstate = stage_c[s - 1];
    pf_stage_pointers(h, a, s, h->cur);
    int rc = launch_stage(h, s, a);
    if (rc) return rc;
    // the next stage's field is A0 + hh*d0, A0 + hh*d1, A0 + h*d2
    n.coef = (s == 3) ? hstep : hh;
    rc = launch_nodes(h, s, n);
    if (rc) return rc;
  }
  if (!status_out) {
    h->cur = nxt;  // committed optimistically; the block is replayed if it failed
    return PF_OK;
  }
  PF_CUDA(cudaMemcpyAsync(h->h_status, h->d_status, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                          h->stream));
  PF_CUDA(cudaStreamSynchronize(h->stream));
  pf_prof_flush(h);
  *status_out = *h->h_status;
  if (*status_out == 0u) h->cur = nxt;
  return PF_OK;
}

// ---------------------------------------------------------------------------
// The step with the driver's arrays in host memory (rk4par as the
// reference's driver calls it, every step handing in and taking back the
// particle arrays and the inner-window field).  The copies run on a second
// stream and overlap the kernels: the window field goes in first (every
// macroparticle of stage 1 gathers from it), the particles in chunks that
// stage 1 starts on as each arrives, and stage 4's output leaves chunk by
// chunk as it is written, the window field after the last node update.  The
// deposit is an integer sum, so the chunked stages give the bits of the
// whole-beam launches.  When the status word is set (a macroparticle out of
// the window or the mesh, an overflow, a non-finite value) the host arrays
// receive the step's input again and the device state is the step's input.
int pf_rk4_fp64_host(pf_handle *h, double szl, double hstep, double *const host[6], double *wre,
                     double *wim, unsigned int *status_out) {
  const pf_params &p = h->p;
  const double hh = hstep * 0.5, h6 = hstep / 6.0, szh = szl + hh;
  const double stage_sz[4] = {szl, szh, szh, szl + hstep};
  const double stage_c[4] = {0.0, hh, hh, hstep};
  const int cur = h->cur, nxt = cur ^ 1;
  const int64_t np = h->np;
  // chunks of at least 2^20 macroparticles (48 MB of state), at most 16:
  // smaller chunks shorten the first copy in and the last copy out, which
  // nothing overlaps, but their copies' fixed costs measured larger (2^18:
  // 12.3 ms per config-2 step against 11.1; the first and last three
  // chunks graded down to 2^18, the others 2^20: no change, 10.1 ms)
  const int64_t chunk = std::max<int64_t>((int64_t)1 << 20, (np + 15) / 16);
  const int nch = (int)std::max<int64_t>(1, (np + chunk - 1) / chunk);
  if (!h->copy_stream)
    PF_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
  while ((int)h->copy_events.size() < 2 * nch + 1) {
    cudaEvent_t e;
    PF_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    h->copy_events.push_back(e);
  }
  cudaEvent_t *ev_in = h->copy_events.data(), *ev_out = ev_in + nch, ev_w = ev_in[2 * nch];
  cudaStream_t cs = h->copy_stream, st = h->stream;
  const size_t wb = (size_t)h->nwin * sizeof(double);

  PF_CUDA(cudaMemsetAsync(h->d_status, 0, sizeof(unsigned int), st));
  PF_CUDA(cudaMemcpyAsync(h->wr, wre, wb, cudaMemcpyHostToDevice, st));
  PF_CUDA(cudaMemcpyAsync(h->wi, wim, wb, cudaMemcpyHostToDevice, st));
  for (int c = 0; c < nch; ++c) {
    const int64_t off = c * chunk, len = std::min(chunk, np - off);
    for (int j = 0; j < 6; ++j)
      PF_CUDA(cudaMemcpyAsync(h->y[cur][j] + off, host[j] + off, (size_t)len * sizeof(double),
                              cudaMemcpyHostToDevice, cs));
    PF_CUDA(cudaEventRecord(ev_in[c], cs));
  }

  StageArgs a;
  pf_fill_stage_args(h, a, h6);
  NodeArgs n;
  pf_fill_node_args(h, n, hstep);
  // the stage arguments of macroparticles [off, off + len)
  auto range = [](const StageArgs &b, int64_t off, int64_t len) {
    StageArgs r = b;
    r.x += off;
    r.y += off;
    r.z2 += off;
    r.px += off;
    r.py += off;
    r.gam += off;
    r.chi += off;
    for (int j = 0; j < 6; ++j) {
      if (r.kin[j]) r.kin[j] += off;
      if (r.kout[j]) r.kout[j] += off;
      if (r.kacc[j]) r.kacc[j] += off;
      if (r.k1[j]) r.k1[j] += off;
      if (r.ynext[j]) r.ynext[j] += off;
    }
    r.np = len;
    return r;
  };
  for (int s = 1; s <= 4; ++s) {
    double n2col;
    int place;
    pf_taper_stage(h, stage_sz[s - 1], &n2col, &place);
    a.n2col = n2col;
    a.kn2col = p.kappa * n2col;
    pf_stage_coefficients(p, stage_sz[s - 1], n2col, place, &a.bf);
    a.cstate = stage_c[s - 1];
    pf_stage_pointers(h, a, s, cur);
    if (s == 1 || s == 4) {
      for (int c = 0; c < nch; ++c) {
        const int64_t off = c * chunk, len = std::min(chunk, np - off);
        if (s == 1) PF_CUDA(cudaStreamWaitEvent(st, ev_in[c], 0));
        StageArgs r = range(a, off, len);
        int rc = launch_stage(h, s, r);
        if (rc) return rc;
        if (s == 4) {
          // this chunk's new state leaves while the next chunks run
          PF_CUDA(cudaEventRecord(ev_out[c], st));
          PF_CUDA(cudaStreamWaitEvent(cs, ev_out[c], 0));
          for (int j = 0; j < 6; ++j)
            PF_CUDA(cudaMemcpyAsync(host[j] + off, h->y[nxt][j] + off,
                                    (size_t)len * sizeof(double), cudaMemcpyDeviceToHost, cs));
        }
      }
    } else {
      int rc = launch_stage(h, s, a);
      if (rc) return rc;
    }
    n.coef = (s == 3) ? hstep : hh;
    int rc = launch_nodes(h, s, n);
    if (rc) return rc;
  }
  PF_CUDA(cudaMemcpyAsync(wre, h->wr, wb, cudaMemcpyDeviceToHost, st));
  PF_CUDA(cudaMemcpyAsync(wim, h->wi, wb, cudaMemcpyDeviceToHost, st));
  PF_CUDA(cudaMemcpyAsync(h->h_status, h->d_status, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                          st));
  PF_CUDA(cudaEventRecord(ev_w, st));
  PF_CUDA(cudaStreamWaitEvent(cs, ev_w, 0));
  PF_CUDA(cudaStreamSynchronize(cs));
  *status_out = *h->h_status;
  if (*status_out == 0u) {
    h->cur = nxt;
    return PF_OK;
  }
  // a failed step: the window field was left as it came in (stage 4's node
  // update commits nothing once the status is set); the particles go back
  for (int j = 0; j < 6; ++j)
    PF_CUDA(cudaMemcpyAsync(host[j], h->y[cur][j], (size_t)np * sizeof(double),
                            cudaMemcpyDeviceToHost, st));
  PF_CUDA(cudaStreamSynchronize(st));
  return PF_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free RK4 step.
//
// Some callers of this library cannot allocate device memory: a host program
// whose device memory belongs to its own pool allocator and forbids allocations
// from outside it, a plugin host that hands in buffers it allocated up front,
// or a time-critical loop that cannot afford cudaMalloc's implicit device-wide
// synchronisation.  pf_rk4_step_noalloc serves them: the caller owns the
// particle arrays and the inner-window field (device memory, updated in place)
// and the RK4 temporaries live in the fixed-size file-scope device array below,
// which every GPU that loads this library holds until the process exits.
//
// Limits: at most PF_NOALLOC_MAX_PARTICLES macroparticles and
// PF_NOALLOC_MAX_NODES inner-window nodes (nix * niy * planes held); larger
// problems are rejected with PF_BAD_ARG.  Every call uses the same array and
// leaves its contents behind, so each call clears what must start at zero (the
// deposit accumulators and the status word); two calls that overlap on the GPU
// (e.g. on different streams) race on it.  The first call on a device looks up
// the array's device address (cudaGetSymbolAddress) with that device current
// and keeps it for the life of the process, so the device's primary context
// must stay the one in use: a cudaDeviceReset, or a caller-made non-primary
// context, is not supported.  Every call waits for its stream twice (after the
// deposit-scale reduction and after the status read), so no call may be made
// while its stream is being captured into a CUDA graph.
namespace {

constexpr int64_t NA_NP = PF_NOALLOC_MAX_PARTICLES;
constexpr int64_t NA_NW = PF_NOALLOC_MAX_NODES;
// doubles: k1, ka, kb, next state (6 arrays each of NA_NP); stage field,
// field slopes d0, d12 (re, im each of NA_NW); then 4 * NA_NW 64-bit deposit
// words, the status word and a reduction word.
constexpr size_t NA_DOUBLES = (size_t)24 * NA_NP + (size_t)6 * NA_NW;
constexpr size_t NA_BYTES = NA_DOUBLES * 8 + (size_t)4 * NA_NW * 8 + 2 * 256;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[64] = {};

__global__ void k_noalloc_absmax(const double *v, int64_t n, unsigned long long *out) {
  unsigned long long m = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    m = max(m, (unsigned long long)__double_as_longlong(fabs(v[i])));
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

}  // namespace

extern "C" int pf_rk4_step_noalloc(const pf_params *p, double *n2col, double *n2col0,
                                   double szl, double hstep, int64_t np, double *x, double *y,
                                   double *z2, double *px, double *py, double *gam,
                                   const double *chi, double *wr, double *wi, int32_t nix,
                                   int32_t niy, void *stream) {
  if (!p || !n2col || !n2col0 || np < 0 || nix < 1 || niy < 1) return PF_BAD_ARG;
  if (np > 0 && (!x || !y || !z2 || !px || !py || !gam || !chi)) return PF_BAD_ARG;
  if (!wr || !wi) return PF_BAD_ARG;
  if (p->precision != PF_FP64 || p->nz2 < 2 || p->dz2 <= 0.0 || p->dx <= 0.0 || p->dy <= 0.0)
    return PF_BAD_ARG;
  if (p->one_d && (nix != 1 || niy != 1)) return PF_BAD_ARG;
  const int64_t npl = (p->mesh_type == PF_MESH_PERIODIC) ? p->nz2 - 1 : p->nz2;
  const int64_t nwin = (int64_t)nix * niy * npl;
  if (np > NA_NP || nwin > NA_NW) return PF_BAD_ARG;  // beyond the fixed scratch
  cudaStream_t st = (cudaStream_t)stream;

  // one-time lookup of the scratch array's device address on this device
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return PF_CUDA_ERR;
  unsigned char *base;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
      void *ptr = nullptr;
      if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return PF_CUDA_ERR;
      g_noalloc_ptr[dev] = ptr;
    }
    base = (unsigned char *)g_noalloc_ptr[dev];
  }
  double *dbl = (double *)base;
  double *k1[6], *ka[6], *kb[6], *ynext[6];
  for (int j = 0; j < 6; ++j) {
    k1[j] = dbl + (size_t)j * NA_NP;
    ka[j] = dbl + (size_t)(6 + j) * NA_NP;
    kb[j] = dbl + (size_t)(12 + j) * NA_NP;
    ynext[j] = dbl + (size_t)(18 + j) * NA_NP;
  }
  double *fld = dbl + (size_t)24 * NA_NP;
  double *asr = fld, *asi = fld + NA_NW, *d0r = fld + 2 * NA_NW, *d0i = fld + 3 * NA_NW;
  double *d12r = fld + 4 * NA_NW, *d12i = fld + 5 * NA_NW;
  unsigned long long *acc = (unsigned long long *)(base + NA_DOUBLES * 8);
  unsigned int *status = (unsigned int *)(base + NA_DOUBLES * 8 + (size_t)4 * NA_NW * 8);
  unsigned long long *red = (unsigned long long *)((unsigned char *)status + 256);

  // the array keeps the previous call's contents: clear what must start at zero
  if (cudaMemsetAsync(acc, 0, (size_t)4 * NA_NW * 8, st) != cudaSuccess) return PF_CUDA_ERR;
  if (cudaMemsetAsync(status, 0, sizeof(unsigned int), st) != cudaSuccess) return PF_CUDA_ERR;
  if (cudaMemsetAsync(red, 0, sizeof(unsigned long long), st) != cudaSuccess) return PF_CUDA_ERR;

  // fixed-point scale of the deposit from max |chi| / dV3
  double chimax = 0.0;
  if (np > 0) {
    k_noalloc_absmax<<<(unsigned)std::min<int64_t>((np + 255) / 256, 1024), 256, 0, st>>>(chi, np, red);
    if (cudaGetLastError() != cudaSuccess) return PF_CUDA_ERR;
    unsigned long long r = 0;
    if (cudaMemcpyAsync(&r, red, sizeof(r), cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return PF_CUDA_ERR;
    if (cudaStreamSynchronize(st) != cudaSuccess) return PF_CUDA_ERR;
    memcpy(&chimax, &r, sizeof(r));
  }
  int lg = 0;
  while ((int64_t(1) << lg) < 2 * np + 2) ++lg;
  const int fix_maxexp = 126 - lg;
  const double smax = chimax / (p->dx * p->dy * p->dz2);
  const int fix_e = fix_maxexp - 16 - ((smax > 0.0 && isfinite(smax)) ? ilogb(smax) + 1 : 0);

  StageArgs a;
  memset(&a, 0, sizeof(a));
  a.x = x;
  a.y = y;
  a.z2 = z2;
  a.px = px;
  a.py = py;
  a.gam = gam;
  a.chi = chi;
  a.np = np;
  a.h6 = hstep / 6.0;
  a.acc_lo_r = acc;
  a.acc_hi_r = acc + NA_NW;
  a.acc_lo_i = acc + 2 * NA_NW;
  a.acc_hi_i = acc + 3 * NA_NW;
  a.nix = nix;
  a.niy = niy;
  a.npl = npl;
  a.nz2 = p->nz2;
  a.periodic = (p->mesh_type == PF_MESH_PERIODIC);
  a.one_d = p->one_d;
  a.dx = p->dx;
  a.dy = p->dy;
  a.dz2 = p->dz2;
  a.dV3 = p->dx * p->dy * p->dz2;
  a.halfx = ((double)(nix - 1) / 2.0) * p->dx;
  a.halfy = ((double)(niy - 1) / 2.0) * p->dy;
  a.eta = p->eta;
  a.kappa = p->kappa;
  a.rho = p->rho;
  a.gamma_r = p->gamma_r * p->gamma_r;
  a.aw = p->aw * p->aw;
  a.sInv2rho = 1.0 / (2.0 * p->rho);
  a.dxc = 2.0 * p->rho * p->kappa / sqrt(p->eta);
  a.k2 = p->kappa * p->kappa;
  a.inv_eta = 1.0 / p->eta;
  a.eta_k2 = p->eta / a.k2;
  a.rho2 = 2.0 * p->rho;
  a.inv_dx = 1.0 / p->dx;
  a.inv_dy = 1.0 / p->dy;
  a.inv_dz2 = 1.0 / p->dz2;
  a.inv_dV3 = 1.0 / a.dV3;
  a.field_evolve = p->field_evolve;
  a.electrons_evolve = p->electrons_evolve;
  a.coupling = p->coupling;
  a.fix_e = fix_e;
  a.fix_maxexp = fix_maxexp;
  a.status = status;

  NodeArgs nd;
  memset(&nd, 0, sizeof(nd));
  nd.n = nwin;
  nd.acc_lo_r = a.acc_lo_r;
  nd.acc_hi_r = a.acc_hi_r;
  nd.acc_lo_i = a.acc_lo_i;
  nd.acc_hi_i = a.acc_hi_i;
  nd.wr = wr;
  nd.wi = wi;
  nd.asr = asr;
  nd.asi = asi;
  nd.d0r = d0r;
  nd.d0i = d0i;
  nd.d12r = d12r;
  nd.d12i = d12i;
  nd.h6 = a.h6;
  nd.fix_e = fix_e;
  nd.status = status;

  const double hh = hstep * 0.5, szh = szl + hh;
  const double stage_sz[4] = {szl, szh, szh, szl + hstep};
  const double stage_c[4] = {0.0, hh, hh, hstep};
  const unsigned pg = (unsigned)std::max<int64_t>(1, (np + 255) / 256);
  const unsigned ng = (unsigned)std::max<int64_t>(1, (nwin + 255) / 256);
  for (int s = 1; s <= 4; ++s) {
    // getAlpha (wiggler_taper.f90:39-47) and adjUndPlace on the caller's state
    const double sz = stage_sz[s - 1];
    if ((sz >= p->szfs) && (sz <= p->szfe)) *n2col = *n2col0 + p->undgrad * (sz - p->szfs);
    else if (sz > p->szfe) *n2col0 = *n2col;
    int place = 1;
    if (p->und_ends) place = (sz <= p->szfs) ? 0 : (sz >= p->szfe) ? 2 : 1;
    a.n2col = *n2col;
    a.kn2col = p->kappa * *n2col;
    pf_stage_coefficients(*p, sz, *n2col, place, &a.bf);
    a.cstate = stage_c[s - 1];
    a.ar = (s == 1) ? wr : asr;
    a.ai = (s == 1) ? wi : asi;
    for (int j = 0; j < 6; ++j) {
      a.kin[j] = (s == 2) ? k1[j] : (s == 3) ? ka[j] : (s == 4) ? kb[j] : nullptr;
      a.kout[j] = (s == 1) ? k1[j] : (s == 3) ? kb[j] : nullptr;
      a.kacc[j] = (s >= 2) ? ka[j] : nullptr;
      a.k1[j] = k1[j];
      a.ynext[j] = ynext[j];
    }
    if (np > 0) {
      const bool oned = p->one_d != 0;
      switch (s) {
        case 1: oned ? k_stage<1, true><<<pg, 256, 0, st>>>(a) : k_stage<1, false><<<pg, 256, 0, st>>>(a); break;
        case 2: oned ? k_stage<2, true><<<pg, 256, 0, st>>>(a) : k_stage<2, false><<<pg, 256, 0, st>>>(a); break;
        case 3: oned ? k_stage<3, true><<<pg, 256, 0, st>>>(a) : k_stage<3, false><<<pg, 256, 0, st>>>(a); break;
        default: oned ? k_stage<4, true><<<pg, 256, 0, st>>>(a) : k_stage<4, false><<<pg, 256, 0, st>>>(a); break;
      }
      if (cudaGetLastError() != cudaSuccess) return PF_CUDA_ERR;
    }
    nd.coef = (s == 3) ? hstep : hh;
    switch (s) {
      case 1: k_nodes<1><<<ng, 256, 0, st>>>(nd); break;
      case 2: k_nodes<2><<<ng, 256, 0, st>>>(nd); break;
      case 3: k_nodes<3><<<ng, 256, 0, st>>>(nd); break;
      default: k_nodes<4><<<ng, 256, 0, st>>>(nd); break;
    }
    if (cudaGetLastError() != cudaSuccess) return PF_CUDA_ERR;
  }
  unsigned int hst = 0;
  if (cudaMemcpyAsync(&hst, status, sizeof(hst), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return PF_CUDA_ERR;
  if (cudaStreamSynchronize(st) != cudaSuccess) return PF_CUDA_ERR;
  if (hst != 0u) return pf_status_of(hst);  // state left unchanged, as the reference
  double *dst[6] = {x, y, z2, px, py, gam};
  for (int j = 0; j < 6 && np > 0; ++j)
    if (cudaMemcpyAsync(dst[j], ynext[j], sizeof(double) * (size_t)np, cudaMemcpyDeviceToDevice,
                        st) != cudaSuccess)
      return PF_CUDA_ERR;
  if (cudaStreamSynchronize(st) != cudaSuccess) return PF_CUDA_ERR;
  return PF_OK;
}
