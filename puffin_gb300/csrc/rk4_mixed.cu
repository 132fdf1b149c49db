// Mixed-precision RK4 macroparticle push.
//
// FP64: the particle state (x, y, z2, px, py, Gamma) in HBM and every RK4
// stage combination y + h/6 (k1 + k4 + 2 (k2 + k3)); the stage values of z2
// and Gamma; p2 (the z2 velocity, which sets the ponderomotive phase) and the
// z2 cell index and fraction.
// FP32: the field window, the transverse stage coordinates and momenta
// (px^2 + py^2 enters p2 as a 1e-4 correction, so FP32 keeps u to ~1e-11)
// and interpolation weights, the gather, the source term and its deposit, the
// b-fields, the momentum/energy equations, and the slopes of x, y, px, py and
// Gamma (the z2 slope p2 stays FP64).
//
// GB300 issues FP64 at 1/64 of the FP32 rate, so this kernel is bound by its
// FP64 instruction count: conversions between FP32 and FP64 are done with
// integer operations (f2d, d2f_rn below), which keeps them off the FP64 pipe,
// and 1/Gamma is a FP32 reciprocal refined by one FP64 Newton step.
//
// p2 (gamma_to_p2.f90:84-85) is (1/sqrt(1-u) - 1)/eta with
// u = (1 + aw^2 p_perp^2)/(gamma0^2 Gamma^2) of order 1e-7: the reference form
// cancels 7 digits.  Here r - 1 = 1/sqrt(1-u) - 1 is summed as its binomial
// series u/2 + 3u^2/8 + 5u^3/16 + ... (below u = 2e-6 as (u/2)(1 + c) with
// the small correction c in FP32; five terms for u < 1e-4, seven for
// u < 1e-3, truncation below 1e-16 of the result; the reference form above
// that), which is accurate to 1e-13 or better and needs no square root or
// division.
//
// Deposit: each block of up to 3072 macroparticles (6 per thread; 8 for beams
// dense along z2; fewer
// for beams too small to fill the SMs) accumulates its
// contributions to the three z2 planes from the lowest plane its particles
// start from in a shared-memory tile, deposited as each macroparticle's
// slopes are computed (nothing per particle is kept, which keeps the kernel
// near 64 registers and two 512-thread blocks per SM).  The tile sums are
// exact: each FP32 contribution is converted to a fixed-point integer
// v * 2^E truncated (|v * 2^E| < 2^31, E chosen per beam from max
// chi/dV3, one float-to-int conversion) split into a signed high part
// (v >> 20) and a 20-bit low part, which are added with two non-returning
// 32-bit shared-memory reductions into separate words; the at most 4096 low
// parts (< 2^20 each) a node can receive from one block stay below 2^32, so
// no carry is lost.
// The flush forms (sum_hi 2^20 + sum_lo) 2^-E in FP32 once per node and adds
// it to HBM with one float atomic per component.  Contributions
// outside the tile, or larger than the tile's range, go straight to HBM.
// Macroparticles ordered along z2 (as Puffin's beams are generated) make the
// tile catch nearly all.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <mutex>

#include "mixed_common.cuh"
#include "pf_internal.h"

namespace {

constexpr int MX_THREADS = 512;
constexpr int MX_PPT = 8;  // macroparticles per thread, at most
// the unsigned low words of the exact tile hold up to 4096 parts below 2^20
static_assert(MX_THREADS * MX_PPT <= 4096, "tile low words could carry");
// planes of the shared deposit tile: 3, or 8 where eight fit MX_TILE_BYTES
// (three 512-thread blocks per SM); a compile-time count keeps the kernel
// within its 40 registers
constexpr int MX_TILE_PLANES = 3;
constexpr int MX_TILE_PLANES_WIDE = 8;
constexpr size_t MX_TILE_BYTES = 72 * 1024;

struct MixArgs {
  const void *coef_tab;  // non-null: StageCoefF at [*step_ctr * 4 + stage - 1]
  const int *step_ctr;
  const double *x, *y, *z2, *px, *py, *gam;
  const float *chi_f;  // chi rounded to FP32 (set with the particles)
  float4 *base4;       // x, y, px, py of the step's start state in FP32 (stage 1 writes)
  // slopes: FP32 arrays for x, y, px, py, Gamma (index 2 unused), FP64 for z2
  const float *kin_f[6];
  const double *kin_z;
  float *kout_f[6];
  double *kout_z;
  float *kacc_f[6];
  double *kacc_z;
  const float *k1_f[6];
  const double *k1_z;
  double *ynext[6];
  int64_t np;
  double cstate, h6;
  float cstate_f, eta_f, inv_dx_f, inv_dy_f, hx_dx, hy_dy, inv_dz2_f;
  float ser_r1, ser_r2;  // ser[1] / ser[0], ser[2] / ser[0]
  int ppt;             // macroparticles per thread (1..MX_PPT)
  int fixE;            // tile fixed-point exponent
  float fix_scale;     // 2^fixE
  float tile_vmax;     // contributions at or above this go to HBM
  float npl_f, inv_npl_f;  // planes held (periodic plane estimate of the tile origin)
  double aw2g, g02;    // aw^2 / gamma0^2, 1 / gamma0^2
  double ser[7];       // binomial coefficients of 1/sqrt(1-u) - 1, times 1/eta
  const float2 *as;  // stage field (window, interleaved complex)
  float2 *acc;       // deposit accumulator (window)
  int nix, niy;
  int64_t npl, nz2;
  int periodic, one_d, tile;
  double halfx, halfy, inv_dx, inv_dy, inv_dz2;
  double inv_g02, aw2, inv_eta, eta;
  float inv_dV3, sInv2rho, dxc, eta_k2, kn2col, n2col, rho2;
  BFieldF bf;
  int field_evolve, electrons_evolve, coupling;
  unsigned int *status;
};

struct MixNodeArgs {
  int64_t n;
  float2 *acc, *w, *as, *d0, *d12;
  float coef, h6;
  const unsigned int *status;
  int *step_ctr;  // non-null: stage 4 advances it once per step
};

// per-(step, stage) coefficients of a replayed step block (FP32 form)
struct StageCoefF {
  BFieldF bf;
  float n2col, kn2col;
};

// v * 2^E truncated toward zero (scale = 2^E, so the product is exact);
// the caller guarantees |v * 2^E| < 2^31
__device__ __forceinline__ int f2fix(float v, float scale) { return __float2int_rz(v * scale); }

// exact shared-tile add of a fixed-point value: high part (signed) and the
// 20-bit low part into separate 32-bit words, non-returning reductions
// (straight-line: a zero contribution adds zero)
__device__ __forceinline__ void tile_add(int *hi, unsigned *lo, int r) {
  atomicAdd(hi, r >> 20);
  atomicAdd(lo, (unsigned)r & 0xFFFFFu);
}

// one vector reduction (both components) per node in global memory
__device__ __forceinline__ void global_add(float2 *a, float2 v) { atomicAdd(a, v); }

// One block's macroparticles i0 + q MX_THREADS + threadIdx.x (q < ppt,
// below i1).  Every thread of the block calls it (it holds block barriers
// when the tile is on).
template <int STAGE, bool ONED, int TP>
__device__ __forceinline__ void mixed_block(const MixArgs &a, const int64_t i0, const int64_t i1,
                                            const int ppt, float *tile, int &s_pzlo) {
  const int ntr = a.nix * a.niy;
  const int tile_n = TP * ntr;
  // [re hi | im hi | re lo | im lo], tile_n words each
  int *thi_r = reinterpret_cast<int *>(tile);
  int *thi_i = thi_r + tile_n;
  unsigned *tlo_r = reinterpret_cast<unsigned *>(thi_i + tile_n);
  unsigned *tlo_i = tlo_r + tile_n;

  const bool halted = (*((volatile unsigned int *)a.status) != 0u);
  if (a.tile) {
    // tile origin: the lowest z2 plane the block's macroparticles start from
    // (stage positions only move forward from there, p2 > 0)
    for (int t = threadIdx.x; t < 4 * tile_n; t += MX_THREADS) thi_r[t] = 0;
    if (threadIdx.x == 0) s_pzlo = INT_MAX;
    __syncthreads();
    // an estimate is enough (a wrong origin only sends deposits to HBM): the
    // smallest z2 of the warp's particles, as the integer order of the bits
    // of z2 >= 0, converted once per warp
    long long kmin = LLONG_MAX;
#pragma unroll
    for (int q = 0; q < ppt; ++q) {
      const int64_t i = i0 + q * MX_THREADS + threadIdx.x;
      if (halted || i >= i1) continue;
      kmin = min(kmin, __double_as_longlong(a.z2[i]));
    }
    for (int o = 16; o > 0; o >>= 1) kmin = min(kmin, __shfl_xor_sync(0xffffffffu, kmin, o));
    if ((threadIdx.x & 31) == 0 && kmin != LLONG_MAX) {
      float fz = floorf(d2f_rn(__longlong_as_double(kmin)) * a.inv_dz2_f);
      if (fabsf(fz) < 1.0e7f) {
        if (a.periodic) fz = fmaxf(fz - a.npl_f * floorf(fz * a.inv_npl_f), 0.f);
        atomicMin(&s_pzlo, (int)fz);
      }
    }
    __syncthreads();
  }
  const int pzlo = a.tile ? s_pzlo : 0;

#pragma unroll 1
  for (int q = 0; q < ppt; ++q) {
    const int64_t i = i0 + q * MX_THREADS + threadIdx.x;
    if (halted || i >= i1) continue;
    // FP64 state; stage values of z2 and Gamma in FP64, of x, y, px, py in
    // FP32 from their FP32 roundings, which stage 1 keeps for the later stages
    const double z0 = a.z2[i], g0 = a.gam[i];
    float kin[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    double kz_in = 0.0;
    double zs = z0, gs = g0;
    float X, Y, PX, PY;
    if (STAGE == 1) {
      X = d2f_rn(a.x[i]);
      Y = d2f_rn(a.y[i]);
      PX = d2f_rn(a.px[i]);
      PY = d2f_rn(a.py[i]);
      a.base4[i] = make_float4(X, Y, PX, PY);
    } else {
      const float4 b = a.base4[i];
      X = b.x;
      Y = b.y;
      PX = b.z;
      PY = b.w;
    }
    if (STAGE > 1) {
      kin[0] = a.kin_f[0][i];
      kin[1] = a.kin_f[1][i];
      kin[3] = a.kin_f[3][i];
      kin[4] = a.kin_f[4][i];
      kin[5] = a.kin_f[5][i];
      kz_in = a.kin_z[i];
      zs = fma(a.cstate, kz_in, z0);
      gs = fma(a.cstate, f2d(kin[5]), g0);
      PX = fmaf(a.cstate_f, kin[3], PX);
      PY = fmaf(a.cstate_f, kin[4], PY);
      X = fmaf(a.cstate_f, kin[0], X);
      Y = fmaf(a.cstate_f, kin[1], Y);
    }
    // a NaN or infinity in the stage state stops the step (PF_NOT_FINITE)
    if (!(pf_finite(zs) && pf_finite(gs) && isfinite(X + Y + PX + PY)))
      atomicOr(a.status, ST_NOT_FINITE);
    const float Gf = d2f_rn(gs);
    // 1/Gamma: FP32 reciprocal and one FP64 Newton step (relative error ~1e-14)
    const float rGf = __frcp_rn(Gf);
    double rG = f2d(rGf);
    rG = fma(rG, fma(-gs, rG, 1.0), rG);
    // px^2 + py^2 in FP32: aw^2 (px^2 + py^2) is ~1e-4 of 1 + aw^2 (px^2 + py^2),
    // so its rounding stays near 1e-11 of u
    const double u = fma(a.aw2g, f2d(fmaf(PX, PX, PY * PY)), a.g02) * (rG * rG);
    const double p2 = p2_series(u, a.ser, a.inv_eta, a.ser_r1, a.ser_r2);
    const float p2f = d2f_rn(p2);
    const float qrG = fmaf(a.eta_f, p2f, 1.f) * rGf;

    // z2 cell and fraction from the FP64 position, fraction and weights in FP32
    const double tz = zs * a.inv_dz2;
    int iz = 0;
    float zw2 = 0.f;
    bool ok = true;
    if (!cell_split(tz, iz, zw2)) {
      const double fz = floor(tz);
      if (!(fabs(fz) < 2.0e9)) {
        ok = false;
      } else {
        iz = (int)fz;
        zw2 = d2f_rn(tz - fz);
      }
    }
    int pz0 = 0, pz1 = 0;
    if (!ok) {
      atomicOr(a.status, ST_OUT_OF_Z2);
    } else if (a.periodic) {
      const int npl = (int)a.npl;
      int m = iz;
      if ((unsigned)m >= (unsigned)npl) {  // z2 outside the first period (rare)
        m %= npl;
        if (m < 0) m += npl;
      }
      pz0 = m;
      pz1 = (m + 1 == a.npl) ? 0 : m + 1;
    } else if (!(iz >= 0 && iz + 1 < a.nz2)) {
      ok = false;
      atomicOr(a.status, ST_OUT_OF_Z2);
    } else {
      pz0 = iz;
      pz1 = iz + 1;
    }
    float x2 = 0.f, y2 = 0.f;
    int64_t b0 = 0;
    if (!ONED) {
      // (x + halfx) / dx in one rounding
      const float tx = fmaf(X, a.inv_dx_f, a.hx_dx);
      const float fx = floorf(tx);
      const float ty = fmaf(Y, a.inv_dy_f, a.hy_dy);
      const float fy = floorf(ty);
      if (!(fx >= 0.f && fx + 1.f < (float)a.nix && fy >= 0.f && fy + 1.f < (float)a.niy)) {
        ok = false;
        atomicOr(a.status, ST_OUT_OF_WINDOW);
      } else {
        x2 = tx - fx;
        y2 = ty - fy;
        b0 = (int64_t)fx + (int64_t)fy * a.nix;
      }
    }
    const float x1 = 1.f - x2, y1 = 1.f - y2, zw1 = 1.f - zw2;

    float fr = 0.f, fi = 0.f;
    if (ok) {
      if (ONED) {
        const float2 c0 = a.as[pz0], c1 = a.as[pz1];
        fr = zw1 * c0.x + zw2 * c1.x;
        fi = zw1 * c0.y + zw2 * c1.y;
      } else {
        const float2 *p0 = a.as + (int64_t)pz0 * ntr + b0;
        const float2 *p1 = a.as + (int64_t)pz1 * ntr + b0;
        const float2 c0 = p0[0], c1 = p0[1], c2 = p0[a.nix], c3 = p0[a.nix + 1];
        const float2 c4 = p1[0], c5 = p1[1], c6 = p1[a.nix], c7 = p1[a.nix + 1];
        const float w0 = x1 * y1, w1 = x2 * y1, w2 = x1 * y2, w3 = x2 * y2;
        fr = zw1 * (w0 * c0.x + w1 * c1.x + w2 * c2.x + w3 * c3.x) +
             zw2 * (w0 * c4.x + w1 * c5.x + w2 * c6.x + w3 * c7.x);
        fi = zw1 * (w0 * c0.y + w1 * c1.y + w2 * c2.y + w3 * c3.y) +
             zw2 * (w0 * c4.y + w1 * c5.y + w2 * c6.y + w3 * c7.y);
      }
      if (!isfinite(fr + fi)) atomicOr(a.status, ST_NOT_FINITE);
      if (a.field_evolve) {
        // deposit (chi/dV3) (1 + eta p2)/Gamma p w_c to the 8 (2 on 1D) nodes
        const float dw = a.chi_f[i] * a.inv_dV3 * qrG;
        const float sr = dw * PX, si = dw * PY;
        const int nc = ONED ? 2 : 8;
        // tile planes from the origin (a block straddling the end of the
        // periodic mesh takes the per-corner path below, which wraps)
        const int tp0 = pz0 - pzlo, tp1 = pz1 - pzlo;
        if (a.tile && (unsigned)tp0 < (unsigned)TP &&
            (unsigned)tp1 < (unsigned)TP && fabsf(sr) < a.tile_vmax &&
            fabsf(si) < a.tile_vmax) {
          // the common case: both planes in the tile, and every corner's
          // |w s| <= |s| fits the tile's range (0 <= w <= 1)
          const int t0 = tp0 * ntr + (ONED ? 0 : (int)b0), t1 = tp1 * ntr + (ONED ? 0 : (int)b0);
          // the source scaled to the tile's fixed point once (a power of two:
          // exact), so each corner is one product and one conversion
          const float srs = sr * a.fix_scale, sis = si * a.fix_scale;
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            if (c >= nc) break;
            float w;
            int ti;
            if (ONED) {
              w = (c == 0) ? zw1 : zw2;
              ti = (c == 0) ? t0 : t1;
            } else {
              const int cx = c & 1, cy = (c >> 1) & 1, cz = c >> 2;
              w = (cx ? x2 : x1) * (cy ? y2 : y1) * (cz ? zw2 : zw1);
              ti = (cz ? t1 : t0) + cx + cy * a.nix;
            }
            tile_add(thi_r + ti, tlo_r + ti, __float2int_rz(w * srs));
            tile_add(thi_i + ti, tlo_i + ti, __float2int_rz(w * sis));
          }
        } else {
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          if (c >= nc) break;
          float w;
          int64_t node;
          int plane;
          if (ONED) {
            plane = (c == 0) ? pz0 : pz1;
            w = (c == 0) ? zw1 : zw2;
            node = 0;
          } else {
            const int cx = c & 1, cy = (c >> 1) & 1, cz = c >> 2;
            w = (cx ? x2 : x1) * (cy ? y2 : y1) * (cz ? zw2 : zw1);
            plane = cz ? pz1 : pz0;
            node = b0 + cx + (int64_t)cy * a.nix;
          }
          const float vr = w * sr, vi = w * si;
          int tp = plane - pzlo;
          if (a.periodic && tp < 0) tp += (int)a.npl;
          if (a.tile && tp >= 0 && tp < TP && fabsf(vr) < a.tile_vmax &&
              fabsf(vi) < a.tile_vmax) {
            const int ti = tp * ntr + (int)node;
            tile_add(thi_r + ti, tlo_r + ti, f2fix(vr, a.fix_scale));
            tile_add(thi_i + ti, tlo_i + ti, f2fix(vi, a.fix_scale));
          } else {
            global_add(a.acc + (int64_t)plane * ntr + node, make_float2(vr, vi));
          }
        }
        }
      }
    }
    if (!a.coupling) {
      fr = 0.f;
      fi = 0.f;
    }

    float k[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    double kz = 0.0;
    if (a.electrons_evolve) {
      float bx, by, bz;
      const StageCoefF *tc =
          a.coef_tab ? (const StageCoefF *)a.coef_tab + (*a.step_ctr) * 4 + (STAGE - 1) : nullptr;
      bfield_f(tc ? tc->bf : a.bf, X, Y, bx, by, bz);
      const float n2col = tc ? tc->n2col : a.n2col, kn2col = tc ? tc->kn2col : a.kn2col;
      const float ep = p2f * a.eta_k2;
      const float cz = kn2col * qrG * bz;
      kz = p2;
      k[0] = a.dxc * qrG * PX;
      k[1] = -(a.dxc * qrG * PY);
      k[3] = a.sInv2rho * (n2col * by - ep * fr) + cz * PY;
      k[4] = a.sInv2rho * (n2col * bx - ep * fi) - cz * PX;
      k[5] = -(a.rho2 * qrG * (PX * fr + PY * fi));
    }
    constexpr int kF[5] = {0, 1, 3, 4, 5};
    if (STAGE == 1) {
#pragma unroll
      for (int t = 0; t < 5; ++t) a.kout_f[kF[t]][i] = k[kF[t]];
      a.kout_z[i] = kz;
    } else if (STAGE == 2) {
#pragma unroll
      for (int t = 0; t < 5; ++t) a.kacc_f[kF[t]][i] = k[kF[t]];
      a.kacc_z[i] = kz;
    } else if (STAGE == 3) {
#pragma unroll
      // k2 is read again here rather than kept live through the body (the
      // kernel runs at 40 registers)
      for (int t = 0; t < 5; ++t) {
        a.kout_f[kF[t]][i] = k[kF[t]];
        a.kacc_f[kF[t]][i] = a.kin_f[kF[t]][i] + k[kF[t]];
      }
      a.kout_z[i] = kz;
      a.kacc_z[i] = a.kin_z[i] + kz;
    } else {
      // y + h/6 (k1 + k4 + 2 (k2 + k3)): the slope sum in FP32, the update in
      // FP64 on the state read again (not kept live through the body)
      const double y0[6] = {a.x[i], a.y[i], a.z2[i], a.px[i], a.py[i], a.gam[i]};
#pragma unroll
      for (int t = 0; t < 5; ++t) {
        const int j = kF[t];
        const float sum = a.k1_f[j][i] + k[j] + 2.f * a.kacc_f[j][i];
        a.ynext[j][i] = fma(a.h6, f2d(sum), y0[j]);
      }
      a.ynext[2][i] = fma(a.h6, a.k1_z[i] + kz + 2.0 * a.kacc_z[i], y0[2]);
    }
  }

  if (a.tile) {
    __syncthreads();
    if (pzlo != INT_MAX) {
      // (hi 2^20 + lo) 2^-E in FP32 (the accumulators are FP32)
      const float shi = ldexpf(1.f, 20 - a.fixE), slo = ldexpf(1.f, -a.fixE);
      for (int t = threadIdx.x; t < tile_n; t += MX_THREADS) {
        int plane = pzlo + t / ntr;
        if (plane >= a.npl) {  // past the end: the periodic mesh's first planes
          if (!a.periodic) break;
          plane -= (int)a.npl;
        }
        const float2 v = make_float2(fmaf((float)thi_r[t], shi, (float)tlo_r[t] * slo),
                                     fmaf((float)thi_i[t], shi, (float)tlo_i[t] * slo));
        if (v.x != 0.f || v.y != 0.f) global_add(a.acc + (int64_t)plane * ntr + (t % ntr), v);
      }
    }
  }
}

// Every input of the node is loaded before the first store (the arrays
// could alias as far as the compiler knows), so a thread waits for HBM once.
template <int STAGE>
__device__ __forceinline__ void node_update_mixed(const MixNodeArgs &a, const int64_t n) {
  const float2 d = a.acc[n];
  const float2 w = a.w[n];
  float2 e12 = make_float2(0.f, 0.f), d0 = make_float2(0.f, 0.f);
  if (STAGE == 3 || STAGE == 4) e12 = a.d12[n];
  if (STAGE == 4) d0 = a.d0[n];
  const unsigned st = (STAGE == 4) ? *a.status : 0u;
  // a non-finite field value stops the step before stage 4 commits
  if (STAGE == 1 && !isfinite(w.x + w.y)) atomicOr(const_cast<unsigned int *>(a.status), ST_NOT_FINITE);
  if (STAGE == 1) {
    a.d0[n] = d;
    a.as[n] = make_float2(w.x + a.coef * d.x, w.y + a.coef * d.y);
  } else if (STAGE == 2) {
    a.d12[n] = d;
    a.as[n] = make_float2(w.x + a.coef * d.x, w.y + a.coef * d.y);
  } else if (STAGE == 3) {
    a.as[n] = make_float2(w.x + a.coef * d.x, w.y + a.coef * d.y);
    a.d12[n] = make_float2(e12.x + d.x, e12.y + d.y);
  } else {
    if (st == 0u)
      a.w[n] = make_float2(w.x + a.h6 * (d0.x + d.x + 2.f * e12.x), w.y + a.h6 * (d0.y + d.y + 2.f * e12.y));
  }
  // The accumulator is cleared last, with zeros computed from the loaded
  // value (its sign bit alone: a signed zero, also for a NaN left by a
  // failed step): a store of a constant to an address whose load is still in
  // flight is several times slower on this GPU than the same store issued
  // once the load has returned.
  a.acc[n] = make_float2(__int_as_float(__float_as_int(d.x) & (int)0x80000000),
                         __int_as_float(__float_as_int(d.y) & (int)0x80000000));
}

template <int STAGE>
__global__ void __launch_bounds__(256) k_nodes_mixed(const MixNodeArgs a) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.n) return;
  node_update_mixed<STAGE>(a, n);
  if (STAGE == 4 && a.step_ctr && n == 0) *a.step_ctr += 1;
}

template <int STAGE, bool ONED, int TP = MX_TILE_PLANES>
__global__ void __launch_bounds__(MX_THREADS, 3) k_stage_mixed(const MixArgs a) {
  extern __shared__ __align__(16) float tile[];
  __shared__ int s_pzlo;
  const int64_t i0 = (int64_t)blockIdx.x * (MX_THREADS * a.ppt);
  mixed_block<STAGE, ONED, TP>(a, i0, min(a.np, i0 + (int64_t)MX_THREADS * a.ppt), a.ppt, tile,
                               s_pzlo);
}

// Batched mixed stage over (instance, macroparticle range) tiles of at most
// MX_THREADS * MX_PPT macroparticles; the arguments of each tile's instance
// are staged in shared memory.
template <int STAGE>
__global__ void __launch_bounds__(MX_THREADS, 3) k_stage_mixed_batch(const MixArgs *__restrict__ args,
                                                                  const BatchTile *__restrict__ tiles,
                                                                  const int ntiles) {
  extern __shared__ __align__(16) float tile[];
  __shared__ int s_pzlo;
  __shared__ __align__(16) unsigned long long sa_raw[sizeof(MixArgs) / 8];
  static_assert(sizeof(MixArgs) % 8 == 0, "MixArgs is copied as 64-bit words");
  const MixArgs &sa = *reinterpret_cast<const MixArgs *>(sa_raw);
  int cur = -1;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BatchTile tl = tiles[t];
    __syncthreads();  // the previous range is done with the arguments and the tile
    if (tl.inst != cur) {
      const unsigned long long *src = reinterpret_cast<const unsigned long long *>(args + tl.inst);
      for (int k = threadIdx.x; k < (int)(sizeof(MixArgs) / 8); k += MX_THREADS) sa_raw[k] = src[k];
      cur = tl.inst;
      __syncthreads();
    }
    const int ppt = (int)((tl.end - tl.begin + MX_THREADS - 1) / MX_THREADS);
    mixed_block<STAGE, false, MX_TILE_PLANES>(sa, tl.begin, tl.end, ppt, tile, s_pzlo);
  }
}

// Batched mixed node update over (instance, node range) tiles.
template <int STAGE>
__global__ void __launch_bounds__(256) k_nodes_mixed_batch(const MixNodeArgs *__restrict__ args,
                                                           const BatchTile *__restrict__ tiles,
                                                           const int ntiles, int *step_ctr) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BatchTile tl = tiles[t];
    const MixNodeArgs a = args[tl.inst];
    for (int64_t n = tl.begin + threadIdx.x; n < tl.end; n += blockDim.x) node_update_mixed<STAGE>(a, n);
  }
  if (STAGE == 4 && step_ctr && blockIdx.x == 0 && threadIdx.x == 0) *step_ctr += 1;
}


}  // namespace

// FP32 stage-coefficient entries of one step (advances the taper state)
void pf_step_coefficients_f(pf_handle *h, double szl, double hstep, void *out_) {
  StageCoefF *out = (StageCoefF *)out_;
  const double hh = hstep * 0.5, szh = szl + hh;
  const double stage_sz[4] = {szl, szh, szh, szl + hstep};
  for (int s = 0; s < 4; ++s) {
    double n2col;
    int place;
    pf_taper_stage(h, stage_sz[s], &n2col, &place);
    BFieldCoef bf;
    pf_stage_coefficients(h->p, stage_sz[s], n2col, place, &bf);
    out[s].bf = to_float(bf);
    out[s].n2col = (float)n2col;
    out[s].kn2col = (float)(h->p.kappa * n2col);
  }
}

size_t pf_step_coefficients_f_bytes() { return 4 * sizeof(StageCoefF); }

// Stage arguments of the handle's state that do not change between stages.
static void fill_mix_args(pf_handle *h, MixArgs &a, double hstep) {
  const pf_params &p = h->p;
  memset(&a, 0, sizeof(a));
  a.chi_f = h->chi_f;
  a.np = h->np;
  a.h6 = hstep / 6.0;
  a.acc = (float2 *)h->acc32;
  a.nix = h->nix;
  a.niy = h->niy;
  a.npl = h->npl;
  a.nz2 = p.nz2;
  a.periodic = (p.mesh_type == PF_MESH_PERIODIC);
  a.one_d = p.one_d;
  a.npl_f = (float)h->npl;
  a.inv_npl_f = 1.0f / (float)h->npl;
  a.halfx = ((double)(h->nix - 1) / 2.0) * p.dx;
  a.halfy = ((double)(h->niy - 1) / 2.0) * p.dy;
  a.inv_dx = 1.0 / p.dx;
  a.inv_dy = 1.0 / p.dy;
  a.inv_dz2 = 1.0 / p.dz2;
  a.inv_dx_f = (float)(1.0 / p.dx);
  a.inv_dy_f = (float)(1.0 / p.dy);
  a.hx_dx = (float)(a.halfx / p.dx);
  a.hy_dy = (float)(a.halfy / p.dy);
  a.eta_f = (float)p.eta;
  a.inv_dz2_f = (float)(1.0 / p.dz2);
  a.aw2g = (p.aw * p.aw) / (p.gamma_r * p.gamma_r);
  a.g02 = 1.0 / (p.gamma_r * p.gamma_r);
  {
    // 1/sqrt(1-u) - 1 = sum_k C(2k,k)/4^k u^k, k >= 1
    const double cb[7] = {1.0 / 2.0, 3.0 / 8.0, 5.0 / 16.0, 35.0 / 128.0, 63.0 / 256.0,
                          231.0 / 1024.0, 429.0 / 2048.0};
    for (int k = 0; k < 7; ++k) a.ser[k] = cb[k] / p.eta;
    a.ser_r1 = (float)(cb[1] / cb[0]);
    a.ser_r2 = (float)(cb[2] / cb[0]);
  }
  a.inv_g02 = 1.0 / (p.gamma_r * p.gamma_r);
  a.aw2 = p.aw * p.aw;
  a.inv_eta = 1.0 / p.eta;
  a.eta = p.eta;
  a.inv_dV3 = (float)(1.0 / (p.dx * p.dy * p.dz2));
  a.sInv2rho = (float)(1.0 / (2.0 * p.rho));
  a.dxc = (float)(2.0 * p.rho * p.kappa / sqrt(p.eta));
  a.eta_k2 = (float)(p.eta / (p.kappa * p.kappa));
  a.rho2 = (float)(2.0 * p.rho);
  a.field_evolve = p.field_evolve;
  a.electrons_evolve = p.electrons_evolve;
  a.coupling = p.coupling;
  a.status = h->d_status;
  {
    // |chi/dV3 (1 + eta p2)/Gamma p w| below 16 chi_max/dV3 for |p| (1+eta p2)/Gamma < 16;
    // the rest goes to HBM
    const double vmax = 16.0 * h->chi_max / (p.dx * p.dy * p.dz2);
    int e = 0;
    frexp(vmax > 0.0 ? vmax : 1.0, &e);  // vmax < 2^e
    a.fixE = 31 - e;
    a.fix_scale = (float)ldexp(1.0, a.fixE);
    a.tile_vmax = (float)ldexp(1.0, e);
  }
  // the tile needs a window that fits shared memory and a scale 2^E that is
  // a normal float (beams with any usable charge weights)
  a.tile = (pf_mixed_tile_smem(h) > 0 && a.fixE >= -126 && a.fixE <= 127) ? 1 : 0;
}

// Per-stage fields: the state and slope arrays of stage s for buffer cur.
static void mix_stage_pointers(pf_handle *h, MixArgs &a, int s, int cur, double hstep) {
  const double hh = hstep * 0.5;
  const double stage_c[4] = {0.0, hh, hh, hstep};
  const int nxt = cur ^ 1;
  a.x = h->y[cur][0];
  a.y = h->y[cur][1];
  a.z2 = h->y[cur][2];
  a.px = h->y[cur][3];
  a.py = h->y[cur][4];
  a.gam = h->y[cur][5];
  a.base4 = h->base4;
  a.cstate = stage_c[s - 1];
  a.cstate_f = (float)stage_c[s - 1];
  a.as = (const float2 *)((s == 1) ? h->w32 : h->as32);
  // the slope arrays are FP64-sized; in this mode they hold FP32 values,
  // except the z2 slope
  double *const *kin = (s == 2) ? h->k1 : (s == 3) ? h->ka : (s == 4) ? h->kb : nullptr;
  double *const *kout = (s == 1) ? h->k1 : (s == 3) ? h->kb : nullptr;
  double *const *kacc = (s >= 2) ? h->ka : nullptr;
  for (int j = 0; j < 6; ++j) {
    a.kin_f[j] = kin ? (const float *)kin[j] : nullptr;
    a.kout_f[j] = kout ? (float *)kout[j] : nullptr;
    a.kacc_f[j] = kacc ? (float *)kacc[j] : nullptr;
    a.k1_f[j] = (const float *)h->k1[j];
    a.ynext[j] = h->y[nxt][j];
  }
  a.kin_z = kin ? kin[2] : nullptr;
  a.kout_z = kout ? kout[2] : nullptr;
  a.kacc_z = kacc ? kacc[2] : nullptr;
  a.k1_z = h->k1[2];
}

static void fill_mix_nodes(pf_handle *h, MixNodeArgs &n, int s, double hstep) {
  memset(&n, 0, sizeof(n));
  n.n = h->nwin;
  n.acc = (float2 *)h->acc32;
  n.w = (float2 *)h->w32;
  n.as = (float2 *)h->as32;
  n.d0 = (float2 *)h->d0_32;
  n.d12 = (float2 *)h->d12_32;
  n.h6 = (float)(hstep / 6.0);
  n.coef = (float)((s == 3) ? hstep : hstep * 0.5);
  n.status = h->d_status;
}

// shared bytes of the 3-plane tile (0: it does not fit); the batched kernel
// and the default of the single-instance kernel
size_t pf_mixed_tile_smem(const pf_handle *h) {
  const size_t bytes = (size_t)4 * MX_TILE_PLANES * h->nix * h->niy * sizeof(int);
  return bytes <= 96 * 1024 ? bytes : 0;
}

// planes of the single-instance kernel's tile: 8 where they fit
// MX_TILE_BYTES (small windows, such as the 21 x 21 of the config-1 mesh:
// a bunched beam's blocks spread over several planes), else 3
static int mixed_tile_planes(const pf_handle *h) {
  const size_t per_plane = (size_t)4 * h->nix * h->niy * sizeof(int);
  return (size_t)MX_TILE_PLANES_WIDE * per_plane <= MX_TILE_BYTES ? MX_TILE_PLANES_WIDE
                                                                 : MX_TILE_PLANES;
}

size_t pf_mixed_stage_args_bytes() { return sizeof(MixArgs); }
size_t pf_mixed_node_args_bytes() { return sizeof(MixNodeArgs); }

void pf_mixed_fill_stage(pf_handle *h, int stage, int cur, double hstep, int tile,
                         const void *coef_tab, const int *step_ctr, unsigned *status, void *out) {
  MixArgs a;
  fill_mix_args(h, a, hstep);
  mix_stage_pointers(h, a, stage, cur, hstep);
  a.tile = (tile && a.tile) ? 1 : 0;
  a.ppt = MX_PPT;
  a.coef_tab = coef_tab;
  a.step_ctr = step_ctr;
  a.status = status;
  memcpy(out, &a, sizeof(a));
}

void pf_mixed_fill_nodes(pf_handle *h, int stage, double hstep, unsigned *status, void *out) {
  MixNodeArgs n;
  fill_mix_nodes(h, n, stage, hstep);
  n.status = status;
  memcpy(out, &n, sizeof(n));
}

static cudaError_t mixed_attrs() {
  static PfDeviceOnce attr_once;  // the attribute is per device
  return pf_device_once(attr_once, [] {
    cudaError_t attr = cudaSuccess;
    // the tile may exceed the 48 KB default of dynamic shared memory
    const void *fns[] = {(const void *)k_stage_mixed<1, false>, (const void *)k_stage_mixed<2, false>,
                         (const void *)k_stage_mixed<3, false>, (const void *)k_stage_mixed<4, false>,
                         (const void *)k_stage_mixed<1, true>,  (const void *)k_stage_mixed<2, true>,
                         (const void *)k_stage_mixed<3, true>,  (const void *)k_stage_mixed<4, true>,
                         (const void *)k_stage_mixed<1, false, MX_TILE_PLANES_WIDE>,
                         (const void *)k_stage_mixed<2, false, MX_TILE_PLANES_WIDE>,
                         (const void *)k_stage_mixed<3, false, MX_TILE_PLANES_WIDE>,
                         (const void *)k_stage_mixed<4, false, MX_TILE_PLANES_WIDE>,
                         (const void *)k_stage_mixed<1, true, MX_TILE_PLANES_WIDE>,
                         (const void *)k_stage_mixed<2, true, MX_TILE_PLANES_WIDE>,
                         (const void *)k_stage_mixed<3, true, MX_TILE_PLANES_WIDE>,
                         (const void *)k_stage_mixed<4, true, MX_TILE_PLANES_WIDE>,
                         (const void *)k_stage_mixed_batch<1>,  (const void *)k_stage_mixed_batch<2>,
                         (const void *)k_stage_mixed_batch<3>,  (const void *)k_stage_mixed_batch<4>};
    for (const void *f : fns) {
      const cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
      if (e != cudaSuccess) attr = e;
    }
    return attr;
  });
}

cudaError_t pf_mixed_stage_batch(cudaStream_t st, int stage, const void *args,
                                 const BatchTile *tiles, int ntiles, int grid, size_t smem) {
  const cudaError_t e = mixed_attrs();
  if (e != cudaSuccess) return e;
  if (ntiles <= 0) return cudaSuccess;
  if (grid < 0) grid = pf_resident_blocks((const void *)k_stage_mixed_batch<1>, MX_THREADS, smem);
  const unsigned g = (unsigned)(grid == 0 ? ntiles : std::max(1, std::min(grid, ntiles)));
  const MixArgs *a = (const MixArgs *)args;
  switch (stage) {
    case 1: k_stage_mixed_batch<1><<<g, MX_THREADS, smem, st>>>(a, tiles, ntiles); break;
    case 2: k_stage_mixed_batch<2><<<g, MX_THREADS, smem, st>>>(a, tiles, ntiles); break;
    case 3: k_stage_mixed_batch<3><<<g, MX_THREADS, smem, st>>>(a, tiles, ntiles); break;
    default: k_stage_mixed_batch<4><<<g, MX_THREADS, smem, st>>>(a, tiles, ntiles); break;
  }
  return cudaGetLastError();
}

cudaError_t pf_mixed_nodes_batch(cudaStream_t st, int stage, const void *args,
                                 const BatchTile *tiles, int ntiles, int grid, int threads,
                                 int *step_ctr) {
  if (ntiles <= 0) return cudaSuccess;
  if (grid < 0) grid = pf_resident_blocks((const void *)k_nodes_mixed_batch<1>, threads, 0);
  const unsigned g = (unsigned)(grid == 0 ? ntiles : std::max(1, std::min(grid, ntiles)));
  const MixNodeArgs *a = (const MixNodeArgs *)args;
  switch (stage) {
    case 1: k_nodes_mixed_batch<1><<<g, threads, 0, st>>>(a, tiles, ntiles, nullptr); break;
    case 2: k_nodes_mixed_batch<2><<<g, threads, 0, st>>>(a, tiles, ntiles, nullptr); break;
    case 3: k_nodes_mixed_batch<3><<<g, threads, 0, st>>>(a, tiles, ntiles, nullptr); break;
    default: k_nodes_mixed_batch<4><<<g, threads, 0, st>>>(a, tiles, ntiles, step_ctr); break;
  }
  return cudaGetLastError();
}

// Macroparticles per thread of the single-instance stage kernel: six (3072
// per block), eight for beams dense along z2 (a block then still spans a
// fraction of a plane; six and eight measured best for the config-2 and the
// config-1-mesh 2^24 beams), fewer when the beam is too small to give every
// SM two blocks.
static int mixed_ppt(const pf_handle *h) {
  const int64_t per_plane = h->np / std::max<int64_t>(1, (int64_t)h->npl);
  const int64_t want = (per_plane >= (int64_t)16 * MX_THREADS) ? MX_PPT : 6;
  int64_t ppt = std::max<int64_t>(1, std::min<int64_t>(want, h->np / ((int64_t)pf_sm_count() * 2 * MX_THREADS)));
  // fewer macroparticles per thread when the grid's waves of resident blocks
  // (three per SM) would be less than 85 % full: 2^22 macroparticles at 8
  // per thread made 2.25 waves, at 6 they make 3.0
  const int64_t slots = (int64_t)3 * pf_sm_count(), per = (int64_t)MX_THREADS;
  const int64_t nb = (h->np + per * ppt - 1) / (per * ppt);
  const int64_t waves = std::max<int64_t>(1, (nb + slots - 1) / slots);
  if (nb < (int64_t)(0.85 * (double)(waves * slots)))
    ppt = std::max<int64_t>(1, std::min<int64_t>(ppt, (h->np + waves * slots * per - 1) / (waves * slots * per)));
  return (int)ppt;
}

namespace {
// Macroparticles of the stage kernel's blocks (as the kernel cuts them)
// whose z2 cell lies outside the fast path of their block's shared tile:
// the lowest plane the block starts from is estimated as the kernel does,
// and a macroparticle counts when its two planes are not both in the tile.
__global__ void __launch_bounds__(MX_THREADS) k_order_misses(const double *z2, int64_t np, int ppt,
                                                             double inv_dz2, int npl, int periodic,
                                                             int tp, unsigned *count) {
  __shared__ int s_lo;
  __shared__ unsigned s_cnt;
  const int64_t i0 = (int64_t)blockIdx.x * MX_THREADS * ppt;
  const int64_t i1 = min(np, i0 + (int64_t)MX_THREADS * ppt);
  if (threadIdx.x == 0) {
    s_lo = INT_MAX;
    s_cnt = 0;
  }
  __syncthreads();
  long long kmin = LLONG_MAX;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += MX_THREADS)
    kmin = min(kmin, __double_as_longlong(z2[i]));
  for (int o = 16; o > 0; o >>= 1) kmin = min(kmin, __shfl_xor_sync(0xffffffffu, kmin, o));
  if ((threadIdx.x & 31) == 0 && kmin != LLONG_MAX) {
    double fz = floor(__longlong_as_double(kmin) * inv_dz2);
    if (fabs(fz) < 1.0e9) {
      if (periodic) fz = fmax(fz - npl * floor(fz / npl), 0.0);
      atomicMin(&s_lo, (int)fz);
    }
  }
  __syncthreads();
  unsigned miss = 0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += MX_THREADS) {
    double fz = floor(z2[i] * inv_dz2);
    if (!(fabs(fz) < 1.0e9)) {
      ++miss;
      continue;
    }
    if (periodic) fz = fz - npl * floor(fz / npl);
    const int t = (int)fz - s_lo;
    if (!(t >= 0 && t + 1 < tp && !(periodic && (int)fz + 1 == npl))) ++miss;
  }
  for (int o = 16; o > 0; o >>= 1) miss += __shfl_xor_sync(0xffffffffu, miss, o);
  if ((threadIdx.x & 31) == 0 && miss) atomicAdd(&s_cnt, miss);
  __syncthreads();
  if (threadIdx.x == 0 && s_cnt) atomicAdd(count, s_cnt);
}
}  // namespace

// Fraction of the macroparticles (current state) whose deposits would miss
// their stage block's shared tile; 0 when the stage kernel uses no tile.
int pf_mixed_order_misses(pf_handle *h, double *frac) {
  *frac = 0.0;
  MixArgs a;
  fill_mix_args(h, a, 0.0);
  if (!a.tile || h->np == 0 || h->p.one_d) return PF_OK;
  const int ppt = mixed_ppt(h);
  const int64_t per_block = (int64_t)MX_THREADS * ppt;
  const unsigned g = (unsigned)((h->np + per_block - 1) / per_block);
  unsigned *cnt = h->d_status + 1;
  PF_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned), h->stream));
  k_order_misses<<<g, MX_THREADS, 0, h->stream>>>(h->y[h->cur][2], h->np, ppt, 1.0 / h->p.dz2,
                                                  (int)h->npl, h->p.mesh_type == PF_MESH_PERIODIC,
                                                  mixed_tile_planes(h), cnt);
  PF_LAUNCHED(h);
  PF_CUDA(cudaMemcpyAsync(h->h_status + 1, cnt, sizeof(unsigned), cudaMemcpyDeviceToHost,
                          h->stream));
  PF_CUDA(cudaStreamSynchronize(h->stream));
  *frac = (double)h->h_status[1] / (double)h->np;
  return PF_OK;
}

// k_stage_mixed<stage> over pg blocks in the tile form the handle's window takes
static void launch_mixed_stage(pf_handle *h, int s, const MixArgs &a, unsigned pg, size_t smem,
                               bool wide, bool oned) {
#define PF_MIX_CASE(S)                                                                 \
  case S:                                                                              \
    if (wide) {                                                                        \
      if (oned) k_stage_mixed<S, true, MX_TILE_PLANES_WIDE><<<pg, MX_THREADS, smem, h->stream>>>(a); \
      else k_stage_mixed<S, false, MX_TILE_PLANES_WIDE><<<pg, MX_THREADS, smem, h->stream>>>(a);     \
    } else if (oned) k_stage_mixed<S, true><<<pg, MX_THREADS, smem, h->stream>>>(a);   \
    else k_stage_mixed<S, false><<<pg, MX_THREADS, smem, h->stream>>>(a);              \
    break;
  switch (s) {
    PF_MIX_CASE(1)
    PF_MIX_CASE(2)
    PF_MIX_CASE(3)
    PF_MIX_CASE(4)
  }
#undef PF_MIX_CASE
}

// shared bytes of the stage kernel's tile for the handle's window, and
// whether it is the eight-plane form
static size_t mixed_stage_smem(const pf_handle *h, const MixArgs &a, bool *wide) {
  *wide = a.tile && mixed_tile_planes(h) == MX_TILE_PLANES_WIDE;
  return !a.tile ? 0
         : *wide ? (size_t)4 * MX_TILE_PLANES_WIDE * h->nix * h->niy * sizeof(int)
                 : pf_mixed_tile_smem(h);
}

int pf_rk4_mixed(pf_handle *h, double szl, double hstep, unsigned int *status_out) {
  const pf_params &p = h->p;
  const double hh = hstep * 0.5, szh = szl + hh;
  const double stage_sz[4] = {szl, szh, szh, szl + hstep};
  const int nxt = h->cur ^ 1;
  // status_out == nullptr: enqueue only (a step of an asynchronous block;
  // the caller clears the status word once per block and reads it after)
  if (status_out) PF_CUDA(cudaMemsetAsync(h->d_status, 0, sizeof(unsigned int), h->stream));

  MixArgs a;
  fill_mix_args(h, a, hstep);
  if (h->capturing) {
    a.coef_tab = h->coef_dev;
    a.step_ctr = h->step_ctr;
  }
  bool wide = false;
  const size_t smem = mixed_stage_smem(h, a, &wide);
  MixNodeArgs n;
  fill_mix_nodes(h, n, 1, hstep);
  if (h->capturing) n.step_ctr = h->step_ctr;

  PF_CUDA(mixed_attrs());
  a.ppt = mixed_ppt(h);
  const int64_t per_block = (int64_t)MX_THREADS * a.ppt;
  const unsigned pg = (unsigned)std::max<int64_t>(1, (h->np + per_block - 1) / per_block);
  const unsigned ng = (unsigned)std::max<int64_t>(1, (h->nwin + 255) / 256);
  const bool oned = p.one_d != 0;
  for (int s = 1; s <= 4; ++s) {
    double n2col;
    int place;
    pf_taper_stage(h, stage_sz[s - 1], &n2col, &place);
    BFieldCoef bf;
    pf_stage_coefficients(p, stage_sz[s - 1], n2col, place, &bf);
    a.bf = to_float(bf);
    a.n2col = (float)n2col;
    a.kn2col = (float)(p.kappa * n2col);
    mix_stage_pointers(h, a, s, h->cur, hstep);
    if (h->np > 0) {
      pf_prof_begin(h, PROF_STAGE);
      launch_mixed_stage(h, s, a, pg, smem, wide, oned);
      pf_prof_end(h);
      PF_LAUNCHED(h);
    }
    n.coef = (float)((s == 3) ? hstep : hh);
    pf_prof_begin(h, PROF_NODES);
    switch (s) {
      case 1: k_nodes_mixed<1><<<ng, 256, 0, h->stream>>>(n); break;
      case 2: k_nodes_mixed<2><<<ng, 256, 0, h->stream>>>(n); break;
      case 3: k_nodes_mixed<3><<<ng, 256, 0, h->stream>>>(n); break;
      default: k_nodes_mixed<4><<<ng, 256, 0, h->stream>>>(n); break;
    }
    pf_prof_end(h);
    PF_LAUNCHED(h);
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

namespace {
// FP64 split window field <-> the interleaved complex-float window, as
// pf_set_window_field and pf_get_window_field convert it
__global__ void k_win_in_c32(float2 *w, const double *re, const double *im, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) w[t] = make_float2((float)re[t], (float)im[t]);
}
__global__ void k_win_out_c32(const float2 *w, double *re, double *im, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) {
    const float2 v = w[t];
    re[t] = (double)v.x;
    im[t] = (double)v.y;
  }
}
}  // namespace

// The mixed step with the driver's arrays in host memory: the copies of
// pf_rk4_fp64_host (the window field first, the particles by chunks that
// stage 1 starts on as they arrive, stage 4's output leaving chunk by
// chunk), the window field converted to and from its complex-float form
// on the device through the staging buffer.
int pf_rk4_mixed_host(pf_handle *h, double szl, double hstep, double *const host[6], double *wre,
                      double *wim, unsigned int *status_out) {
  const pf_params &p = h->p;
  const double hh = hstep * 0.5, szh = szl + hh;
  const double stage_sz[4] = {szl, szh, szh, szl + hstep};
  const int cur = h->cur, nxt = cur ^ 1;
  const int64_t np = h->np, nw = h->nwin;
  const int64_t chunk = std::max<int64_t>((int64_t)1 << 20, (np + 15) / 16);
  const int nch = (int)std::max<int64_t>(1, (np + chunk - 1) / chunk);
  if (!h->copy_stream)
    PF_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
  while ((int)h->copy_events.size() < 2 * nch + 1) {
    cudaEvent_t e;
    PF_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    h->copy_events.push_back(e);
  }
  if (!h->staging) PF_CUDA(cudaMalloc(&h->staging, 2 * sizeof(double) * (size_t)h->nouter));
  cudaEvent_t *ev_in = h->copy_events.data(), *ev_out = ev_in + nch, ev_w = ev_in[2 * nch];
  cudaStream_t cs = h->copy_stream, st = h->stream;
  const size_t wb = (size_t)nw * sizeof(double);
  const unsigned gw = (unsigned)std::max<int64_t>(1, (nw + 255) / 256);

  PF_CUDA(cudaMemsetAsync(h->d_status, 0, sizeof(unsigned int), st));
  PF_CUDA(cudaMemcpyAsync(h->staging, wre, wb, cudaMemcpyHostToDevice, st));
  PF_CUDA(cudaMemcpyAsync(h->staging + nw, wim, wb, cudaMemcpyHostToDevice, st));
  k_win_in_c32<<<gw, 256, 0, st>>>((float2 *)h->w32, h->staging, h->staging + nw, nw);
  PF_LAUNCHED(h);
  for (int c = 0; c < nch; ++c) {
    const int64_t off = c * chunk, len = std::min(chunk, np - off);
    for (int j = 0; j < 6; ++j)
      PF_CUDA(cudaMemcpyAsync(h->y[cur][j] + off, host[j] + off, (size_t)len * sizeof(double),
                              cudaMemcpyHostToDevice, cs));
    PF_CUDA(cudaEventRecord(ev_in[c], cs));
  }

  MixArgs a;
  fill_mix_args(h, a, hstep);
  bool wide = false;
  const size_t smem = mixed_stage_smem(h, a, &wide);
  MixNodeArgs n;
  fill_mix_nodes(h, n, 1, hstep);
  PF_CUDA(mixed_attrs());
  a.ppt = mixed_ppt(h);
  const int64_t per_block = (int64_t)MX_THREADS * a.ppt;
  const bool oned = p.one_d != 0;
  // the stage arguments of macroparticles [off, off + len)
  auto range = [](const MixArgs &b, int64_t off, int64_t len) {
    MixArgs r = b;
    r.x += off;
    r.y += off;
    r.z2 += off;
    r.px += off;
    r.py += off;
    r.gam += off;
    r.chi_f += off;
    r.base4 += off;
    for (int j = 0; j < 6; ++j) {
      if (r.kin_f[j]) r.kin_f[j] += off;
      if (r.kout_f[j]) r.kout_f[j] += off;
      if (r.kacc_f[j]) r.kacc_f[j] += off;
      if (r.k1_f[j]) r.k1_f[j] += off;
      if (r.ynext[j]) r.ynext[j] += off;
    }
    if (r.kin_z) r.kin_z += off;
    if (r.kout_z) r.kout_z += off;
    if (r.kacc_z) r.kacc_z += off;
    if (r.k1_z) r.k1_z += off;
    r.np = len;
    return r;
  };
  for (int s = 1; s <= 4; ++s) {
    double n2col;
    int place;
    pf_taper_stage(h, stage_sz[s - 1], &n2col, &place);
    BFieldCoef bf;
    pf_stage_coefficients(p, stage_sz[s - 1], n2col, place, &bf);
    a.bf = to_float(bf);
    a.n2col = (float)n2col;
    a.kn2col = (float)(p.kappa * n2col);
    mix_stage_pointers(h, a, s, cur, hstep);
    if (np > 0) {
      if (s == 1 || s == 4) {
        for (int c = 0; c < nch; ++c) {
          const int64_t off = c * chunk, len = std::min(chunk, np - off);
          if (s == 1) PF_CUDA(cudaStreamWaitEvent(st, ev_in[c], 0));
          const MixArgs r = range(a, off, len);
          launch_mixed_stage(h, s, r, (unsigned)((len + per_block - 1) / per_block), smem, wide,
                             oned);
          PF_LAUNCHED(h);
          if (s == 4) {
            PF_CUDA(cudaEventRecord(ev_out[c], st));
            PF_CUDA(cudaStreamWaitEvent(cs, ev_out[c], 0));
            for (int j = 0; j < 6; ++j)
              PF_CUDA(cudaMemcpyAsync(host[j] + off, h->y[nxt][j] + off,
                                      (size_t)len * sizeof(double), cudaMemcpyDeviceToHost, cs));
          }
        }
      } else {
        launch_mixed_stage(h, s, a, (unsigned)std::max<int64_t>(1, (np + per_block - 1) / per_block),
                           smem, wide, oned);
        PF_LAUNCHED(h);
      }
    }
    n.coef = (float)((s == 3) ? hstep : hh);
    switch (s) {
      case 1: k_nodes_mixed<1><<<gw, 256, 0, st>>>(n); break;
      case 2: k_nodes_mixed<2><<<gw, 256, 0, st>>>(n); break;
      case 3: k_nodes_mixed<3><<<gw, 256, 0, st>>>(n); break;
      default: k_nodes_mixed<4><<<gw, 256, 0, st>>>(n); break;
    }
    PF_LAUNCHED(h);
  }
  k_win_out_c32<<<gw, 256, 0, st>>>((const float2 *)h->w32, h->staging, h->staging + nw, nw);
  PF_LAUNCHED(h);
  PF_CUDA(cudaMemcpyAsync(wre, h->staging, wb, cudaMemcpyDeviceToHost, st));
  PF_CUDA(cudaMemcpyAsync(wim, h->staging + nw, wb, cudaMemcpyDeviceToHost, st));
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
  for (int j = 0; j < 6; ++j)
    PF_CUDA(cudaMemcpyAsync(host[j], h->y[cur][j], (size_t)np * sizeof(double),
                            cudaMemcpyDeviceToHost, st));
  PF_CUDA(cudaStreamSynchronize(st));
  return PF_OK;
}

// One stage of the mixed step on explicit arrays (the adjoint's recorded
// forward): the stage roles and arithmetic of pf_rk4_mixed, the b-field and
// taper of position sz.
int pf_mixed_stage_rec(pf_handle *h, int stage, double hstep, double sz, const PfMixRec &r) {
  if (h->np == 0) return PF_OK;
  const pf_params &p = h->p;
  const double hh = hstep * 0.5;
  const double stage_c[4] = {0.0, hh, hh, hstep};
  MixArgs a;
  fill_mix_args(h, a, hstep);
  double n2col;
  int place;
  pf_taper_stage(h, sz, &n2col, &place);
  BFieldCoef bf;
  pf_stage_coefficients(p, sz, n2col, place, &bf);
  a.bf = to_float(bf);
  a.n2col = (float)n2col;
  a.kn2col = (float)(p.kappa * n2col);
  a.x = r.y[0];
  a.y = r.y[1];
  a.z2 = r.y[2];
  a.px = r.y[3];
  a.py = r.y[4];
  a.gam = r.y[5];
  a.base4 = h->base4;
  a.cstate = stage_c[stage - 1];
  a.cstate_f = (float)stage_c[stage - 1];
  a.as = (const float2 *)r.as;
  for (int j = 0; j < 6; ++j) {
    a.kin_f[j] = (const float *)r.kin[j];
    a.kout_f[j] = (float *)r.kout[j];
    a.kacc_f[j] = (float *)r.kacc[j];
    a.k1_f[j] = (const float *)r.k1[j];
    a.ynext[j] = r.ynext[j];
  }
  a.kin_z = (const double *)r.kin[2];
  a.kout_z = (double *)r.kout[2];
  a.kacc_z = (double *)r.kacc[2];
  a.k1_z = (const double *)r.k1[2];
  PF_CUDA(mixed_attrs());
  a.ppt = mixed_ppt(h);
  const int64_t per_block = (int64_t)MX_THREADS * a.ppt;
  const unsigned pg = (unsigned)std::max<int64_t>(1, (h->np + per_block - 1) / per_block);
  bool wide = false;
  const size_t smem = mixed_stage_smem(h, a, &wide);
  launch_mixed_stage(h, stage, a, pg, smem, wide, p.one_d != 0);
  PF_LAUNCHED(h);
  return PF_OK;
}

void pf_mixed_constants(pf_handle *h, PfMixConst *c) {
  MixArgs a;
  fill_mix_args(h, a, 0.0);
  c->aw2g = a.aw2g;
  c->g02 = a.g02;
  c->inv_eta = a.inv_eta;
  c->inv_dz2 = a.inv_dz2;
  for (int k = 0; k < 7; ++k) c->ser[k] = a.ser[k];
  c->ser_r1 = a.ser_r1;
  c->ser_r2 = a.ser_r2;
  c->inv_dx_f = a.inv_dx_f;
  c->inv_dy_f = a.inv_dy_f;
  c->hx_dx = a.hx_dx;
  c->hy_dy = a.hy_dy;
  c->eta_f = a.eta_f;
  c->inv_dV3 = a.inv_dV3;
  c->sInv2rho = a.sInv2rho;
  c->dxc = a.dxc;
  c->eta_k2 = a.eta_k2;
  c->rho2 = a.rho2;
}
