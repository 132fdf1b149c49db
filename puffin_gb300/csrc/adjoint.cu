// Adjoint of the interpolate-push-deposit-diffract step, with
// checkpoint-and-recompute, for the FP64 path and the mixed-precision path
// (the forward recorded with the handle's own stage kernels).
//
// Forward model: UndSection's loop (puffin/lib/undulator.f90:182-333) over
// nsteps RK4 steps with the diffraction schedule of pf_run, a piecewise-
// linear taper profile alpha(z) (pf_set_taper_profile), the initial field
// seed_amp * seed and the beam's energy chirp gamma += chirp (z2 - <z2>).
// Output: the pulse energy E = dx dy dz2 sum |A|^2 over the outer mesh (the
// unique z2 planes).  Reverse mode gives dE/d(alpha control points),
// dE/d(seed_amp) and dE/d(chirp).
//
// One RK4 step, particles y and window field W (rk4par,
// puffin_mpi_RK4.f90:142-328):
//   k_i = f(s_i, A_i), d_i = D(s_i),  s_1 = y, s_2 = y + h/2 k_1,
//   s_3 = y + h/2 k_2, s_4 = y + h k_3, A likewise from W and d,
//   y' = y + h/6 (k_1 + 2 k_2 + 2 k_3 + k_4), W' = W + h/6 (d_1 + ... ).
// Its adjoint, given (ly', lW'): mu_4 = h/6 ly', nu_4 = h/6 lW'; stage 4's
// vector-Jacobian product gives (ls_4, lA_4); mu_3 = h/3 ly' + h ls_4,
// nu_3 = h/3 lW' + h lA_4; mu_2 = h/3 ly' + h/2 ls_3 (...); mu_1 = h/6 ly' +
// h/2 ls_2 (...); ly = ly' + sum ls_i, lW = lW' + sum lA_i.
//
// k_vjp (one thread per macroparticle) is the vector-Jacobian product of one
// stage: it recomputes the stage (p2, weights, gather, b-fields) and applies
// the transposed derivatives of the six equations (puffin_equations.f90),
// of the deposit (system_interpolation.f90:150-248; its adjoint is a gather
// of nu), of the gather (its adjoint is a deposit of the field adjoint,
// FP64 atomics), of the trilinear weights (piecewise linear in x, y, z2), of
// p2 and of the b-fields; it also reduces dE/d(alpha) of the stage.
//
// Storage: the state (particles, window, outer field) every K steps; during
// the backward sweep one segment of K steps is recomputed and keeps, per
// step, y, W, k_1..k_3 and d_1..d_3, so each step's adjoint needs no further
// recomputation.  The periodic z2 wrap is the identity for the adjoint.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "mixed_common.cuh"
#include "pf_internal.h"

namespace {

inline unsigned grid_for(int64_t n, int threads) {
  const int64_t g = (n + threads - 1) / threads;
  return (unsigned)(g < 1 ? 1 : g);
}

// b-field and its x, y derivatives (the field of bfields.f90 as evaluated by
// the stage kernel, then differentiated)
__device__ __forceinline__ void bfield_jac(const BFieldCoef &b, double x, double y, double &bx,
                                           double &by, double &bz, double &bxx, double &bxy,
                                           double &byx, double &byy, double &bzx, double &bzy) {
  const double pi = PF_PUFFIN_PI;
  bx = b.bx0;
  by = b.by0;
  bz = 0.0;
  bxx = bxy = byx = byy = bzx = bzy = 0.0;
  if (b.type == PF_UND_CURVED) {
    const double shx = sinh(b.kx * x), shy = sinh(b.ky * y);
    const double chx = cosh(b.kx * x), chy = cosh(b.ky * y);
    double kxy, kyy, kz;
    if (b.place == 0) {
      kxy = b.kxky * b.szt / 4.0 / pi * b.S;
      kyy = b.szt / 4.0 / pi * b.S;
      kz = b.czs * b.u3 * b.C;
    } else if (b.place == 2) {
      kxy = b.kxky * b.u3 * b.S;
      kyy = b.u3 * b.S;
      kz = b.cze * b.u3 * b.C;
    } else {
      kxy = b.kxky * b.S;
      kyy = b.S;
      kz = b.cze * b.C;
    }
    bx = kxy * shx * shy;
    by = kyy * chx * chy;
    bxx = kxy * b.kx * chx * shy;
    bxy = kxy * b.ky * shx * chy;
    byx = kyy * b.kx * shx * chy;
    byy = kyy * b.ky * chx * shy;
    if (!b.one_d) {
      bz = kz * chx * shy;
      bzx = kz * b.kx * shx * shy;
      bzy = kz * b.ky * chx * chy;
    }
  } else if (b.type == PF_UND_PLANEPOLE) {
    if (!b.one_d) {
      const double k = (b.place == 1) ? b.C : b.u3 * b.C;
      bz = sinh(b.c1 * y) * k;
      bzy = b.c1 * cosh(b.c1 * y) * k;
    }
  } else if (!b.one_d) {
    const bool hel = (b.type == PF_UND_HELICAL);
    if (b.place == 1) {
      const double ax = hel ? -b.c1 * b.S : -b.c1 * b.fx * b.S;
      const double ay = hel ? b.c1 * b.C : b.c1 * b.fy * b.C;
      bz = ax * x + ay * y;
      bzx = ax;
      bzy = ay;
    } else {
      const double ax = (b.tcase == 0) ? 0.0 : -(b.ux * b.S);
      bz = ax * x + b.uy * y * b.C;
      bzx = ax;
      bzy = b.uy * b.C;
    }
  }
  if (b.focusing) {
    bx = b.focx * y + bx;
    by = -(b.focy * x) + by;
    bxy += b.focx;
    byx -= b.focy;
  }
}

struct VjpArgs {
  StageArgs st;                 // geometry, physics, stage coefficients
  const double *y[6];           // y_n
  const double *kin[6];         // slope forming the stage state (null: stage 1)
  double c;                     // s = y + c kin
  const double *wr, *wi;        // W_n
  const double *dr, *di;        // d forming the stage field (null: stage 1)
  double cA;                    // A = W + cA d
  const double *lnext[6];       // ly'
  const double *lprev[6];       // ls of the previous adjoint stage (null: none)
  double ma, mb;                // mu = ma ly' + mb ls_prev
  const double *nur, *nui;      // nu on the window (times nus)
  double nus;
  int lsum_init;                // lsum = ly' + ls (the step's first adjoint stage), else +=
  double *ls[6];                // out: ls of this stage
  double *lsum[6];              // ls added here
  double *lar, *lai;            // out: field adjoint, scatter-added
  double *galpha;               // out: dE/dalpha of this stage, added
};

__global__ void __launch_bounds__(256) k_vjp(const VjpArgs v) {
  const StageArgs &a = v.st;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double galpha = 0.0;
  if (i < a.np) {
    double s[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) s[j] = v.kin[0] ? v.y[j][i] + v.c * v.kin[j][i] : v.y[j][i];
    const double X = s[0], Y = s[1], Z2 = s[2], PX = s[3], PY = s[4], G = s[5];
    const double chi = a.chi[i];
    double mu[6];
#pragma unroll
    for (int j = 0; j < 6; ++j)
      mu[j] = v.ma * v.lnext[j][i] + (v.lprev[0] ? v.mb * v.lprev[j][i] : 0.0);
    if (!a.electrons_evolve) {
#pragma unroll
      for (int j = 0; j < 6; ++j) mu[j] = 0.0;
    }

    // p2, q / Gamma (gamma_to_p2.f90:84-85; a.gamma_r holds gamma0^2, a.aw aw^2)
    const double aa = 1.0 / (a.gamma_r * (G * G));
    const double bb = 1.0 + a.aw * ((PX * PX) + (PY * PY));
    const double u = aa * bb;
    const double r = 1.0 / sqrt(1.0 - u);
    const double p2 = (r - 1.0) * a.inv_eta;
    const double rG = 1.0 / G;
    const double qrG = (1.0 + a.eta * p2) * rG;

    // weights and nodes (getInterps_3D / _1D)
    const int ONED = a.one_d;
    double wx2 = 0.0, wy2 = 0.0, wz2;
    int64_t pz0, pz1, xy0 = 0;
    {
      const double tz = Z2 * a.inv_dz2;
      const double fz = floor(tz);
      wz2 = tz - fz;
      int64_t m = (int64_t)fz;
      if (a.periodic) {
        m %= a.npl;
        if (m < 0) m += a.npl;
        pz0 = m;
        pz1 = (m + 1 == a.npl) ? 0 : m + 1;
      } else {
        pz0 = min(max(m, (int64_t)0), a.nz2 - 2);
        pz1 = pz0 + 1;
      }
      if (!ONED) {
        const double tx = (X + a.halfx) * a.inv_dx, fx = floor(tx);
        const double ty = (Y + a.halfy) * a.inv_dy, fy = floor(ty);
        wx2 = tx - fx;
        wy2 = ty - fy;
        const int64_t ix = min(max((int64_t)fx, (int64_t)0), a.nix - 2);
        const int64_t iy = min(max((int64_t)fy, (int64_t)0), a.niy - 2);
        xy0 = ix + iy * a.nix;
      }
    }
    const int64_t ntr = a.nix * a.niy;
    const int nc = ONED ? 2 : 8;
    double w[8], gsx[8], gsy[8], gsz[8];  // weight and its factors' signs
    int64_t node[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      if (c >= nc) break;
      if (ONED) {
        const int cz = c;
        w[c] = cz ? wz2 : 1.0 - wz2;
        gsz[c] = cz ? 1.0 : -1.0;
        gsx[c] = gsy[c] = 0.0;
        node[c] = cz ? pz1 : pz0;
      } else {
        const int cx = c & 1, cy = (c >> 1) & 1, cz = c >> 2;
        const double fxw = cx ? wx2 : 1.0 - wx2, fyw = cy ? wy2 : 1.0 - wy2;
        const double fzw = cz ? wz2 : 1.0 - wz2;
        w[c] = fxw * fyw * fzw;
        gsx[c] = (cx ? 1.0 : -1.0) * fyw * fzw;
        gsy[c] = (cy ? 1.0 : -1.0) * fxw * fzw;
        gsz[c] = (cz ? 1.0 : -1.0) * fxw * fyw;
        node[c] = (cz ? pz1 : pz0) * ntr + xy0 + cx + (int64_t)cy * a.nix;
      }
    }
    // gather of the stage field A = W + cA d
    double Ar[8], Ai[8];
    double fr = 0.0, fi = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      if (c >= nc) break;
      Ar[c] = v.wr[node[c]] + (v.dr ? v.cA * v.dr[node[c]] : 0.0);
      Ai[c] = v.wi[node[c]] + (v.di ? v.cA * v.di[node[c]] : 0.0);
      fr += w[c] * Ar[c];
      fi += w[c] * Ai[c];
    }
    const double cpl = a.coupling ? 1.0 : 0.0;
    fr *= cpl;
    fi *= cpl;
    double bx, by, bz, bxx, bxy, byx, byy, bzx, bzy;
    bfield_jac(a.bf, X, Y, bx, by, bz, bxx, bxy, byx, byy, bzx, bzy);
    const double ep = p2 * a.eta_k2;
    const double cz = a.kn2col * qrG * bz;

    // transposed derivatives of the equations
    double g_fr = -mu[3] * a.sInv2rho * ep - mu[5] * a.rho2 * qrG * PX;
    double g_fi = -mu[4] * a.sInv2rho * ep - mu[5] * a.rho2 * qrG * PY;
    const double g_ep = -mu[3] * a.sInv2rho * fr - mu[4] * a.sInv2rho * fi;
    const double g_cz = mu[3] * PY - mu[4] * PX;
    const double g_bx = mu[4] * a.sInv2rho * a.n2col;
    const double g_by = mu[3] * a.sInv2rho * a.n2col;
    const double g_bz = g_cz * a.kn2col * qrG;
    galpha = mu[3] * a.sInv2rho * by + mu[4] * a.sInv2rho * bx + g_cz * a.kappa * qrG * bz;
    double g_qrG = mu[0] * a.dxc * PX - mu[1] * a.dxc * PY + g_cz * a.kn2col * bz -
                   mu[5] * a.rho2 * (PX * fr + PY * fi);
    double g_PX = mu[0] * a.dxc * qrG - mu[4] * cz - mu[5] * a.rho2 * qrG * fr;
    double g_PY = -mu[1] * a.dxc * qrG + mu[3] * cz - mu[5] * a.rho2 * qrG * fi;
    double g_p2 = mu[2] + g_ep * a.eta_k2;
    g_fr *= cpl;
    g_fi *= cpl;

    // deposit adjoint (gather of nu) and gather adjoint (deposit of g_f)
    double gw[8];
    const double dw = chi * a.inv_dV3 * qrG;
    const double sr = dw * PX, si = dw * PY;
    double G_sr = 0.0, G_si = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      if (c >= nc) break;
      gw[c] = g_fr * Ar[c] + g_fi * Ai[c];
      if (a.field_evolve) {
        const double nr = v.nus * v.nur[node[c]], ni = v.nus * v.nui[node[c]];
        gw[c] += nr * sr + ni * si;
        G_sr += w[c] * nr;
        G_si += w[c] * ni;
      }
      if (g_fr != 0.0) atomicAdd(v.lar + node[c], w[c] * g_fr);
      if (g_fi != 0.0) atomicAdd(v.lai + node[c], w[c] * g_fi);
    }
    const double g_dw = G_sr * PX + G_si * PY;
    g_PX += G_sr * dw;
    g_PY += G_si * dw;
    g_qrG += g_dw * chi * a.inv_dV3;

    // qrG = (1 + eta p2) / Gamma
    g_p2 += g_qrG * a.eta * rG;
    double g_G = -g_qrG * qrG * rG;
    // p2 = ((1 - u)^(-1/2) - 1) / eta, u = aa bb
    const double g_u = g_p2 * (r * r * r) * 0.5 * a.inv_eta;
    g_PX += g_u * aa * 2.0 * a.aw * PX;
    g_PY += g_u * aa * 2.0 * a.aw * PY;
    g_G += -2.0 * g_u * u * rG;

    // positions: weights and b-fields
    double g_X = 0.0, g_Y = 0.0, g_Z = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      if (c >= nc) break;
      g_X += gw[c] * gsx[c];
      g_Y += gw[c] * gsy[c];
      g_Z += gw[c] * gsz[c];
    }
    g_X *= a.inv_dx;
    g_Y *= a.inv_dy;
    g_Z *= a.inv_dz2;
    if (ONED) {
      g_X = 0.0;
      g_Y = 0.0;
    }
    g_X += g_bx * bxx + g_by * byx + g_bz * bzx;
    g_Y += g_bx * bxy + g_by * byy + g_bz * bzy;

    const double ls[6] = {g_X, g_Y, g_Z, g_PX, g_PY, g_G};
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      v.ls[j][i] = ls[j];
      v.lsum[j][i] = (v.lsum_init ? v.lnext[j][i] : v.lsum[j][i]) + ls[j];
    }
  }
  // block reduction of dE/dalpha
  __shared__ double sred[8];
  for (int o = 16; o > 0; o >>= 1) galpha += __shfl_xor_sync(0xffffffffu, galpha, o);
  if ((threadIdx.x & 31) == 0) sred[threadIdx.x >> 5] = galpha;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sred[k];
    if (t != 0.0) atomicAdd(v.galpha, t);
  }
}

// nu_next = a lW' + b lA; lWsum += lA (init: lWsum = lW' + lA); lA = 0
__global__ void k_adj_nodes(int64_t n, const double *lwr, const double *lwi, double *lar,
                            double *lai, double *lsr, double *lsi, double *nur, double *nui,
                            double ca, double cb, int init) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double ar = lar[t], ai = lai[t], wr = lwr[t], wi = lwi[t];
  nur[t] = ca * wr + cb * ar;
  nui[t] = ca * wi + cb * ai;
  lsr[t] = (init ? wr : lsr[t]) + ar;
  lsi[t] = (init ? wi : lsi[t]) + ai;
  // zeros computed from the loaded values, so that the stores issue once
  // the loads have returned (a constant store to an address whose load is
  // in flight is several times slower)
  lar[t] = ar - ar;
  lai[t] = ai - ai;
}

__global__ void k_scale2(int64_t n, const double *xr, const double *xi, double *yr, double *yi,
                         double c) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  yr[t] = c * xr[t];
  yi[t] = c * xi[t];
}

// y' = y + h/6 (k1 + k4 + 2 (k2 + k3)) on one array
__global__ void k_commit(int64_t n, const double *y, const double *k1, const double *k2,
                         const double *k3, const double *k4, double h6, double *out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  out[t] = y[t] + h6 * (k1[t] + k4[t] + 2.0 * (k2[t] + k3[t]));
}

// window <-> outer (the window sits centred in x and y, all its planes)
__global__ void k_win(double *wr, double *wi, double *orr, double *oi, int nix, int niy,
                      int64_t npl, int nx, int ny, int to_outer) {
  const int64_t nw = (int64_t)nix * niy * npl;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nw) return;
  const int ix = (int)(t % nix), iy = (int)((t / nix) % niy);
  const int64_t iz = t / ((int64_t)nix * niy);
  const int64_t o = (ix + (nx - nix) / 2) + (int64_t)nx * (iy + (ny - niy) / 2) +
                    (int64_t)nx * ny * iz;
  if (to_outer) {
    orr[o] = wr[t];
    oi[o] = wi[t];
  } else {
    wr[t] = orr[o];
    wi[t] = oi[o];
  }
}

__global__ void k_wrap(double *z2, int64_t n, double lenz2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) z2[i] = z2[i] - (floor(z2[i] / lenz2) * lenz2);
}

// gamma += chirp (z2 - zmean)
__global__ void k_chirp(int64_t n, const double *z2, double *gam, double chirp, double zmean) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) gam[t] += chirp * (z2[t] - zmean);
}

// dot products for the seed and chirp gradients (one block, fixed order)
__global__ void k_dot2(int64_t n, const double *ar, const double *ai, const double *br,
                       const double *bi, double *out) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int64_t t = threadIdx.x; t < n; t += 256) acc += ar[t] * br[t] + (ai ? ai[t] * bi[t] : 0.0);
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if ((int)threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

__global__ void k_chirp_grad(int64_t n, const double *lg, const double *z2, double zmean,
                             double *out) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int64_t t = threadIdx.x; t < n; t += 256) acc += lg[t] * (z2[t] - zmean);
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if ((int)threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

// ---- the mixed-precision form -------------------------------------------
// The recorded forward runs pf_rk4_mixed's kernels (FP32 field, weights,
// gather, deposit and transverse slopes; FP64 state, z2 and Gamma stage
// values, p2 and the stage combination).  Its adjoint keeps the same split:
// the field adjoint (window, outer mesh) is FP32 complex, the particle
// adjoint state, its sums and the RK4 combination FP64; the vector-Jacobian
// product of a stage recomputes the stage's FP64 values (z2, Gamma, p2) as
// the forward does and applies the transposed derivatives in FP32, except
// the z2 (phase) adjoint, which is formed and added to the p2 adjoint in
// FP64.

// b-field of bfield_f and its x, y derivatives, in FP32
__device__ __forceinline__ void bfield_jac_f(const BFieldF &b, float x, float y, float &bx,
                                             float &by, float &bz, float &bxx, float &bxy,
                                             float &byx, float &byy, float &bzx, float &bzy) {
  const float pi = (float)PF_PUFFIN_PI;
  bx = b.bx0;
  by = b.by0;
  bz = 0.f;
  bxx = bxy = byx = byy = bzx = bzy = 0.f;
  if (b.type == PF_UND_CURVED) {
    const float shx = sinhf(b.kx * x), shy = sinhf(b.ky * y);
    const float chx = coshf(b.kx * x), chy = coshf(b.ky * y);
    float kxy, kyy, kz;
    if (b.place == 0) {
      kxy = b.kxky * b.szt / 4.f / pi * b.S;
      kyy = b.szt / 4.f / pi * b.S;
      kz = b.czs * b.u3 * b.C;
    } else if (b.place == 2) {
      kxy = b.kxky * b.u3 * b.S;
      kyy = b.u3 * b.S;
      kz = b.cze * b.u3 * b.C;
    } else {
      kxy = b.kxky * b.S;
      kyy = b.S;
      kz = b.cze * b.C;
    }
    bx = kxy * shx * shy;
    by = kyy * chx * chy;
    bxx = kxy * b.kx * chx * shy;
    bxy = kxy * b.ky * shx * chy;
    byx = kyy * b.kx * shx * chy;
    byy = kyy * b.ky * chx * shy;
    if (!b.one_d) {
      bz = kz * chx * shy;
      bzx = kz * b.kx * shx * shy;
      bzy = kz * b.ky * chx * chy;
    }
  } else if (b.type == PF_UND_PLANEPOLE) {
    if (!b.one_d) {
      const float k = (b.place == 1) ? b.C : b.u3 * b.C;
      bz = sinhf(b.c1 * y) * k;
      bzy = b.c1 * coshf(b.c1 * y) * k;
    }
  } else if (!b.one_d) {
    const bool hel = (b.type == PF_UND_HELICAL);
    if (b.place == 1) {
      const float ax = hel ? -b.c1 * b.S : -b.c1 * b.fx * b.S;
      const float ay = hel ? b.c1 * b.C : b.c1 * b.fy * b.C;
      bz = ax * x + ay * y;
      bzx = ax;
      bzy = ay;
    } else {
      const float ax = (b.tcase == 0) ? 0.f : -(b.ux * b.S);
      bz = ax * x + b.uy * y * b.C;
      bzx = ax;
      bzy = b.uy * b.C;
    }
  }
  if (b.focusing) {
    bx = b.focx * y + bx;
    by = -(b.focy * x) + by;
    bxy += b.focx;
    byx -= b.focy;
  }
}

struct VjpMixArgs {
  const double *y[6];       // y_n
  const float *kin_f[6];    // FP32 slope forming the stage state (null: stage 1; index 2 unused)
  const double *kin_z;      // FP64 z2 slope
  double c;                 // s = y + c kin
  float c_f;
  const float2 *w, *d;      // W_n and the d forming the stage field (d null: stage 1)
  float cA_f;               // A = W + cA d
  const double *lnext[6];   // ly'
  const double *lprev[6];   // ls of the previous adjoint stage (null: none)
  double ma, mb;            // mu = ma ly' + mb ls_prev
  const float2 *nu;         // nu on the window (times nus)
  float nus;
  int lsum_init;            // lsum = ly' + ls (the step's first adjoint stage), else +=
  double *ls[6];            // out: ls of this stage
  double *lsum[6];          // ls added here
  float2 *la;               // out: field adjoint, scatter-added
  double *galpha;           // out: dE/dalpha of this stage, added
  const float *chi_f;
  int64_t np, npl, nz2;
  int nix, niy, periodic, one_d;
  PfMixConst k;             // the stage kernel's constants
  float kn2col, n2col, kappa;
  float inv_eta_f, aw2g_f, inv_dz2_f;
  BFieldF bf;
  int field_evolve, electrons_evolve, coupling;
};

__global__ void __launch_bounds__(256) k_vjp_mixed(const VjpMixArgs v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float galpha = 0.f;
  if (i < v.np) {
    // the stage state as the mixed stage kernel forms it
    const double z0 = v.y[2][i], g0 = v.y[5][i];
    float X = d2f_rn(v.y[0][i]), Y = d2f_rn(v.y[1][i]);
    float PX = d2f_rn(v.y[3][i]), PY = d2f_rn(v.y[4][i]);
    double zs = z0, gs = g0;
    if (v.kin_z) {
      zs = fma(v.c, v.kin_z[i], z0);
      gs = fma(v.c, f2d(v.kin_f[5][i]), g0);
      PX = fmaf(v.c_f, v.kin_f[3][i], PX);
      PY = fmaf(v.c_f, v.kin_f[4][i], PY);
      X = fmaf(v.c_f, v.kin_f[0][i], X);
      Y = fmaf(v.c_f, v.kin_f[1][i], Y);
    }
    // mu = ma ly' + mb ls_prev: the z2 component in FP64, the others in FP32
    // (conversions with integer operations: GB300's cvt between the formats
    // runs on the FP64 pipe)
    double lnext[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) lnext[j] = v.lnext[j][i];
    double mu2 = 0.0;
    float m[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (v.electrons_evolve) {
      const float maf = d2f_rn(v.ma), mbf = d2f_rn(v.mb);
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        if (j == 2) continue;
        m[j] = maf * d2f_rn(lnext[j]);
        if (v.lprev[0]) m[j] = fmaf(mbf, d2f_rn(v.lprev[j][i]), m[j]);
      }
      mu2 = v.ma * lnext[2] + (v.lprev[0] ? v.mb * v.lprev[2][i] : 0.0);
      m[2] = d2f_rn(mu2);
    }
    // 1/Gamma, u, p2 and q/Gamma as the forward computes them
    const float rGf = __frcp_rn(d2f_rn(gs));
    double rG = f2d(rGf);
    rG = fma(rG, fma(-gs, rG, 1.0), rG);
    const double u = fma(v.k.aw2g, f2d(fmaf(PX, PX, PY * PY)), v.k.g02) * (rG * rG);
    const double p2 = p2_series(u, v.k.ser, v.k.inv_eta, v.k.ser_r1, v.k.ser_r2);
    const float p2f = d2f_rn(p2);
    const float qrG = fmaf(v.k.eta_f, p2f, 1.f) * rGf;

    // cell, weights (FP32) and nodes
    const double tz = zs * v.k.inv_dz2;
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
    if (ok && v.periodic) {
      int m = iz % (int)v.npl;
      if (m < 0) m += (int)v.npl;
      pz0 = m;
      pz1 = (m + 1 == v.npl) ? 0 : m + 1;
    } else if (ok) {
      ok = (iz >= 0 && iz + 1 < v.nz2);
      pz0 = iz;
      pz1 = iz + 1;
    }
    const bool ONED = v.one_d != 0;
    float x2 = 0.f, y2 = 0.f;
    int64_t b0 = 0;
    if (!ONED && ok) {
      const float tx = fmaf(X, v.k.inv_dx_f, v.k.hx_dx), fx = floorf(tx);
      const float ty = fmaf(Y, v.k.inv_dy_f, v.k.hy_dy), fy = floorf(ty);
      ok = (fx >= 0.f && fx + 1.f < (float)v.nix && fy >= 0.f && fy + 1.f < (float)v.niy);
      x2 = tx - fx;
      y2 = ty - fy;
      b0 = (int64_t)fx + (int64_t)fy * v.nix;
    }
    // a macroparticle outside the mesh or the window stopped the recorded
    // forward (the adjoint run reports it), so none reaches here with !ok;
    // it is skipped rather than indexed out of range
    if (ok) {
      const int64_t ntr = (int64_t)v.nix * v.niy;
      const int nc = ONED ? 2 : 8;
      const float x1 = 1.f - x2, y1 = 1.f - y2, zw1 = 1.f - zw2;
      float w[8], gsx[8], gsy[8], gsz[8];
      int64_t node[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        if (c >= nc) break;
        if (ONED) {
          w[c] = c ? zw2 : zw1;
          gsz[c] = c ? 1.f : -1.f;
          gsx[c] = gsy[c] = 0.f;
          node[c] = c ? pz1 : pz0;
        } else {
          const int cx = c & 1, cy = (c >> 1) & 1, cz = c >> 2;
          const float fxw = cx ? x2 : x1, fyw = cy ? y2 : y1, fzw = cz ? zw2 : zw1;
          w[c] = fxw * fyw * fzw;
          gsx[c] = (cx ? 1.f : -1.f) * fyw * fzw;
          gsy[c] = (cy ? 1.f : -1.f) * fxw * fzw;
          gsz[c] = (cz ? 1.f : -1.f) * fxw * fyw;
          node[c] = (int64_t)(cz ? pz1 : pz0) * ntr + b0 + cx + (int64_t)cy * v.nix;
        }
      }
      // gather of the stage field A = W + cA d (the node kernel's arithmetic)
      float Ar[8], Ai[8];
      float fr = 0.f, fi = 0.f;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        if (c >= nc) break;
        const float2 wn = v.w[node[c]];
        if (v.d) {
          const float2 dn = v.d[node[c]];
          Ar[c] = wn.x + v.cA_f * dn.x;
          Ai[c] = wn.y + v.cA_f * dn.y;
        } else {
          Ar[c] = wn.x;
          Ai[c] = wn.y;
        }
        fr += w[c] * Ar[c];
        fi += w[c] * Ai[c];
      }
      const float cpl = v.coupling ? 1.f : 0.f;
      fr *= cpl;
      fi *= cpl;
      float bx, by, bz, bxx, bxy, byx, byy, bzx, bzy;
      bfield_jac_f(v.bf, X, Y, bx, by, bz, bxx, bxy, byx, byy, bzx, bzy);
      const float ep = p2f * v.k.eta_k2;
      const float cz = v.kn2col * qrG * bz;

      // transposed derivatives of the slopes
      float g_fr = -m[3] * v.k.sInv2rho * ep - m[5] * v.k.rho2 * qrG * PX;
      float g_fi = -m[4] * v.k.sInv2rho * ep - m[5] * v.k.rho2 * qrG * PY;
      const float g_ep = -m[3] * v.k.sInv2rho * fr - m[4] * v.k.sInv2rho * fi;
      const float g_cz = m[3] * PY - m[4] * PX;
      const float g_bx = m[4] * v.k.sInv2rho * v.n2col;
      const float g_by = m[3] * v.k.sInv2rho * v.n2col;
      const float g_bz = g_cz * v.kn2col * qrG;
      galpha = m[3] * v.k.sInv2rho * by + m[4] * v.k.sInv2rho * bx + g_cz * v.kappa * qrG * bz;
      float g_qrG = m[0] * v.k.dxc * PX - m[1] * v.k.dxc * PY + g_cz * v.kn2col * bz -
                    m[5] * v.k.rho2 * (PX * fr + PY * fi);
      float g_PX = m[0] * v.k.dxc * qrG - m[4] * cz - m[5] * v.k.rho2 * qrG * fr;
      float g_PY = -m[1] * v.k.dxc * qrG + m[3] * cz - m[5] * v.k.rho2 * qrG * fi;
      g_fr *= cpl;
      g_fi *= cpl;

      // deposit adjoint (gather of nu) and gather adjoint (deposit of g_f)
      float gw[8];
      const float dw = v.chi_f[i] * v.k.inv_dV3 * qrG;
      const float sr = dw * PX, si = dw * PY;
      float G_sr = 0.f, G_si = 0.f;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        if (c >= nc) break;
        gw[c] = g_fr * Ar[c] + g_fi * Ai[c];
        if (v.field_evolve) {
          float2 nn = v.nu[node[c]];
          nn.x *= v.nus;
          nn.y *= v.nus;
          gw[c] += nn.x * sr + nn.y * si;
          G_sr += w[c] * nn.x;
          G_si += w[c] * nn.y;
        }
        if (g_fr != 0.f || g_fi != 0.f) atomicAdd(v.la + node[c], make_float2(w[c] * g_fr, w[c] * g_fi));
      }
      g_PX += G_sr * dw;
      g_PY += G_si * dw;
      g_qrG += (G_sr * PX + G_si * PY) * v.chi_f[i] * v.k.inv_dV3;

      // qrG = (1 + eta p2) / Gamma and p2 = ((1 - u)^(-1/2) - 1) / eta with
      // u = (aw^2 p_perp^2 + 1) / (gamma0^2 Gamma^2): the adjoint of p2 sums
      // the z2 adjoint (FP64) and the FP32 terms in FP64; its chain through u
      // is FP32
      const double g_p2 = mu2 + f2d(fmaf(g_qrG * v.k.eta_f, rGf, g_ep * v.k.eta_k2));
      const float uf = d2f_rn(u);
      const float rf = rsqrtf(1.f - uf);
      const float g_u = d2f_rn(g_p2) * (0.5f * v.inv_eta_f) * (rf * rf * rf);
      const float gpp = g_u * v.aw2g_f * (rGf * rGf);  // d/d(px^2 + py^2)
      const float gPX = fmaf(2.f * gpp, PX, g_PX);
      const float gPY = fmaf(2.f * gpp, PY, g_PY);
      const float gG = -g_qrG * qrG * rGf - 2.f * g_u * uf * rGf;

      // positions: weights and b-fields
      float g_X = 0.f, g_Y = 0.f, g_Z = 0.f;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        if (c >= nc) break;
        g_X += gw[c] * gsx[c];
        g_Y += gw[c] * gsy[c];
        g_Z += gw[c] * gsz[c];
      }
      g_X *= v.k.inv_dx_f;
      g_Y *= v.k.inv_dy_f;
      if (ONED) {
        g_X = 0.f;
        g_Y = 0.f;
      }
      g_X += g_bx * bxx + g_by * byx + g_bz * bzx;
      g_Y += g_bx * bxy + g_by * byy + g_bz * bzy;
      const double ls[6] = {f2d(g_X), f2d(g_Y), f2d(g_Z * v.inv_dz2_f), f2d(gPX), f2d(gPY),
                            f2d(gG)};
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        v.ls[j][i] = ls[j];
        v.lsum[j][i] = (v.lsum_init ? lnext[j] : v.lsum[j][i]) + ls[j];
      }
    } else {
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        v.ls[j][i] = 0.0;
        if (v.lsum_init) v.lsum[j][i] = lnext[j];
      }
    }
  }
  // dE/dalpha: FP32 within the warp, FP64 across warps and blocks
  __shared__ double sred[8];
  for (int o = 16; o > 0; o >>= 1) galpha += __shfl_xor_sync(0xffffffffu, galpha, o);
  if ((threadIdx.x & 31) == 0) sred[threadIdx.x >> 5] = f2d(galpha);
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sred[k];
    if (t != 0.0) atomicAdd(v.galpha, t);
  }
}

// Recorded node update of the mixed step: d_s = acc kept in dout, the next
// stage field W + coef d_s, the accumulator cleared; with wout (stage 4),
// W' = W + h/6 (d1 + d4 + 2 (d2 + d3)) in the node kernel's arithmetic.
__global__ void k_rec_nodes_c32(int64_t n, float2 *acc, const float2 *w, float2 *dout, float2 *as,
                                float coef, const float2 *d1, const float2 *d2, const float2 *d3,
                                float2 *wout, float h6) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float2 d = acc[t], wn = w[t];
  if (wout) {
    const float2 a = d1[t], b = d2[t], c = d3[t];
    const float2 e12 = make_float2(b.x + c.x, b.y + c.y);
    wout[t] = make_float2(wn.x + h6 * (a.x + d.x + 2.f * e12.x),
                          wn.y + h6 * (a.y + d.y + 2.f * e12.y));
  } else {
    dout[t] = d;
    as[t] = make_float2(wn.x + coef * d.x, wn.y + coef * d.y);
  }
  acc[t] = make_float2(0.f, 0.f);
}

// nu_next = a lW' + b lA; lWsum += lA (init: lWsum = lW' + lA); lA = 0
// (FP32 complex)
__global__ void k_adj_nodes_c32(int64_t n, const float2 *lw, float2 *la, float2 *lws, float2 *nu,
                                float ca, float cb, int init) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float2 a = la[t], w = lw[t], s = init ? w : lws[t];
  nu[t] = make_float2(ca * w.x + cb * a.x, ca * w.y + cb * a.y);
  lws[t] = make_float2(s.x + a.x, s.y + a.y);
  la[t] = make_float2(a.x - a.x, a.y - a.y);
}

__global__ void k_scale_c32(int64_t n, const float2 *x, float2 *y, float c) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) y[t] = make_float2(c * x[t].x, c * x[t].y);
}

// complex-float outer mesh = c (re + i im) from the FP64 split seed
__global__ void k_seed_c32(int64_t n, const double *re, const double *im, float2 *o, double c) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) o[t] = make_float2((float)(c * re[t]), (float)(c * im[t]));
}

// window <-> outer mesh, complex float
__global__ void k_win_c32(float2 *w, float2 *o, int nix, int niy, int64_t npl, int nx, int ny,
                          int to_outer) {
  const int64_t nw = (int64_t)nix * niy * npl;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nw) return;
  const int ix = (int)(t % nix), iy = (int)((t / nix) % niy);
  const int64_t iz = t / ((int64_t)nix * niy);
  const int64_t o_ = (ix + (nx - nix) / 2) + (int64_t)nx * (iy + (ny - niy) / 2) +
                     (int64_t)nx * ny * iz;
  if (to_outer)
    o[o_] = w[t];
  else
    w[t] = o[o_];
}

// sum a . b over n complex-float values, b complex float or FP64 split
// (one block, fixed order)
__global__ void k_dot_c32(int64_t n, const float2 *a, const float2 *b, const double *br,
                          const double *bi, double *out) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int64_t t = threadIdx.x; t < n; t += 256) {
    const float2 x = a[t];
    if (b) {
      const float2 y = b[t];
      acc += (double)x.x * (double)y.x + (double)x.y * (double)y.y;
    } else {
      acc += (double)x.x * br[t] + (double)x.y * bi[t];
    }
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if ((int)threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

}  // namespace

// ---------------------------------------------------------------------------
struct AdjCtx {
  int32_t nsteps = 0, every = 0, qdiff = 0, K = 0, nseg = 0;
  bool mixed = false;        // the mixed-precision form (complex-float field arrays)
  int64_t csteps0 = 0;
  double hstep = 0.0, seed_amp = 0.0, chirp = 0.0, zmean = 0.0, energy = 0.0;
  int64_t np = 0, nwin = 0, nouter = 0;
  double *base = nullptr;    // base beam (6 np), restored after the calls
  double *seed = nullptr;    // seed field (2 nouter)
  double *ckpt = nullptr;    // per segment: particles 6 np, window 2 nwin, outer 2 nouter
  double *store = nullptr;   // per step of a segment: y 6np, k1..k3 18np, W 2nwin, d1..d3 6nwin
  double *work = nullptr;    // adjoint state and temporaries
  double *galpha = nullptr;  // dE/dalpha per (step, stage)
  double *fin = nullptr;     // final outer field of the forward run (2 nouter)
  bool ready = false;
  ~AdjCtx() {
    cudaFree(base);
    cudaFree(seed);
    cudaFree(ckpt);
    cudaFree(store);
    cudaFree(work);
    cudaFree(galpha);
    cudaFree(fin);
  }
};

void pf_adj_destroy(AdjCtx *c) { delete c; }

namespace {

size_t ckpt_doubles(const AdjCtx &c) { return 6 * c.np + 2 * c.nwin + 2 * c.nouter; }
size_t slot_doubles(const AdjCtx &c) { return 24 * c.np + 8 * c.nwin; }

// dz of the diffraction that follows step istep (0 before the first step),
// 0 when none follows; the schedule of pf_run (undulator.f90:222-289)
double diff_after(int istep, int nsteps, int every, double h) {
  if (istep == 0) return (double)every * h / 2.0;
  if (!(istep % every == 0 || istep == nsteps)) return 0.0;
  auto start = [&](int k) -> double {  // dzdS set at step k
    if (k == 0) return (double)every * h / 2.0;
    if (k == nsteps) return 0.0;
    if (k + every <= nsteps) return (double)every * h / 2;
    return (double)(nsteps - k) * h / 2;
  };
  const int prev = ((istep - 1) / every) * every;  // the previous diffraction point
  return start(prev) + start(istep);
}

struct StepPtrs {
  double *y[6], *k1[6], *k2[6], *k3[6], *wr, *wi, *d1r, *d1i, *d2r, *d2i, *d3r, *d3i;
};

StepPtrs slot(const AdjCtx &c, int k) {
  double *b = c.store + (size_t)k * slot_doubles(c);
  StepPtrs s;
  for (int j = 0; j < 6; ++j) {
    s.y[j] = b + j * c.np;
    s.k1[j] = b + (6 + j) * c.np;
    s.k2[j] = b + (12 + j) * c.np;
    s.k3[j] = b + (18 + j) * c.np;
  }
  double *w = b + 24 * c.np;
  s.wr = w;
  s.wi = w + c.nwin;
  s.d1r = w + 2 * c.nwin;
  s.d1i = w + 3 * c.nwin;
  s.d2r = w + 4 * c.nwin;
  s.d2i = w + 5 * c.nwin;
  s.d3r = w + 6 * c.nwin;
  s.d3i = w + 7 * c.nwin;
  return s;
}

// stage coefficients of (step istep, stage s) from the taper profile
void stage_setup(pf_handle *h, double sz, StageArgs &a) {
  const pf_params &p = h->p;
  double n2col;
  int place;
  pf_taper_stage(h, sz, &n2col, &place);
  a.n2col = n2col;
  a.kn2col = p.kappa * n2col;
  pf_stage_coefficients(p, sz, n2col, place, &a.bf);
}

// One forward step from slot k (y, W) to the state (y', W') at yout/wout,
// keeping k1..k3 and d1..d3 in slot k.  k4 and d4 use the handle's kb and
// d0 arrays as scratch.
int record_step(pf_handle *h, AdjCtx &c, int k, double szl, double *const yout[6], double *woutr,
                double *wouti) {
  const double hs = c.hstep, hh = hs * 0.5, h6 = hs / 6.0;
  StepPtrs S = slot(c, k);
  StageArgs a;
  pf_fill_stage_args(h, a, h6);
  a.x = S.y[0];
  a.y = S.y[1];
  a.z2 = S.y[2];
  a.px = S.y[3];
  a.py = S.y[4];
  a.gam = S.y[5];
  NodeArgs n;
  memset(&n, 0, sizeof(n));
  n.n = h->nwin;
  n.acc_lo_r = a.acc_lo_r;
  n.acc_hi_r = a.acc_hi_r;
  n.acc_lo_i = a.acc_lo_i;
  n.acc_hi_i = a.acc_hi_i;
  n.wr = S.wr;
  n.wi = S.wi;
  n.asr = h->asr;
  n.asi = h->asi;
  n.fix_e = h->fix_e;
  n.status = h->d_status;
  double *const *kk[4] = {S.k1, S.k2, S.k3, h->kb};
  double *dr[4] = {S.d1r, S.d2r, S.d3r, h->d0r};
  double *di[4] = {S.d1i, S.d2i, S.d3i, h->d0i};
  const double sz[4] = {szl, szl + hh, szl + hh, szl + hs};
  const double cs[4] = {0.0, hh, hh, hs};
  const double cn[4] = {hh, hh, hs, 0.0};
  for (int s = 0; s < 4; ++s) {
    stage_setup(h, sz[s], a);
    a.cstate = cs[s];
    a.ar = (s == 0) ? S.wr : h->asr;
    a.ai = (s == 0) ? S.wi : h->asi;
    for (int j = 0; j < 6; ++j) {
      a.kin[j] = (s == 0) ? nullptr : kk[s - 1][j];
      a.kout[j] = kk[s][j];  // stage 1 writes kout
      a.kacc[j] = kk[s][j];  // the stage-2 form writes kacc
    }
    int rc = pf_launch_stage(h, s == 0 ? 1 : 2, a);
    if (rc) return rc;
    n.coef = cn[s];
    n.d12r = dr[s];
    n.d12i = di[s];
    rc = pf_launch_nodes(h, 2, n);  // d_s = dA/dz, A_{s+1} = W + coef d_s
    if (rc) return rc;
  }
  for (int j = 0; j < 6; ++j) {
    k_commit<<<grid_for(c.np, 256), 256, 0, h->stream>>>(c.np, S.y[j], S.k1[j], S.k2[j], S.k3[j],
                                                          h->kb[j], h6, yout[j]);
    PF_LAUNCHED(h);
  }
  k_commit<<<grid_for(c.nwin, 256), 256, 0, h->stream>>>(c.nwin, S.wr, S.d1r, S.d2r, S.d3r,
                                                          h->d0r, h6, woutr);
  PF_LAUNCHED(h);
  k_commit<<<grid_for(c.nwin, 256), 256, 0, h->stream>>>(c.nwin, S.wi, S.d1i, S.d2i, S.d3i,
                                                          h->d0i, h6, wouti);
  PF_LAUNCHED(h);
  return PF_OK;
}

// The mixed form of record_step: the slot's window and d arrays hold one
// float2 per node, its slope arrays FP32 values (z2: FP64); k2 + k3 goes to
// the handle's ka scratch, as pf_rk4_mixed forms it.
int record_step_mixed(pf_handle *h, AdjCtx &c, int k, double szl, double *const yout[6],
                      float2 *wout) {
  const double hs = c.hstep, hh = hs * 0.5;
  StepPtrs S = slot(c, k);
  float2 *W = (float2 *)S.wr;
  float2 *D[3] = {(float2 *)S.d1r, (float2 *)S.d2r, (float2 *)S.d3r};
  const double sz[4] = {szl, szl + hh, szl + hh, szl + hs};
  const float coef[3] = {(float)hh, (float)hh, (float)hs};
  const unsigned ng = grid_for(c.nwin, 256);
  float2 *acc = (float2 *)h->acc32, *as = (float2 *)h->as32;
  for (int s = 1; s <= 4; ++s) {
    PfMixRec r;
    memset(&r, 0, sizeof(r));
    for (int j = 0; j < 6; ++j) {
      r.y[j] = S.y[j];
      r.k1[j] = S.k1[j];
      r.ynext[j] = yout[j];
      r.kin[j] = (s == 2) ? S.k1[j] : (s == 3) ? S.k2[j] : (s == 4) ? S.k3[j] : nullptr;
      r.kout[j] = (s == 1) ? S.k1[j] : (s == 3) ? S.k3[j] : nullptr;
      r.kacc[j] = (s == 2) ? S.k2[j] : (s >= 3) ? h->ka[j] : nullptr;
    }
    r.as = (s == 1) ? (const void *)W : (const void *)as;
    int rc = pf_mixed_stage_rec(h, s, hs, sz[s - 1], r);
    if (rc) return rc;
    if (s < 4)
      k_rec_nodes_c32<<<ng, 256, 0, h->stream>>>(c.nwin, acc, W, D[s - 1], as, coef[s - 1],
                                                 nullptr, nullptr, nullptr, nullptr, 0.f);
    else
      k_rec_nodes_c32<<<ng, 256, 0, h->stream>>>(c.nwin, acc, W, nullptr, nullptr, 0.f, D[0], D[1],
                                                 D[2], wout, (float)(hs / 6.0));
    PF_LAUNCHED(h);
  }
  return PF_OK;
}

// diffraction of a complex-float window state through the handle's
// complex-float outer mesh
int diffract_window_c32(pf_handle *h, float2 *w, double dz) {
  const unsigned g = grid_for(h->nwin, 256);
  k_win_c32<<<g, 256, 0, h->stream>>>(w, (float2 *)h->oc32, h->nix, h->niy, h->npl, h->p.nx,
                                      h->p.ny, 1);
  PF_LAUNCHED(h);
  int rc = pf_diffract_outer_c32(h, h->oc32, dz);
  if (rc) return rc;
  k_win_c32<<<g, 256, 0, h->stream>>>(w, (float2 *)h->oc32, h->nix, h->niy, h->npl, h->p.nx,
                                      h->p.ny, 0);
  PF_LAUNCHED(h);
  return PF_OK;
}

// diffraction of the window state (wr, wi) through the outer mesh
int diffract_window(pf_handle *h, double *wr, double *wi, double dz) {
  k_win<<<grid_for(h->nwin, 256), 256, 0, h->stream>>>(wr, wi, h->or_, h->oi_, h->nix, h->niy,
                                                       h->npl, h->p.nx, h->p.ny, 1);
  PF_LAUNCHED(h);
  int rc = pf_diffract_outer(h, dz);
  if (rc) return rc;
  k_win<<<grid_for(h->nwin, 256), 256, 0, h->stream>>>(wr, wi, h->or_, h->oi_, h->nix, h->niy,
                                                       h->npl, h->p.nx, h->p.ny, 0);
  PF_LAUNCHED(h);
  return PF_OK;
}

int check_status(pf_handle *h) {
  PF_CUDA(cudaMemcpyAsync(h->h_status, h->d_status, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                          h->stream));
  PF_CUDA(cudaStreamSynchronize(h->stream));
  if (*h->h_status != 0u) {
    h->err = "adjoint run: a macroparticle left the window or the mesh (the adjoint needs a "
             "window that holds the beam for the whole run)";
    return PF_OUT_OF_WINDOW;
  }
  return PF_OK;
}

// Run segment seg forward from its checkpoint, keeping every step in the
// store; with save_next, write the next segment's checkpoint.
int run_segment(pf_handle *h, AdjCtx &c, int seg, bool save_next) {
  const size_t pb = (size_t)c.np * sizeof(double), wb = (size_t)c.nwin * sizeof(double);
  const size_t ob = (size_t)c.nouter * sizeof(double);
  double *ck = c.ckpt + (size_t)seg * ckpt_doubles(c);
  StepPtrs s0 = slot(c, 0);
  for (int j = 0; j < 6; ++j)
    PF_CUDA(cudaMemcpyAsync(s0.y[j], ck + j * c.np, pb, cudaMemcpyDeviceToDevice, h->stream));
  if (c.mixed) {  // one float2 per node: the window and the outer mesh in one array each
    PF_CUDA(cudaMemcpyAsync(s0.wr, ck + 6 * c.np, wb, cudaMemcpyDeviceToDevice, h->stream));
    PF_CUDA(cudaMemcpyAsync(h->oc32, ck + 6 * c.np + 2 * c.nwin, ob, cudaMemcpyDeviceToDevice,
                            h->stream));
  } else {
    PF_CUDA(cudaMemcpyAsync(s0.wr, ck + 6 * c.np, wb, cudaMemcpyDeviceToDevice, h->stream));
    PF_CUDA(cudaMemcpyAsync(s0.wi, ck + 6 * c.np + c.nwin, wb, cudaMemcpyDeviceToDevice,
                            h->stream));
    PF_CUDA(cudaMemcpyAsync(h->or_, ck + 6 * c.np + 2 * c.nwin, ob, cudaMemcpyDeviceToDevice,
                            h->stream));
    PF_CUDA(cudaMemcpyAsync(h->oi_, ck + 6 * c.np + 2 * c.nwin + c.nouter, ob,
                            cudaMemcpyDeviceToDevice, h->stream));
  }
  const int first = seg * c.K + 1, last = std::min(c.nsteps, (seg + 1) * c.K);
  const double lenz2 = h->p.dz2 * (double)(h->p.nz2 - 1);
  const int redist = h->p.redist_every > 0 ? h->p.redist_every : 60;
  for (int n = first; n <= last; ++n) {
    const int k = n - first;
    // the output goes to slot k+1, or to the handle's state after the last step
    StepPtrs nx = slot(c, k + 1);
    double *yout[6];
    double *woutr, *wouti;
    const bool end = (n == last);
    for (int j = 0; j < 6; ++j) yout[j] = end ? h->y[h->cur][j] : nx.y[j];
    woutr = end ? (c.mixed ? (double *)h->w32 : h->wr) : nx.wr;
    wouti = end ? h->wi : nx.wi;
    double szl = 0.0;
    for (int q = 1; q < n; ++q) szl = szl + c.hstep;
    int rc = c.mixed ? record_step_mixed(h, c, k, szl, yout, (float2 *)woutr)
                     : record_step(h, c, k, szl, yout, woutr, wouti);
    if (rc) return rc;
    if (c.qdiff && (n % c.every == 0 || n == c.nsteps)) {
      const double dz = diff_after(n, c.nsteps, c.every, c.hstep);
      rc = c.mixed ? diffract_window_c32(h, (float2 *)woutr, dz)
                   : diffract_window(h, woutr, wouti, dz);
      if (rc) return rc;
    }
    if (h->p.mesh_type == PF_MESH_PERIODIC && (c.csteps0 + n) % redist == 0) {
      // the periodic wrap (para_field.f90:212-215) of the step's output z2;
      // its derivative is one, so the adjoint passes through it
      k_wrap<<<grid_for(c.np, 256), 256, 0, h->stream>>>(yout[2], c.np, lenz2);
      PF_LAUNCHED(h);
    }
  }
  if (save_next && last < c.nsteps) {
    double *nk = c.ckpt + (size_t)(seg + 1) * ckpt_doubles(c);
    for (int j = 0; j < 6; ++j)
      PF_CUDA(cudaMemcpyAsync(nk + j * c.np, h->y[h->cur][j], pb, cudaMemcpyDeviceToDevice,
                              h->stream));
    if (c.mixed) {
      PF_CUDA(cudaMemcpyAsync(nk + 6 * c.np, h->w32, wb, cudaMemcpyDeviceToDevice, h->stream));
      PF_CUDA(cudaMemcpyAsync(nk + 6 * c.np + 2 * c.nwin, h->oc32, ob, cudaMemcpyDeviceToDevice,
                              h->stream));
    } else {
      PF_CUDA(cudaMemcpyAsync(nk + 6 * c.np, h->wr, wb, cudaMemcpyDeviceToDevice, h->stream));
      PF_CUDA(cudaMemcpyAsync(nk + 6 * c.np + c.nwin, h->wi, wb, cudaMemcpyDeviceToDevice,
                              h->stream));
      PF_CUDA(cudaMemcpyAsync(nk + 6 * c.np + 2 * c.nwin, h->or_, ob, cudaMemcpyDeviceToDevice,
                              h->stream));
      PF_CUDA(cudaMemcpyAsync(nk + 6 * c.np + 2 * c.nwin + c.nouter, h->oi_, ob,
                              cudaMemcpyDeviceToDevice, h->stream));
    }
  }
  return check_status(h);
}

}  // namespace

extern "C" {

int pf_diffract_adjoint(pf_handle *h, double dz, double *re, double *im) {
  if (!h || !re || !im) return PF_BAD_ARG;
  if (h->p.precision != PF_FP64) {
    h->err = "the diffraction adjoint runs on the FP64 path";
    return PF_BAD_ARG;
  }
  cudaSetDevice(h->dev);
  const size_t ob = (size_t)h->nouter * sizeof(double);
  double *d = nullptr;
  PF_CUDA(cudaMalloc(&d, 2 * ob));
  int rc = PF_OK;
  do {
    if (cudaMemcpyAsync(d, re, ob, cudaMemcpyDefault, h->stream) != cudaSuccess ||
        cudaMemcpyAsync(d + h->nouter, im, ob, cudaMemcpyDefault, h->stream) != cudaSuccess) {
      rc = PF_CUDA_ERR;
      break;
    }
    rc = pf_diffract_adjoint_split(h, d, d + h->nouter, dz);
    if (rc) break;
    if (cudaMemcpyAsync(re, d, ob, cudaMemcpyDefault, h->stream) != cudaSuccess ||
        cudaMemcpyAsync(im, d + h->nouter, ob, cudaMemcpyDefault, h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess)
      rc = PF_CUDA_ERR;
  } while (0);
  cudaFree(d);
  if (rc == PF_CUDA_ERR) h->err = "pf_diffract_adjoint: CUDA copy failed";
  return rc;
}

int pf_adjoint_forward(pf_handle *h, int32_t nsteps, int32_t isteps4diff, int32_t qdiffraction,
                       double hstep, int32_t checkpoint_every, const double *seed_re,
                       const double *seed_im, double seed_amp, double chirp, double *energy) {
  if (!h || !seed_re || !seed_im || !energy || nsteps < 1 || checkpoint_every < 1 ||
      (qdiffraction && isteps4diff < 1) || !(hstep > 0.0))
    return PF_BAD_ARG;
  if (!h->particles_set || h->nwin == 0 || h->np == 0) {
    h->err = "adjoint run: particles not set";
    return PF_STATE;
  }
  if (h->prof_z.empty()) {
    h->err = "adjoint run: set a taper profile (pf_set_taper_profile) first";
    return PF_STATE;
  }
  cudaSetDevice(h->dev);
  if (!h->adj) h->adj = new AdjCtx();
  AdjCtx &c = *h->adj;
  const bool realloc = c.np != h->np || c.nwin != h->nwin || c.nouter != h->nouter ||
                       c.K != checkpoint_every || c.nsteps != nsteps;
  c.np = h->np;
  c.nwin = h->nwin;
  c.nouter = h->nouter;
  c.K = checkpoint_every;
  c.nsteps = nsteps;
  c.every = isteps4diff;
  c.qdiff = qdiffraction;
  c.hstep = hstep;
  c.seed_amp = seed_amp;
  c.chirp = chirp;
  c.nseg = (nsteps + c.K - 1) / c.K;
  c.csteps0 = h->csteps;
  c.mixed = (h->p.precision == PF_MIXED);
  const size_t pb = (size_t)c.np * sizeof(double);
  const size_t ob = (size_t)c.nouter * sizeof(double);
  if (realloc || !c.base) {
    cudaFree(c.base);
    cudaFree(c.seed);
    cudaFree(c.ckpt);
    cudaFree(c.store);
    cudaFree(c.work);
    cudaFree(c.galpha);
    cudaFree(c.fin);
    c.base = c.seed = c.ckpt = c.store = c.work = c.galpha = c.fin = nullptr;
    PF_CUDA(cudaMalloc(&c.fin, 2 * ob));
    PF_CUDA(cudaMalloc(&c.base, 6 * pb));
    PF_CUDA(cudaMalloc(&c.seed, 2 * ob));
    PF_CUDA(cudaMalloc(&c.ckpt, sizeof(double) * ckpt_doubles(c) * (size_t)c.nseg));
    PF_CUDA(cudaMalloc(&c.store, sizeof(double) * slot_doubles(c) * (size_t)(c.K + 1)));
    PF_CUDA(cudaMalloc(&c.work, sizeof(double) * (24 * (size_t)c.np + 10 * (size_t)c.nwin +
                                                  2 * (size_t)c.nouter + 8)));
    PF_CUDA(cudaMalloc(&c.galpha, sizeof(double) * 4 * (size_t)nsteps));
  }
  // base beam (chirp 0) and seed
  for (int j = 0; j < 6; ++j)
    PF_CUDA(cudaMemcpyAsync(c.base + j * c.np, h->y[h->cur][j], pb, cudaMemcpyDeviceToDevice,
                            h->stream));
  PF_CUDA(cudaMemcpyAsync(c.seed, seed_re, ob, cudaMemcpyDefault, h->stream));
  PF_CUDA(cudaMemcpyAsync(c.seed + c.nouter, seed_im, ob, cudaMemcpyDefault, h->stream));
  // <z2> of the base beam (host, fixed order)
  {
    std::vector<double> z((size_t)c.np);
    PF_CUDA(cudaMemcpyAsync(z.data(), c.base + 2 * c.np, pb, cudaMemcpyDeviceToHost, h->stream));
    PF_CUDA(cudaStreamSynchronize(h->stream));
    double s = 0.0;
    for (double v : z) s += v;
    c.zmean = s / (double)c.np;
  }
  // initial state: chirped beam, outer = seed_amp seed, window from it
  double *ck0 = c.ckpt;
  for (int j = 0; j < 6; ++j)
    PF_CUDA(cudaMemcpyAsync(ck0 + j * c.np, c.base + j * c.np, pb, cudaMemcpyDeviceToDevice,
                            h->stream));
  k_chirp<<<grid_for(c.np, 256), 256, 0, h->stream>>>(c.np, ck0 + 2 * c.np, ck0 + 5 * c.np, chirp,
                                                       c.zmean);
  PF_LAUNCHED(h);
  double *o0r = ck0 + 6 * c.np + 2 * c.nwin, *o0i = o0r + c.nouter;
  if (c.mixed) {
    // the complex-float outer mesh and window (one array each)
    float2 *o0 = (float2 *)o0r, *w0 = (float2 *)(ck0 + 6 * c.np);
    k_seed_c32<<<grid_for(c.nouter, 256), 256, 0, h->stream>>>(c.nouter, c.seed,
                                                                c.seed + c.nouter, o0, seed_amp);
    PF_LAUNCHED(h);
    k_win_c32<<<grid_for(c.nwin, 256), 256, 0, h->stream>>>(w0, o0, h->nix, h->niy, h->npl,
                                                            h->p.nx, h->p.ny, 0);
    PF_LAUNCHED(h);
    if (qdiffraction) {  // the first half step of diffraction (undulator.f90:156-161)
      PF_CUDA(cudaMemcpyAsync(h->oc32, o0, ob, cudaMemcpyDeviceToDevice, h->stream));
      int rc = diffract_window_c32(h, w0, diff_after(0, nsteps, isteps4diff, hstep));
      if (rc) return rc;
      PF_CUDA(cudaMemcpyAsync(o0, h->oc32, ob, cudaMemcpyDeviceToDevice, h->stream));
    }
  } else {
    k_scale2<<<grid_for(c.nouter, 256), 256, 0, h->stream>>>(c.nouter, c.seed, c.seed + c.nouter,
                                                              o0r, o0i, seed_amp);
    PF_LAUNCHED(h);
    k_win<<<grid_for(c.nwin, 256), 256, 0, h->stream>>>(ck0 + 6 * c.np, ck0 + 6 * c.np + c.nwin,
                                                        o0r, o0i, h->nix, h->niy, h->npl, h->p.nx,
                                                        h->p.ny, 0);
    PF_LAUNCHED(h);
    if (qdiffraction) {  // the first half step of diffraction (undulator.f90:156-161)
      PF_CUDA(cudaMemcpyAsync(h->or_, o0r, ob, cudaMemcpyDeviceToDevice, h->stream));
      PF_CUDA(cudaMemcpyAsync(h->oi_, o0i, ob, cudaMemcpyDeviceToDevice, h->stream));
      int rc = diffract_window(h, ck0 + 6 * c.np, ck0 + 6 * c.np + c.nwin,
                               diff_after(0, nsteps, isteps4diff, hstep));
      if (rc) return rc;
      PF_CUDA(cudaMemcpyAsync(o0r, h->or_, ob, cudaMemcpyDeviceToDevice, h->stream));
      PF_CUDA(cudaMemcpyAsync(o0i, h->oi_, ob, cudaMemcpyDeviceToDevice, h->stream));
    }
  }
  PF_CUDA(cudaMemsetAsync(h->d_status, 0, sizeof(unsigned int), h->stream));
  for (int seg = 0; seg < c.nseg; ++seg) {
    int rc = run_segment(h, c, seg, true);
    if (rc) return rc;
  }
  // final field on the outer mesh and its energy
  const int64_t nuniq = (int64_t)h->p.nx * h->p.ny * h->npl;
  double *dot = c.work;
  if (c.mixed) {
    k_win_c32<<<grid_for(c.nwin, 256), 256, 0, h->stream>>>(
        (float2 *)h->w32, (float2 *)h->oc32, h->nix, h->niy, h->npl, h->p.nx, h->p.ny, 1);
    PF_LAUNCHED(h);
    k_dot_c32<<<1, 256, 0, h->stream>>>(nuniq, (const float2 *)h->oc32, (const float2 *)h->oc32,
                                        nullptr, nullptr, dot);
    PF_LAUNCHED(h);
  } else {
    k_win<<<grid_for(c.nwin, 256), 256, 0, h->stream>>>(h->wr, h->wi, h->or_, h->oi_, h->nix,
                                                        h->niy, h->npl, h->p.nx, h->p.ny, 1);
    PF_LAUNCHED(h);
    k_dot2<<<1, 256, 0, h->stream>>>(nuniq, h->or_, h->oi_, h->or_, h->oi_, dot);
    PF_LAUNCHED(h);
  }
  double e = 0.0;
  PF_CUDA(cudaMemcpyAsync(&e, dot, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  PF_CUDA(cudaStreamSynchronize(h->stream));
  c.energy = e * h->p.dx * h->p.dy * h->p.dz2;
  *energy = c.energy;
  // keep the final field for the backward pass; the handle's particles
  // return to the unchirped beam
  if (c.mixed) {
    PF_CUDA(cudaMemcpyAsync(c.fin, h->oc32, ob, cudaMemcpyDeviceToDevice, h->stream));
  } else {
    PF_CUDA(cudaMemcpyAsync(c.fin, h->or_, ob, cudaMemcpyDeviceToDevice, h->stream));
    PF_CUDA(cudaMemcpyAsync(c.fin + c.nouter, h->oi_, ob, cudaMemcpyDeviceToDevice, h->stream));
  }
  for (int j = 0; j < 6; ++j)
    PF_CUDA(cudaMemcpyAsync(h->y[h->cur][j], c.base + j * c.np, pb, cudaMemcpyDeviceToDevice,
                            h->stream));
  PF_CUDA(cudaStreamSynchronize(h->stream));
  c.ready = true;
  return PF_OK;
}

int pf_adjoint_backward(pf_handle *h, double denergy, double *g_taper, int32_t ntaper,
                        double *g_seed, double *g_chirp) {
  if (!h || !h->adj || !h->adj->ready) return PF_STATE;
  AdjCtx &c = *h->adj;
  if (!g_taper || ntaper != (int32_t)h->prof_z.size() || !g_seed || !g_chirp) return PF_BAD_ARG;
  cudaSetDevice(h->dev);
  const double hs = c.hstep, hh = 0.5 * hs;
  const int64_t np = c.np, nw = c.nwin, no = c.nouter;
  // adjoint state
  double *w = c.work + 8;
  double *ly[6], *lsa[6], *lsb[6], *lsum[6];
  for (int j = 0; j < 6; ++j) {
    ly[j] = w + j * np;
    lsa[j] = w + (6 + j) * np;
    lsb[j] = w + (12 + j) * np;
    lsum[j] = w + (18 + j) * np;
  }
  double *q = w + 24 * np;
  double *lWr = q, *lWi = q + nw, *lAr = q + 2 * nw, *lAi = q + 3 * nw;
  double *lWsr = q + 4 * nw, *lWsi = q + 5 * nw, *nur = q + 6 * nw, *nui = q + 7 * nw;
  double *lFr = q + 10 * nw, *lFi = lFr + no;
  const size_t pb = (size_t)np * sizeof(double), wb = (size_t)nw * sizeof(double);
  const size_t ob = (size_t)no * sizeof(double);

  // the mixed form keeps each complex field adjoint as one float2 array in
  // the space of its re part
  float2 *lW = (float2 *)lWr, *lA = (float2 *)lAr, *lWs = (float2 *)lWsr, *nu = (float2 *)nur;
  float2 *lF = (float2 *)lFr;
  // after each step the running sums become the next step's adjoint state:
  // the two sets of arrays trade places (the step's first adjoint stage
  // initialises the sums from the state)
  auto swap_state = [&]() {
    for (int j = 0; j < 6; ++j) std::swap(ly[j], lsum[j]);
    std::swap(lWr, lWsr);
    std::swap(lWi, lWsi);
    std::swap(lW, lWs);
  };
  const unsigned gw = grid_for(nw, 256);
  // window <-> outer mesh of the field adjoint
  auto win = [&](int to_outer) {
    if (c.mixed)
      k_win_c32<<<gw, 256, 0, h->stream>>>(lW, lF, h->nix, h->niy, h->npl, h->p.nx, h->p.ny,
                                           to_outer);
    else
      k_win<<<gw, 256, 0, h->stream>>>(lWr, lWi, lFr, lFi, h->nix, h->niy, h->npl, h->p.nx,
                                       h->p.ny, to_outer);
  };
  auto diffract_adj = [&](double dz) {
    return c.mixed ? pf_diffract_adjoint_c32(h, lF, dz) : pf_diffract_adjoint_split(h, lFr, lFi, dz);
  };

  // dE/dF = 2 dV F over the unique planes (c.fin holds the final field)
  const double dV = h->p.dx * h->p.dy * h->p.dz2;
  const int64_t nuniq = (int64_t)h->p.nx * h->p.ny * h->npl;
  PF_CUDA(cudaMemsetAsync(lFr, 0, 2 * ob, h->stream));
  if (c.mixed)
    k_scale_c32<<<grid_for(nuniq, 256), 256, 0, h->stream>>>(nuniq, (const float2 *)c.fin, lF,
                                                             (float)(2.0 * dV * denergy));
  else
    k_scale2<<<grid_for(nuniq, 256), 256, 0, h->stream>>>(nuniq, c.fin, c.fin + c.nouter, lFr,
                                                          lFi, 2.0 * dV * denergy);
  PF_LAUNCHED(h);
  win(0);
  PF_LAUNCHED(h);
  PF_CUDA(cudaMemsetAsync(w, 0, 24 * pb, h->stream));
  PF_CUDA(cudaMemsetAsync(lAr, 0, 2 * wb, h->stream));
  PF_CUDA(cudaMemsetAsync(c.galpha, 0, sizeof(double) * 4 * (size_t)c.nsteps, h->stream));
  StageArgs base;
  PfMixConst kc;
  if (c.mixed)
    pf_mixed_constants(h, &kc);
  else
    pf_fill_stage_args(h, base, hs / 6.0);

  for (int seg = c.nseg - 1; seg >= 0; --seg) {
    int rc = run_segment(h, c, seg, false);
    if (rc) return rc;
    const int first = seg * c.K + 1, last = std::min(c.nsteps, (seg + 1) * c.K);
    for (int n = last; n >= first; --n) {
      // diffraction after step n
      if (c.qdiff) {
        const double dz = diff_after(n, c.nsteps, c.every, hs);
        if (n % c.every == 0 || n == c.nsteps) {
          win(1);
          PF_LAUNCHED(h);
          if (dz != 0.0) {
            rc = diffract_adj(dz);
            if (rc) return rc;
          }
          win(0);
          PF_LAUNCHED(h);
        }
      }
      // step n's adjoint from the recorded slot
      StepPtrs S = slot(c, n - first);
      double szl = 0.0;
      for (int t = 1; t < n; ++t) szl = szl + hs;
      const double sz[4] = {szl, szl + hh, szl + hh, szl + hs};
      const double cs[4] = {0.0, hh, hh, hs};         // state: y + c k_{s-1}
      const double ma[4] = {hs / 6.0, hs / 3.0, hs / 3.0, hs / 6.0};
      const double mb[4] = {hs / 2.0, hs / 2.0, hs, 0.0};  // next-stage weight of ls_{s+1}
      double *const *kin[4] = {nullptr, S.k1, S.k2, S.k3};
      const double *din_r[4] = {nullptr, S.d1r, S.d2r, S.d3r};
      const double *din_i[4] = {nullptr, S.d1i, S.d2i, S.d3i};
      // the last stage's nu is h/6 lW', read from lW' with that scale
      double **lcur = lsa, **lprev = lsb;
      for (int s = 3; s >= 0; --s) {
        const double na = (s > 0) ? ma[s - 1] : 0.0, nb = (s > 0) ? mb[s - 1] : 0.0;
        if (c.mixed) {
          VjpMixArgs v;
          memset(&v, 0, sizeof(v));
          for (int j = 0; j < 6; ++j) {
            v.y[j] = S.y[j];
            v.kin_f[j] = kin[s] ? (const float *)kin[s][j] : nullptr;
            v.lnext[j] = ly[j];
            v.lprev[j] = (s == 3) ? nullptr : lprev[j];
            v.ls[j] = lcur[j];
            v.lsum[j] = lsum[j];
          }
          v.kin_z = kin[s] ? kin[s][2] : nullptr;
          v.c = cs[s];
          v.c_f = (float)cs[s];
          v.w = (const float2 *)S.wr;
          v.d = (const float2 *)din_r[s];
          v.cA_f = (float)cs[s];
          v.ma = ma[s];
          v.mb = (s == 3) ? 0.0 : mb[s];
          v.nu = (s == 3) ? lW : nu;
          v.nus = (s == 3) ? (float)(hs / 6.0) : 1.f;
          v.lsum_init = (s == 3);
          v.la = lA;
          v.galpha = c.galpha + 4 * (size_t)(n - 1) + s;
          v.chi_f = h->chi_f;
          v.np = np;
          v.npl = h->npl;
          v.nz2 = h->p.nz2;
          v.nix = h->nix;
          v.niy = h->niy;
          v.periodic = (h->p.mesh_type == PF_MESH_PERIODIC);
          v.one_d = h->p.one_d;
          v.k = kc;
          v.inv_eta_f = (float)kc.inv_eta;
          v.aw2g_f = (float)kc.aw2g;
          v.inv_dz2_f = (float)kc.inv_dz2;
          double n2col;
          int place;
          pf_taper_stage(h, sz[s], &n2col, &place);
          BFieldCoef bf;
          pf_stage_coefficients(h->p, sz[s], n2col, place, &bf);
          v.bf = to_float(bf);
          v.n2col = (float)n2col;
          v.kn2col = (float)(h->p.kappa * n2col);
          v.kappa = (float)h->p.kappa;
          v.field_evolve = h->p.field_evolve;
          v.electrons_evolve = h->p.electrons_evolve;
          v.coupling = h->p.coupling;
          k_vjp_mixed<<<grid_for(np, 256), 256, 0, h->stream>>>(v);
          PF_LAUNCHED(h);
          // nu for the stage before: ma' lW' + mb' lA_s; lWsum += lA_s
          k_adj_nodes_c32<<<gw, 256, 0, h->stream>>>(nw, lW, lA, lWs, nu, (float)na, (float)nb,
                                                     s == 3);
          PF_LAUNCHED(h);
        } else {
          VjpArgs v;
          memset(&v, 0, sizeof(v));
          v.st = base;
          stage_setup(h, sz[s], v.st);
          for (int j = 0; j < 6; ++j) {
            v.y[j] = S.y[j];
            v.kin[j] = kin[s] ? kin[s][j] : nullptr;
            v.lnext[j] = ly[j];
            v.lprev[j] = (s == 3) ? nullptr : lprev[j];
            v.ls[j] = lcur[j];
            v.lsum[j] = lsum[j];
          }
          v.c = cs[s];
          v.wr = S.wr;
          v.wi = S.wi;
          v.dr = din_r[s];
          v.di = din_i[s];
          v.cA = cs[s];
          v.ma = ma[s];
          v.mb = (s == 3) ? 0.0 : mb[s];
          v.nur = (s == 3) ? lWr : nur;
          v.nui = (s == 3) ? lWi : nui;
          v.nus = (s == 3) ? hs / 6.0 : 1.0;
          v.lsum_init = (s == 3);
          v.lar = lAr;
          v.lai = lAi;
          v.galpha = c.galpha + 4 * (size_t)(n - 1) + s;
          k_vjp<<<grid_for(np, 256), 256, 0, h->stream>>>(v);
          PF_LAUNCHED(h);
          // nu for the stage before: ma' lW' + mb' lA_s; lWsum += lA_s
          k_adj_nodes<<<gw, 256, 0, h->stream>>>(nw, lWr, lWi, lAr, lAi, lWsr, lWsi, nur, nui,
                                                 na, nb, s == 3);
          PF_LAUNCHED(h);
        }
        std::swap(lcur, lprev);
      }
      swap_state();
    }
  }
  // the first half step of diffraction, then the window adjoint into the field
  win(1);
  PF_LAUNCHED(h);
  if (c.qdiff) {
    int rc = diffract_adj(diff_after(0, c.nsteps, c.every, hs));
    if (rc) return rc;
  }
  // gradients
  const int64_t nuq = (int64_t)h->p.nx * h->p.ny * h->npl;
  double *dots = c.work;  // [0] seed, [1] chirp
  if (c.mixed)
    k_dot_c32<<<1, 256, 0, h->stream>>>(nuq, lF, nullptr, c.seed, c.seed + c.nouter, dots);
  else
    k_dot2<<<1, 256, 0, h->stream>>>(nuq, lFr, lFi, c.seed, c.seed + c.nouter, dots);
  PF_LAUNCHED(h);
  k_chirp_grad<<<1, 256, 0, h->stream>>>(np, ly[5], c.base + 2 * np, c.zmean, dots + 1);
  PF_LAUNCHED(h);
  double hd[2];
  std::vector<double> ga((size_t)4 * c.nsteps);
  PF_CUDA(cudaMemcpyAsync(hd, dots, sizeof(hd), cudaMemcpyDeviceToHost, h->stream));
  PF_CUDA(cudaMemcpyAsync(ga.data(), c.galpha, sizeof(double) * ga.size(), cudaMemcpyDeviceToHost,
                          h->stream));
  PF_CUDA(cudaStreamSynchronize(h->stream));
  *g_seed = hd[0];
  *g_chirp = hd[1];
  // alpha(sz) = sum_k phi_k(sz) a_k, piecewise linear
  const std::vector<double> &pz = h->prof_z;
  const int nk = (int)pz.size();
  for (int k = 0; k < nk; ++k) g_taper[k] = 0.0;
  for (int n = 1; n <= c.nsteps; ++n) {
    double szl = 0.0;
    for (int t = 1; t < n; ++t) szl = szl + hs;
    const double sz[4] = {szl, szl + hh, szl + hh, szl + hs};
    for (int s = 0; s < 4; ++s) {
      const double g = ga[(size_t)4 * (n - 1) + s];
      const double x = sz[s];
      if (x <= pz[0]) {
        g_taper[0] += g;
      } else if (x >= pz[nk - 1]) {
        g_taper[nk - 1] += g;
      } else {
        const int k = (int)(std::upper_bound(pz.begin(), pz.end(), x) - pz.begin()) - 1;
        const double t = (x - pz[k]) / (pz[k + 1] - pz[k]);
        g_taper[k] += g * (1.0 - t);
        g_taper[k + 1] += g * t;
      }
    }
  }
  // the handle's particles return to the base beam
  for (int j = 0; j < 6; ++j)
    PF_CUDA(cudaMemcpyAsync(h->y[h->cur][j], c.base + j * np, pb, cudaMemcpyDeviceToDevice,
                            h->stream));
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

}  // extern "C"
