/*
 * CPU oracle for the Puffin RK4 macroparticle push (TEST INFRASTRUCTURE ONLY;
 * see puffin_oracle.h for the parity anchors).  Compiled with
 * -ffp-contract=off so every operation is individually rounded in the order
 * the reference's Fortran expressions are written.
 */
#include "puffin_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

void or_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}

/* Puffin's pi is a default-kind (single precision) literal promoted to
 * double: puffin/lib/common/puffin_constants.f90:22. */
static const double PUFFIN_PI = (double)3.14159265358979323846f;

/* ------------------------------------------------------------------------ */
/* Taper and undulator section: wiggler_taper.f90:39-47, puffin_equations.f90:218-254 */
static double profile_at(const or_taper *t, double sz) {
  const int n = t->nprof;
  if (sz <= t->pz[0]) return t->pa[0];
  if (sz >= t->pz[n - 1]) return t->pa[n - 1];
  int k = 0;
  while (k + 1 < n && t->pz[k + 1] <= sz) ++k;
  const double u = (sz - t->pz[k]) / (t->pz[k + 1] - t->pz[k]);
  return t->pa[k] + u * (t->pa[k + 1] - t->pa[k]);
}

void or_stage_setup(const or_params *p, or_taper *t, double sz, or_stage *out) {
  if (t->nprof > 1) {
    t->n2col = profile_at(t, sz);
  } else if ((sz >= p->szfs) && (sz <= p->szfe)) {
    t->n2col = t->n2col0 + t->undgrad * (sz - p->szfs);
  } else if (sz > p->szfe) {
    t->n2col0 = t->n2col;
  }
  out->sz = sz;
  out->n2col = t->n2col;
  if (p->und_ends) {
    if (sz <= p->szfs) out->place = OR_PLACE_START;
    else if (sz >= p->szfe) out->place = OR_PLACE_END;
    else out->place = OR_PLACE_MAIN;
  } else {
    out->place = OR_PLACE_MAIN;
  }
}

/* gamma_to_p2.f90:84-85 */
double or_p2(double gam, double px, double py, double eta, double g0, double aw) {
  double a = 1.0 / ((g0 * g0) * (gam * gam));
  double b = 1.0 + (aw * aw) * ((px * px) + (py * py));
  return ((1.0 / sqrt(1.0 - a * b)) - 1.0) / eta;
}

/* ------------------------------------------------------------------------ */
/* Undulator fields: bfields.f90 getBXfield :59-309, getBYfield :313-523,
 * getBZfield :528-881.  Expression order follows the Fortran source. */
void or_bfield(const or_params *p, const or_stage *st, double x, double y,
               double *bx_, double *by_, double *bz_) {
  const double pi = PUFFIN_PI, rho = p->rho, sz = st->sz;
  const double seta = sqrt(p->eta);
  const int type = p->und_type, place = st->place;
  double szt, bx = 0.0, by = 0.0, bz = 0.0;

  /* ---- bx ---- */
  szt = sz / 2.0 / rho;
  if (type == OR_UND_CURVED) {
    double kx = p->kx_und, ky = p->ky_und;
    if (place == OR_PLACE_START) {
      bx = kx / ky * sinh(kx * x) * sinh(ky * y) * szt / 4.0 / pi * sin(szt);
    } else if (place == OR_PLACE_END) {
      szt = (sz - p->szfe) / 2.0 / rho;
      bx = kx / ky * sinh(kx * x) * sinh(ky * y) * (-szt / 4.0 / pi + 1.0) * sin(szt);
    } else {
      bx = kx / ky * sinh(kx * x) * sinh(ky * y) * sin(szt);
    }
  } else if (type == OR_UND_PLANEPOLE) {
    bx = 0.0;
  } else {
    double f = (type == OR_UND_HELICAL) ? 1.0 : p->fx;
    int hel = (type == OR_UND_HELICAL);
    if (place == OR_PLACE_START) {
      bx = hel ? (sz - pi * rho) / (6.0 * pi * rho) * cos(szt)
               : f * (sz - pi * rho) / (6.0 * pi * rho) * cos(szt);
      if (sz < pi * rho) bx = 0.0;
      else if (sz > 7.0 * pi * rho) bx = hel ? cos(szt) : f * cos(szt);
    } else if (place == OR_PLACE_END) {
      double s2 = sz - p->szfe;
      bx = hel ? -((s2 - 7.0 * pi * rho) / (6.0 * pi * rho) * cos(s2 / 2.0 / rho))
               : -(f * (s2 - 7.0 * pi * rho) / (6.0 * pi * rho) * cos(s2 / 2.0 / rho));
      if (s2 < pi * rho) bx = hel ? cos(s2 / 2.0 / rho) : f * cos(s2 / 2.0 / rho);
      else if (s2 > 7.0 * pi * rho) bx = 0.0;
    } else {
      bx = hel ? cos(szt) : f * cos(szt);
    }
  }
  if (p->focusing) bx = seta * (p->kbysf * p->kbysf) / p->kappa * y + bx;

  /* ---- by ---- */
  szt = sz / 2.0 / rho;
  if (type == OR_UND_CURVED) {
    double kx = p->kx_und, ky = p->ky_und;
    if (place == OR_PLACE_START) {
      by = cosh(kx * x) * cosh(ky * y) * szt / 4.0 / pi * sin(szt);
    } else if (place == OR_PLACE_END) {
      szt = (sz - p->szfe) / 2.0 / rho;
      by = cosh(kx * x) * cosh(ky * y) * (-szt / 4.0 / pi + 1.0) * sin(szt);
    } else {
      by = cosh(kx * x) * cosh(ky * y) * sin(szt);
    }
  } else if (type == OR_UND_PLANEPOLE || type == OR_UND_HELICAL) {
    if (place == OR_PLACE_START) {
      by = szt / 4.0 / pi * sin(szt);
    } else if (place == OR_PLACE_END) {
      szt = (sz - p->szfe) / 2.0 / rho;
      by = (-szt / 4.0 / pi + 1.0) * sin(szt);
    } else {
      by = sin(szt);
    }
  } else {
    double f = p->fy;
    if (place == OR_PLACE_START) {
      by = f * szt / 4.0 / pi * sin(szt);
    } else if (place == OR_PLACE_END) {
      szt = (sz - p->szfe) / 2.0 / rho;
      by = f * (-szt / 4.0 / pi + 1.0) * sin(szt);
    } else {
      by = f * sin(szt);
    }
  }
  if (p->focusing) by = -(seta * (p->kbxsf * p->kbxsf) / p->kappa * x) + by;

  /* ---- bz ---- */
  szt = sz / 2.0 / rho;
  if (p->one_d) {
    bz = 0.0;
  } else if (type == OR_UND_CURVED) {
    double kx = p->kx_und, ky = p->ky_und;
    if (place == OR_PLACE_START) {
      bz = seta / 2.0 / rho / ky * cosh(kx * x) * sinh(ky * y) * (szt / 4.0 / pi) * cos(szt);
    } else if (place == OR_PLACE_END) {
      szt = (sz - p->szfe) / 2.0 / rho;
      bz = seta / 2.0 / rho / kx * cosh(kx * x) * sinh(ky * y) * (-szt / 4.0 / pi + 1.0) * cos(szt);
    } else {
      bz = seta / 2.0 / rho / kx * cosh(kx * x) * sinh(ky * y) * cos(szt);
    }
  } else if (type == OR_UND_PLANEPOLE) {
    if (place == OR_PLACE_START) {
      bz = sinh(seta / 2.0 / rho * y) * (szt / 4.0 / pi) * cos(szt);
    } else if (place == OR_PLACE_END) {
      szt = (sz - p->szfe) / 2.0 / rho;
      bz = sinh(seta / 2.0 / rho * y) * (-szt / 4.0 / pi + 1.0) * cos(szt);
    } else {
      bz = sinh(seta / 2.0 / rho * y) * cos(szt);
    }
  } else {
    int hel = (type == OR_UND_HELICAL);
    double fx = p->fx, fy = p->fy;
    if (place == OR_PLACE_START) {
      bz = hel ? -(seta / 2.0 / rho * (sz - pi * rho) / (6.0 * pi * rho) * x * sin(szt))
               : -(seta / 2.0 / rho * (sz - pi * rho) / (6.0 * pi * rho) * fx * x * sin(szt));
      if (sz < pi * rho) bz = 0.0;
      else if (sz > 7.0 * pi * rho)
        bz = hel ? -(seta / 2.0 / rho * x * sin(szt)) : -(seta / 2.0 / rho * fx * x * sin(szt));
      bz = hel ? bz + szt / 4.0 / pi * seta / 2.0 / rho * y * cos(szt)
               : bz + szt / 4.0 / pi * seta / 2.0 / rho * fy * y * cos(szt);
    } else if (place == OR_PLACE_END) {
      double s2 = sz - p->szfe;
      bz = hel ? -(seta / 2.0 / rho * (s2 - 7.0 * pi * rho) / (6.0 * pi * rho) * x * sin(s2 / 2.0 / rho))
               : -(seta / 2.0 / rho * (s2 - 7.0 * pi * rho) / (6.0 * pi * rho) * fx * x * sin(s2 / 2.0 / rho));
      if (s2 < pi * rho)
        bz = hel ? -(seta / 2.0 / rho * x * sin(s2 / 2.0 / rho))
                 : -(seta / 2.0 / rho * fx * x * sin(s2 / 2.0 / rho));
      else if (s2 > 7.0 * pi * rho) bz = 0.0;
      bz = hel ? bz + (-(s2 / 8.0 / pi / rho) + 1.0) * seta / 2.0 / rho * y * cos(s2 / 2.0 / rho)
               : bz + (-(s2 / 8.0 / pi / rho) + 1.0) * seta / 2.0 / rho * fy * y * cos(s2 / 2.0 / rho);
    } else {
      bz = hel ? seta / 2.0 / rho * (-(x * sin(szt)) + y * cos(szt))
               : seta / 2.0 / rho * (-(fx * x * sin(szt)) + fy * y * cos(szt));
    }
  }
  *bx_ = bx;
  *by_ = by;
  *bz_ = bz;
}

/* ------------------------------------------------------------------------ */
int64_t or_nplanes(const or_params *p) {
  return p->mesh_type == OR_MESH_PERIODIC ? p->nz2 - 1 : p->nz2;
}

void or_wrap_z2(const or_params *p, int64_t np, double *z2) {
  if (p->mesh_type != OR_MESH_PERIODIC) return;
  double lenz2 = p->dz2 * (double)(p->nz2 - 1);
  for (int64_t i = 0; i < np; ++i) z2[i] = z2[i] - (floor(z2[i] / lenz2) * lenz2);
}

/* getrhs (rhs.f90:60-330) with getInterps / getFFelecs / getSource and the
 * six equations.  Deposit: sequential FP64 accumulation in particle order. */
int or_rhs(const or_params *p, const or_stage *st, int64_t np,
           const double *ar, const double *ai,
           const double *x, const double *y, const double *z2,
           const double *px, const double *py, const double *gam,
           const double *chi,
           double *ddx, double *ddy, double *ddz2, double *dpx, double *dpy,
           double *dgam, double *dadz_r, double *dadz_i) {
  const double dx = p->dx, dy = p->dy, dz2 = p->dz2;
  const double dV3 = p->dx * p->dy * p->dz2; /* rhs.f90:361 */
  const double sInv2rho = 1.0 / (2.0 * p->rho);
  const double halfx = ((double)(p->nix - 1) / 2.0) * dx; /* rhs.f90:395 */
  const double halfy = ((double)(p->niy - 1) / 2.0) * dy;
  const int64_t nix = p->nix, niy = p->niy, ntr = nix * niy;
  const int64_t npl = or_nplanes(p);
  const int periodic = p->mesh_type == OR_MESH_PERIODIC;
  const double eta = p->eta, kappa = p->kappa, rho = p->rho, n2col = st->n2col;
  int status = OR_OK;

  double *sp2 = (double *)malloc(sizeof(double) * (size_t)(np > 0 ? np : 1));
  double *fr = (double *)calloc((size_t)(np > 0 ? np : 1), sizeof(double));
  double *fi = (double *)calloc((size_t)(np > 0 ? np : 1), sizeof(double));
  int64_t *node = (int64_t *)malloc(sizeof(int64_t) * 8 * (size_t)(np > 0 ? np : 1));
  double *w = (double *)malloc(sizeof(double) * 8 * (size_t)(np > 0 ? np : 1));

#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < np; ++i) sp2[i] = or_p2(gam[i], px[i], py[i], eta, p->gamma_r, p->aw);

  /* interpolation weights and node lists (getInterps_3D / _1D) */
#pragma omp parallel for schedule(static) reduction(|:status)
  for (int64_t i = 0; i < np; ++i) {
    /* floor for the node as for the weights (system_interpolation.f90:45-58);
       the reference's p_nodes uses truncating int() (rhs.f90:174-178), which
       agrees for every non-negative argument -- the inputs it defines */
    double z2n = floor(z2[i] / dz2) + 1.0;
    double locz2 = z2[i] - (z2n - 1.0) * dz2;
    int64_t iz = (int64_t)z2n; /* 1-based */
    if (!periodic) {
      if (iz >= p->nz2 || iz < 1) status |= OR_OUT_OF_Z2;
    }
    int64_t pz0, pz1;
    if (periodic) {
      int64_t m = (iz - 1) % npl;
      if (m < 0) m += npl;
      pz0 = m;
      pz1 = (m + 1) % npl;
    } else {
      pz0 = iz - 1;
      pz1 = iz;
    }
    if (p->one_d) {
      double w1 = (1.0 - locz2 / dz2);
      w[8 * i + 0] = w1;
      w[8 * i + 1] = 1.0 - w1;
      node[8 * i + 0] = pz0;
      node[8 * i + 1] = pz1;
    } else {
      double xn = floor((x[i] + halfx) / dx) + 1.0;
      double locx = x[i] + halfx - (xn - 1.0) * dx;
      double x2 = locx / dx, x1 = 1.0 - x2;
      double yn = floor((y[i] + halfy) / dy) + 1.0;
      double locy = y[i] + halfy - (yn - 1.0) * dy;
      double y2 = locy / dy, y1 = 1.0 - y2;
      double z2w = locz2 / dz2, z1w = 1.0 - z2w;
      if (xn >= (double)nix || xn < 1.0 || yn >= (double)niy || yn < 1.0)
        status |= OR_OUT_OF_WINDOW;
      int64_t ix = (int64_t)xn - 1, iy = (int64_t)yn - 1;
      int64_t b0 = ix + iy * nix + pz0 * ntr, b1 = ix + iy * nix + pz1 * ntr;
      w[8 * i + 0] = x1 * y1 * z1w;
      w[8 * i + 1] = x2 * y1 * z1w;
      w[8 * i + 2] = x1 * y2 * z1w;
      w[8 * i + 3] = x2 * y2 * z1w;
      w[8 * i + 4] = x1 * y1 * z2w;
      w[8 * i + 5] = x2 * y1 * z2w;
      w[8 * i + 6] = x1 * y2 * z2w;
      w[8 * i + 7] = x2 * y2 * z2w;
      node[8 * i + 0] = b0;
      node[8 * i + 1] = b0 + 1;
      node[8 * i + 2] = b0 + nix;
      node[8 * i + 3] = b0 + nix + 1;
      node[8 * i + 4] = b1;
      node[8 * i + 5] = b1 + 1;
      node[8 * i + 6] = b1 + nix;
      node[8 * i + 7] = b1 + nix + 1;
    }
  }

  if (status == OR_OK) {
    const int nc = p->one_d ? 2 : 8;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < np; ++i) { /* getFFelecs */
      double r = 0.0, m = 0.0;
      for (int c = 0; c < nc; ++c) r = w[8 * i + c] * ar[node[8 * i + c]] + r;
      for (int c = 0; c < nc; ++c) m = w[8 * i + c] * ai[node[8 * i + c]] + m;
      fr[i] = r;
      fi[i] = m;
    }
    if (p->field_evolve) { /* getSource (a zero-filled result otherwise) */
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < np; ++i) {
        double sr, si;
        if (p->one_d) { /* system_interpolation_1D.f90:135,147,164 */
          double dw = (chi[i] / dV3) * (1.0 + eta * sp2[i]) / gam[i];
          sr = dw * px[i];
          si = dw * py[i];
        } else { /* system_interpolation.f90:171-172, 208-209 */
          sr = ((chi[i] / dV3) * (1.0 + eta * sp2[i]) * px[i] / gam[i]);
          si = ((chi[i] / dV3) * (1.0 + eta * sp2[i]) * py[i] / gam[i]);
        }
        /* 16 (3D) or 4 (1D) atomic adds per particle, as the reference's !$OMP ATOMIC */
        for (int c = 0; c < nc; ++c) {
#pragma omp atomic
          dadz_r[node[8 * i + c]] += w[8 * i + c] * sr;
        }
        for (int c = 0; c < nc; ++c) {
#pragma omp atomic
          dadz_i[node[8 * i + c]] += w[8 * i + c] * si;
        }
      }
    }
  }
  if (!p->coupling) {
    memset(fr, 0, sizeof(double) * (size_t)np);
    memset(fi, 0, sizeof(double) * (size_t)np);
  }

  if (p->electrons_evolve) {
    const double k2 = kappa * kappa;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < np; ++i) {
      double bx, by, bz;
      or_bfield(p, st, x[i], y[i], &bx, &by, &bz);
      double q = 1.0 + eta * sp2[i];
      ddz2[i] = sp2[i];
      ddx[i] = 2.0 * rho * kappa / sqrt(eta) * q / gam[i] * px[i];
      ddy[i] = -(2.0 * rho * kappa / sqrt(eta) * q / gam[i] * py[i]);
      dpx[i] = sInv2rho * (n2col * by - eta * sp2[i] / k2 * fr[i]) +
               kappa * py[i] / gam[i] * q * n2col * bz;
      dpy[i] = sInv2rho * (n2col * bx - eta * sp2[i] / k2 * fi[i]) -
               kappa * px[i] / gam[i] * q * n2col * bz;
      dgam[i] = -(rho * q / gam[i] * 2.0 * (px[i] * fr[i] + py[i] * fi[i]));
    }
  } else {
    for (int64_t i = 0; i < np; ++i) ddx[i] = ddy[i] = ddz2[i] = dpx[i] = dpy[i] = dgam[i] = 0.0;
  }
  free(sp2);
  free(fr);
  free(fi);
  free(node);
  free(w);
  return status;
}

/* rk4par (puffin_mpi_RK4.f90:142-328) on one rank: upd8a is a no-op and the
 * periodic fold of upd8da is the modular plane indexing inside or_rhs. */
int or_rk4_step(const or_params *p, or_taper *t, double sz, double h,
                int64_t np, double *x, double *y, double *z2, double *px,
                double *py, double *gam, const double *chi,
                double *ar, double *ai) {
  const int64_t nw = p->nix * p->niy * or_nplanes(p);
  const double hh = h * 0.5, h6 = h / 6.0, szh = sz + hh;
  size_t pb = sizeof(double) * (size_t)(np > 0 ? np : 1), fb = sizeof(double) * (size_t)nw;
  double *ys[6] = {x, y, z2, px, py, gam};
  double *k1[6], *kt[6], *km[6], *yt[6];
  for (int j = 0; j < 6; ++j) {
    k1[j] = (double *)calloc(1, pb);
    kt[j] = (double *)calloc(1, pb);
    km[j] = (double *)calloc(1, pb);
    yt[j] = (double *)calloc(1, pb);
  }
  double *d0r = calloc(1, fb), *d0i = calloc(1, fb), *d1r = calloc(1, fb), *d1i = calloc(1, fb);
  double *d2r = calloc(1, fb), *d2i = calloc(1, fb), *a1r = calloc(1, fb), *a1i = calloc(1, fb);
  or_stage st;
  int s;

  or_stage_setup(p, t, sz, &st);
  s = or_rhs(p, &st, np, ar, ai, x, y, z2, px, py, gam, chi, k1[0], k1[1], k1[2], k1[3], k1[4], k1[5], d0r, d0i);
  if (s) goto done;
#pragma omp parallel for collapse(2) schedule(static)
  for (int j = 0; j < 6; ++j)
    for (int64_t i = 0; i < np; ++i) yt[j][i] = ys[j][i] + hh * k1[j][i];
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < nw; ++n) { a1r[n] = ar[n] + hh * d0r[n]; a1i[n] = ai[n] + hh * d0i[n]; }

  or_stage_setup(p, t, szh, &st);
  s = or_rhs(p, &st, np, a1r, a1i, yt[0], yt[1], yt[2], yt[3], yt[4], yt[5], chi, kt[0], kt[1], kt[2], kt[3], kt[4], kt[5], d1r, d1i);
  if (s) goto done;
#pragma omp parallel for collapse(2) schedule(static)
  for (int j = 0; j < 6; ++j)
    for (int64_t i = 0; i < np; ++i) yt[j][i] = ys[j][i] + hh * kt[j][i];
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < nw; ++n) { a1r[n] = ar[n] + hh * d1r[n]; a1i[n] = ai[n] + hh * d1i[n]; }

  or_stage_setup(p, t, szh, &st);
  s = or_rhs(p, &st, np, a1r, a1i, yt[0], yt[1], yt[2], yt[3], yt[4], yt[5], chi, km[0], km[1], km[2], km[3], km[4], km[5], d2r, d2i);
  if (s) goto done;
#pragma omp parallel for collapse(2) schedule(static)
  for (int j = 0; j < 6; ++j)
    for (int64_t i = 0; i < np; ++i) yt[j][i] = ys[j][i] + h * km[j][i];
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < nw; ++n) { a1r[n] = ar[n] + h * d2r[n]; a1i[n] = ai[n] + h * d2i[n]; }
#pragma omp parallel for collapse(2) schedule(static)
  for (int j = 0; j < 6; ++j)
    for (int64_t i = 0; i < np; ++i) km[j][i] = kt[j][i] + km[j][i];
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < nw; ++n) {
    d2r[n] = d1r[n] + d2r[n];
    d2i[n] = d1i[n] + d2i[n];
    d1r[n] = 0.0;
    d1i[n] = 0.0;
  }

  or_stage_setup(p, t, sz + h, &st);
  s = or_rhs(p, &st, np, a1r, a1i, yt[0], yt[1], yt[2], yt[3], yt[4], yt[5], chi, kt[0], kt[1], kt[2], kt[3], kt[4], kt[5], d1r, d1i);
  if (s) goto done;
#pragma omp parallel for collapse(2) schedule(static)
  for (int j = 0; j < 6; ++j)
    for (int64_t i = 0; i < np; ++i) ys[j][i] = ys[j][i] + h6 * (k1[j][i] + kt[j][i] + 2.0 * km[j][i]);
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < nw; ++n) {
    ar[n] = ar[n] + h6 * (d0r[n] + d1r[n] + 2.0 * d2r[n]);
    ai[n] = ai[n] + h6 * (d0i[n] + d1i[n] + 2.0 * d2i[n]);
  }
done:
  for (int j = 0; j < 6; ++j) { free(k1[j]); free(kt[j]); free(km[j]); free(yt[j]); }
  free(d0r); free(d0i); free(d1r); free(d1i); free(d2r); free(d2i); free(a1r); free(a1i);
  return s;
}
