/*
 * CPU oracle for the Puffin RK4 macroparticle push (TEST INFRASTRUCTURE ONLY).
 *
 * This is a plain-C restatement of the reference's per-stage right-hand side
 * and RK4 integrator, written so that the GPU library can be checked against
 * it.  It is never linked into, loaded by, or called from the product path:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 *
 * Parity anchors (reference file:line, paths inside the Puffin project):
 *   getP2                  puffin/lib/utilities/gamma_to_p2.f90:84-85
 *   getrhs / rhs_tmsavers  puffin/lib/interaction/rhs.f90:60-330, 346-399
 *   getInterps_3D etc.     puffin/lib/interaction/system_interpolation.f90:25-248
 *   1D variants            puffin/lib/interaction/system_interpolation_1D.f90:24-179
 *   equations              puffin/lib/interaction/puffin_equations.f90:17-176
 *   b-fields               puffin/lib/undulator/bfields.f90:36-881
 *   getAlpha / adjUndPlace puffin/lib/undulator/wiggler_taper.f90:39-47,
 *                          puffin/lib/interaction/puffin_equations.f90:218-254
 *   rk4par                 puffin/lib/interaction/puffin_mpi_RK4.f90:142-328
 *   periodic z2 fold       puffin/lib/parallel/para_field.f90:924-1061 (restated
 *                          as modular plane indexing over nz2-1 unique planes)
 *
 * Parity is pinned for the 1D path by the reference's golden dump
 * (test/expected/f1main_expected_*.h5, see tests/golden/).  The 3D
 * gather/deposit, b-field and diffraction paths have no reference golden
 * vectors: for those the oracle is a restatement only.
 */
#ifndef PUFFIN_ORACLE_H
#define PUFFIN_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Undulator types (bfields.f90 branches). */
enum { OR_UND_PUFFIN = 0, OR_UND_HELICAL = 1, OR_UND_PLANEPOLE = 2, OR_UND_CURVED = 3 };
/* Undulator section (iUndStart_G / iUndMain_G / iUndEnd_G). */
enum { OR_PLACE_START = 0, OR_PLACE_MAIN = 1, OR_PLACE_END = 2 };
/* Field mesh type (deriv_globals.f90: iTemporal = 0, iPeriodic = 1). */
enum { OR_MESH_TEMPORAL = 0, OR_MESH_PERIODIC = 1 };
/* Status bits. */
enum { OR_OK = 0, OR_OUT_OF_WINDOW = 1, OR_OUT_OF_Z2 = 2 };

typedef struct {
  /* scaled physics constants */
  double rho, eta, kappa, aw, gamma_r;
  double fx, fy;             /* undulator polarisation (elliptical branch) */
  double kx_und, ky_und;     /* curved-pole wavenumbers */
  double kbxsf, kbysf;       /* strong-focusing wavenumbers (qFocussing) */
  int und_type;              /* OR_UND_* */
  int one_d;                 /* qOneD */
  int focusing;              /* qFocussing */
  int und_ends;              /* qUndEnds */
  int field_evolve, electrons_evolve, coupling;
  double szfs, szfe;         /* start/end of the main section in zbar */
  /* mesh */
  int mesh_type;             /* OR_MESH_* */
  int64_t nz2;               /* z2 nodes (periodic: nz2-1 unique planes) */
  int64_t nix, niy;          /* inner transverse window (nspinDX, nspinDY) */
  double dx, dy, dz2;
} or_params;

/* Per-stage undulator scalars, computed once per RK4 stage. */
typedef struct {
  double sz;                 /* zbar at which the stage is evaluated */
  double n2col;              /* taper factor alpha(z) */
  int place;                 /* OR_PLACE_* */
} or_stage;

/* Taper state (wiggler_taper.f90 keeps n2col and n2col0 as globals). */
typedef struct {
  double n2col, n2col0, undgrad;
  int nprof;                 /* > 1: piecewise-linear alpha(z) through (pz, pa) */
  const double *pz, *pa;
} or_taper;

/* Evaluate getAlpha + adjUndPlace for one stage; mutates the taper state the
 * same way the reference does. */
void or_stage_setup(const or_params *p, or_taper *t, double sz, or_stage *out);

/* p2 from Gamma, px, py (gamma_to_p2.f90:84-85). */
double or_p2(double gam, double px, double py, double eta, double gamma0, double aw);

/* One evaluation of derivs/getrhs: derivatives of the 6 particle arrays and
 * the deposit into dadz (which is ACCUMULATED into, as upd8da expects a zeroed
 * buffer).  Returns OR_* status bits; on a bounds failure no gather or deposit
 * is done for any particle, as in the reference. */
int or_rhs(const or_params *p, const or_stage *st, int64_t np,
           const double *ar, const double *ai,
           const double *x, const double *y, const double *z2,
           const double *px, const double *py, const double *gam,
           const double *chi,
           double *dx_, double *dy_, double *dz2_, double *dpx, double *dpy,
           double *dgam, double *dadz_r, double *dadz_i);

/* One rk4par step over the particle state and the inner-window field
 * (nwin = nix*niy*nplanes values each for ar/ai).  On failure the state is
 * left unchanged and the status bits are returned. */
int or_rk4_step(const or_params *p, or_taper *t, double sz, double h,
                int64_t np, double *x, double *y, double *z2, double *px,
                double *py, double *gam, const double *chi,
                double *ar, double *ai);

/* Number of planes of the inner-window field held by the oracle. */
int64_t or_nplanes(const or_params *p);

/* Periodic wrap of z2 positions done at each redistribution
 * (para_field.f90:212-215). */
void or_wrap_z2(const or_params *p, int64_t np, double *z2);

/* OpenMP thread count for the particle loops (1 = sequential, reproducible
 * deposit order). */
void or_set_threads(int n);

/* Undulator b-field at one particle (bfields.f90). */
void or_bfield(const or_params *p, const or_stage *st, double x, double y,
               double *bx, double *by, double *bz);

#ifdef __cplusplus
}
#endif
#endif
