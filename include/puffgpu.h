/*
 * puffgpu — GB300 (sm_103a) library for Puffin's per-step hot path:
 * the RK4 macroparticle push with trilinear gather/deposit between the
 * macroparticles and the complex radiation field, and the FFT diffraction
 * step with its absorbing boundary.
 *
 * C ABI only: plain pointers, sizes and int status codes, no C++ or torch
 * types.  The array layouts are the reference's own:
 *   particles  7 SoA FP64 arrays x, y, z2, px, py, gamma, chi of length n,
 *              where "py" holds the stored imaginary p_perp (= -py), exactly
 *              as sElPY_G (simple_electron_gen.f90:330);
 *   field      2 FP64 arrays (re, im) over the outer mesh, x fastest:
 *              idx = ix + nx*iy + nx*ny*iz (diffraction.f90:259-260), nz2
 *              planes; on the periodic mesh the last plane mirrors the first.
 *
 * Every entry point returns a pf_status.  Nothing here exits or stops the
 * process: where the reference STOPs (a particle beyond the temporal z2
 * mesh, system_interpolation.f90:70-76) the call returns PF_OUT_OF_Z2.
 *
 * Reference interfaces replaced (file:line inside the Puffin project):
 *   pf_rk4_step      rk4par(sZ, h, qD)        puffin/lib/interaction/puffin_mpi_RK4.f90:38
 *   pf_rk4_step_host rk4par with the driver's host arrays (sElX_G.., ac_rfield_in)
 *   pf_diffract_host inner2Outer + diffractIM + outer2Inner with the driver's
 *                    host arrays (ac_rfield, ac_rfield_in)
 *                    -> derivs                puffin/lib/interaction/derivative.f90:36
 *                    -> getrhs                puffin/lib/interaction/rhs.f90:60
 *   pf_diffract      inner2Outer + diffractIM(sStep, qD, qOK) + outer2Inner
 *                                             puffin/lib/parallel/para_field.f90:1352,1394
 *                                             puffin/lib/diffraction/diffraction.f90:46
 *   pf_redistribute  getInNode + getLocalFieldIndices (window + periodic z2 wrap)
 *                                             puffin/lib/parallel/para_field.f90:1432, 83
 *   pf_run           the RK4/diffraction loop of UndSection
 *                                             puffin/lib/undulator.f90:182-333
 *   pf_set/get_particles, pf_set/get_field    the module globals sElX_G..sElGam_G,
 *                    s_chi_bar_G, ac_rfield/ac_ifield (deriv_globals.f90)
 *   pf_set/get_taper getAlpha state n2col/n2col0/undgrad
 *                                             puffin/lib/undulator/wiggler_taper.f90:16-53
 */
#ifndef PUFFGPU_H
#define PUFFGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PUFFGPU_ABI_VERSION 1

typedef enum {
  PF_OK = 0,
  PF_OUT_OF_WINDOW = 1,   /* a macroparticle left the inner transverse window
                             (qInnerXYOK_G = .false.); state left unchanged */
  PF_OUT_OF_Z2 = 2,       /* z2 node beyond the temporal mesh (the reference STOPs) */
  PF_BAD_ARG = 3,
  PF_CUDA_ERR = 4,
  PF_TIMEOUT = 5,         /* a bounded device-side wait gave up */
  PF_NO_DEVICE = 6,
  PF_OVERFLOW = 7,        /* a deposit exceeded the fixed-point range */
  PF_STATE = 8,           /* call order error (e.g. step before set_particles) */
  PF_NOT_FINITE = 9       /* a NaN or infinity in a macroparticle's stage state, in the
                             field it gathered or in the inner-window field; state left
                             unchanged (the reference does not check) */
} pf_status;

typedef enum {
  PF_UND_PUFFIN = 0,      /* elliptical 'puffin' undulator (zUndType = '') */
  PF_UND_HELICAL = 1,
  PF_UND_PLANEPOLE = 2,
  PF_UND_CURVED = 3
} pf_und_type;

typedef enum { PF_MESH_TEMPORAL = 0, PF_MESH_PERIODIC = 1 } pf_mesh_type;
typedef enum { PF_FP64 = 0, PF_MIXED = 1 } pf_precision;

/* Scaled-unit constants and flags of one undulator module.  Names follow the
 * reference globals they replace (deriv_globals.f90). */
typedef struct pf_params {
  double rho;          /* sRho_G */
  double eta;          /* sEta_G */
  double kappa;        /* sKappa_G */
  double aw;           /* saw_G (peak) */
  double gamma_r;      /* sGammaR_G */
  double fx, fy;       /* fx_G, fy_G */
  double kx_und, ky_und;   /* kx_und_G, ky_und_G (curved poles) */
  double kbxsf, kbysf;     /* sKBetaXSF_G, sKBetaYSF_G (qFocussing) */
  double szfs, szfe;   /* sZFS, sZFE: main-section bounds in local zbar */
  double n2col0;       /* taper alpha at sZFS (mf of the module) */
  double undgrad;      /* taper gradient d(alpha)/dzbar */
  double dx, dy, dz2;  /* sLengthOfElm{X,Y,Z2}_G */
  double sbeta;        /* sBeta_G: absorption coefficient */
  double sfilt_frac;   /* sFiltFrac: high-pass cut as a fraction of the
                          resonant frequency (the reference's default is the
                          single-precision literal 0.3) */
  double sperwaves;    /* sPerWaves_G (periodic cut-off rule) */
  int32_t und_type;    /* pf_und_type */
  int32_t mesh_type;   /* pf_mesh_type (fieldMesh) */
  int32_t nx, ny, nz2; /* NX_G, NY_G, NZ2_G */
  int32_t nix, niy;    /* nspinDX, nspinDY; 0 = computed from the particles
                          the way getInNode does */
  int32_t nbx, nby, nbz2;  /* absorbing-boundary widths (16, 16, 37) */
  int32_t one_d;       /* qOneD (nx = ny = 1) */
  int32_t focusing;    /* qFocussing */
  int32_t und_ends;    /* qUndEnds */
  int32_t field_evolve, electrons_evolve, coupling;  /* q*Evolve / coupling */
  int32_t qfilter;     /* qFilter */
  int32_t redist_every;/* iRedistStp_G (periodic z2 wrap cadence in pf_run) */
  int32_t precision;   /* pf_precision */
  int32_t device;      /* CUDA device ordinal */
} pf_params;

typedef struct pf_handle pf_handle;

/* Fill *p with the reference's defaults (nb* = 16/16/37, sbeta = 1,
 * sfilt_frac = (double)0.3f, qfilter = 1, evolve/coupling flags = 1,
 * redist_every = 60, FP64). */
void pf_default_params(pf_params *p);

int pf_create(const pf_params *p, pf_handle **out);
int pf_destroy(pf_handle *h);

/* Particles: host arrays (copied in/out) or device arrays (device-to-device).
 * pf_set_particles also computes the inner window the particles need
 * (getInNode, parallel/para_field.f90:1432-1508) when the handle has none
 * yet or the current one is too small; a larger current window is kept (the
 * reference recomputes it only at redistribution: pf_redistribute).  chi may
 * be NULL to keep the handle's chi (rk4par never changes it) when n is the
 * current macroparticle count, else PF_BAD_ARG; pf_get_particles skips every
 * NULL destination.  pf_run may re-order the macroparticles on the device by
 * z2 plane (beams of 2^15 or more, at the wrap cadence); pf_get_particles
 * always returns them in the order pf_set_particles received them. */
int pf_set_particles(pf_handle *h, int64_t n, const double *x, const double *y,
                     const double *z2, const double *px, const double *py,
                     const double *gam, const double *chi);
int pf_get_particles(pf_handle *h, double *x, double *y, double *z2, double *px,
                     double *py, double *gam, double *chi);
int pf_set_particles_dev(pf_handle *h, int64_t n, const double *x, const double *y,
                         const double *z2, const double *px, const double *py,
                         const double *gam, const double *chi);
int pf_get_particles_dev(pf_handle *h, double *x, double *y, double *z2, double *px,
                         double *py, double *gam, double *chi);
int64_t pf_num_particles(const pf_handle *h);

/* Field on the outer mesh (nx*ny*nz2 values each). */
int pf_set_field(pf_handle *h, const double *re, const double *im);
int pf_get_field(pf_handle *h, double *re, double *im);
int pf_set_field_dev(pf_handle *h, const double *re, const double *im);
int pf_get_field_dev(pf_handle *h, double *re, double *im);

/* Inner-window field: the arrays rk4par advances (ac_rfield_in /
 * ac_ifield_in, puffin/lib/interaction/puffin_mpi_RK4.f90:38, filled by
 * outer2Inner and read back by inner2Outer, parallel/para_field.f90:1352-1429).
 * pf_window_nodes() values each: nix * niy * planes, x fastest, planes = nz2
 * (temporal mesh) or nz2 - 1 (periodic), the window centred in the outer
 * mesh.  pf_set_window_field replaces the window that the next pf_rk4_step
 * advances; pf_diffract and pf_get_field copy the window into the outer
 * mesh first, as UndSection's inner2Outer does.  A driver that keeps the
 * window between steps exchanges only these arrays and the particles per
 * step, and the outer field around diffraction calls.  PF_STATE before the
 * particles (and so the window) are set; the window changes size only in
 * pf_set_particles and pf_redistribute. */
int pf_set_window_field(pf_handle *h, const double *re, const double *im);
int pf_get_window_field(pf_handle *h, double *re, double *im);
int pf_set_window_field_dev(pf_handle *h, const double *re, const double *im);
int pf_get_window_field_dev(pf_handle *h, double *re, double *im);
int64_t pf_window_nodes(const pf_handle *h);

/* Taper state (n2col, n2col0, undgrad). */
int pf_set_taper(pf_handle *h, double n2col, double n2col0, double undgrad);
int pf_get_taper(const pf_handle *h, double *n2col, double *n2col0, double *undgrad);

/* Piecewise-linear taper profile: alpha(z) through n >= 2 control points
 * (z increasing, local zbar of the module), constant beyond the end points;
 * n = 0 returns to the module's linear taper n2col0 + undgrad (z - sZFS)
 * (wiggler_taper.f90:39-45).  The profile generalises the reference's
 * per-module linear taper to the aw(z) profile that the adjoint
 * differentiates. */
int pf_set_taper_profile(pf_handle *h, int32_t n, const double *z, const double *alpha);

/* Inner transverse window currently in use. */
int pf_get_window(const pf_handle *h, int32_t *nix, int32_t *niy);

/* One rk4par step at local zbar szl with step size h.  Returns PF_OK, or
 * PF_OUT_OF_WINDOW / PF_OUT_OF_Z2 with the state unchanged. */
int pf_rk4_step(pf_handle *h, double szl, double hstep);

/* One rk4par step with the driver's arrays in host memory:
 * the six evolving particle arrays (pf_get_particles' order; chi stays the
 * handle's, as rk4par never changes it) and the inner-window field
 * (pf_window_nodes() values each) are read, advanced by one step and written
 * back.  The same as pf_set_window_field + pf_set_particles(..., chi NULL)
 * + pf_rk4_step + pf_get_particles + pf_get_window_field, without choosing
 * the window again: the copies in and out run on a second stream,
 * overlapped with the step's kernels (the particles in chunks), so page-
 * locked host arrays are copied while the step computes (on mixed
 * handles the window field is converted to and from its complex-float form
 * on the device, as pf_set/get_window_field do).  Returns PF_OK, or
 * PF_OUT_OF_WINDOW / PF_OUT_OF_Z2 / PF_OVERFLOW / PF_NOT_FINITE with the
 * host arrays and the handle's state holding the step's input (then
 * pf_redistribute and pf_get_window_field give the driver the new window,
 * as the reference's retry does). */
int pf_rk4_step_host(pf_handle *h, double szl, double hstep, double *x, double *y, double *z2,
                     double *px, double *py, double *gam, double *wre, double *wim);

/* inner2Outer + diffractIM + outer2Inner with the driver's arrays in host
 * memory (FP64 and mixed handles; a mixed handle converts them to and from
 * its complex-float field on the device with pf_set_field's and
 * pf_get_field's roundings): the outer field (nx * ny * nz2 values each) and,
 * when the handle has a window, the inner-window field (pf_window_nodes()
 * values each) are read and written in place, as pf_set_field +
 * pf_set_window_field + pf_diffract + pf_get_field + pf_get_window_field
 * would, with the copies overlapped with the transforms (the outer field
 * and the window copied in and out by ranges of z2 planes while the first
 * and the last passes run on the others). */
int pf_diffract_host(pf_handle *h, double dz, double *ore, double *oim, double *wre,
                     double *wim);

/* getInNode + getLocalFieldIndices: recompute the inner window from the
 * particles and apply the periodic z2 wrap. */
int pf_redistribute(pf_handle *h);

/* Periodic z2 wrap alone (the part of getLocalFieldIndices that changes
 * particle data, para_field.f90:212-215). */
int pf_wrap_z2(pf_handle *h);

/* Diffract the field over dz (inner2Outer + diffractIM + outer2Inner). */
int pf_diffract(pf_handle *h, double dz);

/* UndSection's loop for nsteps RK4 steps of size hstep starting at local
 * zbar *szl (updated on return), diffraction every isteps4diff steps with
 * merged half steps (qdiffraction != 0), retries with a recomputed window on
 * PF_OUT_OF_WINDOW (up to 3, as the reference), periodic wraps every
 * redist_every steps.  *steps_done receives the number of completed steps. */
int pf_run(pf_handle *h, int32_t nsteps, int32_t isteps4diff, int32_t qdiffraction,
           double hstep, double *szl, int32_t *steps_done);

/* Diagnostics of the current state, as the reference's integrated-data
 * writer computes them:
 *   pf_power      power per z2 plane, n = nz2 values: |A|^2 on a 1D mesh
 *                 (fPower_1D), else the 2D trapezoid over x and y with the
 *                 reference's single-precision accumulation (fPower_3D,
 *                 m_trapz2D; puffin/lib/io/av_write.f90:141-276);
 *   pf_bunching   |b_m| per slice of one resonant wavelength, harmonic m >= 1,
 *                 linear slice weights, zero where a slice holds no charge
 *                 (getSliceTwiss, av_write.f90:405-770; slice count
 *                 pf_num_slices as write_adapter.f90:110-112);
 *   pf_spectrum   one-sided |DFT|^2 along z2 of the on-axis field (central
 *                 transverse node), x (re) and y (im) parts, nunique =
 *                 ceil((nz2+1)/2) bins (utilities/pyPlotting/plotSpecPow.py:58-110). */
int pf_power(pf_handle *h, double *power, int64_t n);
int64_t pf_num_slices(const pf_handle *h);
int pf_bunching(pf_handle *h, int32_t harmonic, double *b, int64_t nslices);
int pf_spectrum(pf_handle *h, double *sx, double *sy, int64_t nunique);

/* How pf_run issues its steps: 0 one step at a time (a host round trip per
 * step for the status word), 1 asynchronous blocks of steps between two
 * diffraction calls (one status check per block, the block replayed step by
 * step if a particle left the window), 2 (default) as 1 with each full block
 * replayed as a captured CUDA graph whose stage coefficients come from a
 * device table.  Blocks run asynchronously only while the state they can
 * change fits in 256 MB (a copy is kept for the replay). */
int pf_set_launch_mode(pf_handle *h, int32_t mode);

/* Completed RK4 steps counted over the handle's life (the reference's
 * iCsteps, kept across undulator modules): pf_run wraps z2 on the periodic
 * mesh whenever this count reaches a multiple of redist_every
 * (undulator.f90:320-326).  pf_set_step_count restores it on resume. */
int64_t pf_step_count(const pf_handle *h);
int pf_set_step_count(pf_handle *h, int64_t csteps);

/* Beam-line elements between undulator modules, applied to the macroparticles
 * on the device (puffin/lib/acc_lattice.f90; the element loop is
 * puffin/lib/puffin_module.f90:57-89):
 *   pf_drift          driftSection (:478-518): z2 += dz p2, and x, y move
 *                     with the transverse velocity unless one_d; then
 *                     diffracts the field over dz if qdiffraction;
 *   pf_chicane        disperse (:420-463): z2 -= 2 disp (Gamma - 1) and
 *                     += slip, diffraction over zbar (> 0) if qdiffraction,
 *                     then the periodic z2 wrap;
 *   pf_quad           Quad (:531-561): thin-lens kick of px, py (not on 1D);
 *   pf_modulation     bModulation (:575-585): Gamma += mag cos(k z2);
 *   pf_match_in/out   matchIn / matchOut (:743-828 / :638-725): the undulator
 *                     entry/exit offsets of x, y, px, py at zbar sz for the
 *                     handle's undulator type and current taper factor;
 *   pf_correct_trans  correctTrans (:601-623): subtract the chi-weighted
 *                     means of px, py, x, y (a fixed-order reduction, so the
 *                     result is the same every run);
 *   pf_init_undulator initUndulator (:848-895): the module's undulator type,
 *                     ux, uy, focusing factors, taper start value mf and
 *                     gradient, and the ends sZFS / sZFE from nsteps, hstep
 *                     and und_ends. */
int pf_drift(pf_handle *h, double dz, int32_t qdiffraction);
int pf_chicane(pf_handle *h, double disp, double slip, double zbar, int32_t qdiffraction);
int pf_quad(pf_handle *h, double qfx, double qfy);
int pf_modulation(pf_handle *h, double mag, double wavenum);
int pf_match_in(pf_handle *h, double sz);
int pf_match_out(pf_handle *h, double sz);
int pf_correct_trans(pf_handle *h);
int pf_init_undulator(pf_handle *h, int32_t und_type, double fx, double fy, double kbxsf,
                      double kbysf, double mf, double taper, int32_t nsteps, double hstep,
                      int32_t und_ends);

/* Adjoint of the RK4 / diffraction run, with checkpoint and recompute, on
 * an FP64 or a mixed-precision handle.  On a mixed handle the run records
 * the mixed stage kernels and the FP32 diffraction, and the adjoint keeps
 * their split: the field adjoint in FP32 complex; the particle adjoint, the
 * RK4 combination and the z2 (phase) adjoint in FP64; the rest of each
 * stage's vector-Jacobian product in FP32.  pf_adjoint_forward runs nsteps steps
 * the way pf_run does (UndSection's loop, undulator.f90:182-333; no window
 * retries: the window must hold the beam for the whole run) from the
 * handle's particles with the energy chirp gamma += chirp (z2 - <z2>)
 * applied and the initial field seed_amp * (seed_re, seed_im) (outer mesh),
 * under the taper profile set by pf_set_taper_profile, keeping the state
 * every checkpoint_every steps; it returns the final pulse energy
 * E = dx dy dz2 sum |A|^2 over the outer mesh (unique z2 planes).  pf_adjoint_backward then returns denergy * dE/d(the
 * ntaper profile values), dE/d(seed_amp) and dE/d(chirp), recomputing each
 * segment of checkpoint_every steps once.  Both leave the handle's
 * particles at the unchirped beam; the field must be set again before other
 * calls. */
/* Quiet-start beam on the device (the Halton-sequence branch of the
 * reference's generator, mp_sequences.f90:126-433, MPfDists.f90:406-620,
 * noise.f90:25-80): nslices z2 slices with centres z2m[k], width dz2 and
 * ne[k] electrons, nseq beamlets each from the Halton sequences of bases 2,
 * 3, 5, 11, 7 (x, y, px, py, gamma; projected on a unit Gaussian, scaled by
 * sig[5k + d] and shifted by mean[5k + d]) and 13 (z2 offset in the slice).
 * noise != 0 adds the shot noise (Poisson electron counts, z2 jitter) from a
 * counter-based generator seeded with seed (the reference seeds from the
 * clock).  chi = electrons per beamlet * chi_per_electron.  The result
 * becomes the handle's particles (nslices * nseq of them). */
int pf_generate_beam(pf_handle *h, int64_t nslices, const double *z2m, const double *ne,
                     double dz2, int32_t nseq, const double *mean, const double *sig,
                     int32_t noise, uint64_t seed, double chi_per_electron);

/* Adjoint of one FP64 diffraction step over dz, applied in place to
 * (re, im) on the outer mesh (host or device arrays; the unique z2 planes;
 * the periodic mirror plane is left alone): the conjugate propagator and
 * the self-adjoint filter, damping and masks in reversed order. */
int pf_diffract_adjoint(pf_handle *h, double dz, double *re, double *im);
int pf_adjoint_forward(pf_handle *h, int32_t nsteps, int32_t isteps4diff, int32_t qdiffraction,
                       double hstep, int32_t checkpoint_every, const double *seed_re,
                       const double *seed_im, double seed_amp, double chirp, double *energy);
int pf_adjoint_backward(pf_handle *h, double denergy, double *g_taper, int32_t ntaper,
                        double *g_seed, double *g_chirp);

/* Batched runs (no counterpart in the reference, which runs one simulation
 * per process).  A batch groups n independent instances -- handles created
 * with pf_create on one device, one precision, 3D, each with its particles
 * and field set -- and advances them together: every RK4 stage of every
 * instance in one launch over (instance, range) tiles, the blocks of steps
 * between diffraction calls replayed as one CUDA graph.  Each instance
 * follows pf_run's schedule exactly (UndSection, undulator.f90:33-358):
 * pf_batch_run(b, nsteps, isteps4diff, qdiffraction, hstep, szl, status)
 * does what pf_run(inst[i], nsteps, isteps4diff, qdiffraction, hstep[i],
 * &szl[i], NULL) does for every i (FP64: the same bits), with hstep and szl
 * per instance.  status[i] (may be NULL) receives each instance's pf_status;
 * an instance that fails stops, the others go on; the return value is the
 * first failing instance's status (PF_OK when none failed).  The handles stay
 * owned by the caller and must outlive the batch; while a batch call runs,
 * their work is queued on the batch's stream.
 *
 * pf_batch_tune times candidate launch shapes on the instances' current
 * state (restored afterwards) and keeps the fastest: per instance the deposit
 * mode (direct atomics, or a shared-memory tile over ranges of 1024..8192
 * macroparticles), for the batch the macroparticles per direct tile, the FP64
 * stage block size, the node tile length and persistent or per-tile grids.
 * pf_batch_get_shape / pf_batch_set_shape read and override them: shape5 =
 * {stage threads (128 or 256), macroparticles per direct tile, nodes per node
 * tile, stage grid (0 one block per tile, -1 persistent), node grid}, modes =
 * per instance 0 (direct) or the tile range length. */
typedef struct pf_batch pf_batch;
int pf_batch_create(pf_handle *const *handles, int32_t n, pf_batch **out);
int pf_batch_destroy(pf_batch *b);
int pf_batch_run(pf_batch *b, int32_t nsteps, int32_t isteps4diff, int32_t qdiffraction,
                 const double *hstep, double *szl, int32_t *status);
int pf_batch_tune(pf_batch *b, const double *hstep, const double *szl, int32_t repeats);
int pf_batch_get_shape(const pf_batch *b, int64_t *shape5, int64_t *modes);
int pf_batch_set_shape(pf_batch *b, const int64_t *shape5, const int64_t *modes);
/* on = 0: launch the kernels of each block directly instead of a graph */
int pf_batch_use_graphs(pf_batch *b, int32_t on);
int64_t pf_batch_launches(const pf_batch *b);
void *pf_batch_stream(const pf_batch *b);
const char *pf_batch_last_error(const pf_batch *b);

/* Arithmetic of the FP64 path's diffraction FFTs (the field stays FP64 in
 * HBM either way): PF_FFT_PAIRED_FP32 (the default) holds each value as an
 * unevaluated sum of two floats (48 significand bits, about 1e-14 of the
 * field scale per call) and computes with FP32 operations only, which GB300
 * issues at 64 times its FP64 rate (2.5 times faster on the 129 x 129 x
 * 4096 mesh); PF_FFT_FP64 computes in FP64.  The
 * reference transforms with FFTW in FP64 (diffraction/transforms.f90:406-435);
 * no result of this library matches FFTW bit for bit either way.  PF_BAD_ARG
 * on a mixed-precision handle (its FFTs are FP32). */
#define PF_FFT_FP64 0
#define PF_FFT_PAIRED_FP32 1
int pf_set_fft_arithmetic(pf_handle *h, int32_t mode);

/* Block until all work queued by the handle is done. */
int pf_sync(pf_handle *h);

/* Number of kernels this handle has launched so far. */
int64_t pf_kernel_launches(const pf_handle *h);

/* The cudaStream_t (as void*) every kernel of this handle is launched on, so
 * callers can order their own work and timing events against it. */
void *pf_get_stream(const pf_handle *h);

/* Per-kernel-class device timing with CUDA events recorded on the handle's
 * stream around each launch (classes: 0 particle stage kernels, 1 field node
 * kernels, 2 FFT passes, 3 diffraction element-wise kernels, 4 other).
 * pf_profile(h, 1) enables and clears the counters; pf_profile_read returns
 * the summed milliseconds and the number of timed launches of one class. */
int pf_profile(pf_handle *h, int32_t enable);
int pf_profile_read(pf_handle *h, int32_t kernel_class, double *ms_total, int64_t *launches);

/* Human-readable text of the last error on this handle (or a global one when
 * h is NULL). */
const char *pf_last_error(const pf_handle *h);

int pf_abi_version(void);

/* Allocation-free RK4 step (no counterpart in the reference).  For callers
 * that cannot allocate device memory -- a host program whose device memory
 * belongs to its own pool allocator, a plugin host that hands in buffers it
 * allocated up front, or a loop that cannot afford cudaMalloc's implicit
 * device-wide synchronisation.  It does what pf_rk4_step does, without a
 * handle: the caller passes the particle arrays and the inner-window field
 * (nix * niy * planes values each, planes = nz2 or nz2 - 1 on the periodic
 * mesh, layout of outer2Inner) as device pointers, updated in place, and the
 * taper state (n2col, n2col0) in host memory, updated like getAlpha does.
 * The RK4 temporaries live in one fixed-size file-scope device array of the
 * library, held by every GPU that loads it until the process exits.
 * Limits: np <= PF_NOALLOC_MAX_PARTICLES and nix*niy*planes <=
 * PF_NOALLOC_MAX_NODES, else PF_BAD_ARG.  Calls share that array: calls that
 * overlap on the GPU (different streams, several host threads) race.  The
 * first call on a device looks up the array's device address with that device
 * current and keeps it for the process's life, so a cudaDeviceReset or a
 * non-primary context on that device is not supported.  Every call waits for
 * its stream (it reads the deposit scale and the status word back), so it
 * must not be called while that stream is being captured.  stream may be NULL
 * (the default stream).  Returns as pf_rk4_step; on PF_OUT_OF_WINDOW the
 * caller's arrays are left unchanged. */
#define PF_NOALLOC_MAX_PARTICLES 32768
#define PF_NOALLOC_MAX_NODES 32768
int pf_rk4_step_noalloc(const pf_params *p, double *n2col, double *n2col0, double szl,
                        double hstep, int64_t np, double *x, double *y, double *z2, double *px,
                        double *py, double *gam, const double *chi, double *wr, double *wi,
                        int32_t nix, int32_t niy, void *stream);

#ifdef __cplusplus
}
#endif
#endif
