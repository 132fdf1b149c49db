// Internal declarations shared by the puffgpu translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/puffgpu.h"

// One-time set-up per device: CUDA keeps kernel attributes (such as the
// dynamic shared-memory limit) per device, so handles on several devices of
// one process each need them set on their own device.  pf_device_once runs
// f() once for the current device and returns its result on every call.
constexpr int PF_MAX_DEVICES = 64;
struct PfDeviceOnce {
  std::mutex m;
  bool done[PF_MAX_DEVICES] = {};
  cudaError_t err[PF_MAX_DEVICES] = {};
};
template <typename F>
cudaError_t pf_device_once(PfDeviceOnce &o, F &&f) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= PF_MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> g(o.m);
  if (!o.done[dev]) {
    o.err[dev] = f();
    o.done[dev] = true;
  }
  return o.err[dev];
}

// Puffin's global pi is a default-kind (single precision) literal
// (puffin/lib/common/puffin_constants.f90:22).  GetKValues uses its own
// full-precision pi (transforms.f90:492).
#define PF_PUFFIN_PI ((double)3.14159265358979323846f)
#define PF_FULL_PI 3.14159265358979323846

// Device status word bits (one word per handle, OR-ed by the kernels).
enum : unsigned int {
  ST_OUT_OF_WINDOW = 1u,
  ST_OUT_OF_Z2 = 2u,
  ST_OVERFLOW = 4u,
  ST_NOT_FINITE = 8u,
};

// pf_status of a device status word (the most severe condition first).
inline int pf_status_of(unsigned int st) {
  if (st & ST_NOT_FINITE) return PF_NOT_FINITE;
  if (st & ST_OVERFLOW) return PF_OVERFLOW;
  if (st & ST_OUT_OF_Z2) return PF_OUT_OF_Z2;
  if (st & ST_OUT_OF_WINDOW) return PF_OUT_OF_WINDOW;
  return PF_OK;
}

// Finite test from the exponent bits (integer operations, off the FP64 pipe).
__device__ __forceinline__ bool pf_finite(double v) {
  return (__double2hiint(v) & 0x7ff00000) != 0x7ff00000;
}

// Undulator b-field coefficients for one RK4 stage.  Every stage-uniform
// sub-expression of bfields.f90 is evaluated once on the host, left to right
// as the Fortran writes it, so the per-particle remainder keeps the
// reference's operation order.
struct BFieldCoef {
  int type;      // pf_und_type
  int place;     // 0 start, 1 main, 2 end
  int one_d;
  int focusing;
  int tcase;     // helical/puffin start/end: 0 none, 1 use ux, 2 use c1x (7*pi*rho side)
  double bx0, by0;        // x/y-independent parts of bx, by
  double focx, focy;      // strong-focusing coefficients
  double S, C;            // sin/cos of the section's phase argument
  double c1;              // sqrt(eta)/2/rho
  double ux, uy;          // start/end section coefficients of x and y
  double u3;              // planepole/curved section factor
  double fx, fy;
  double kx, ky, kxky, czs, cze;  // curved-pole constants
  double szt;             // phase argument (curved start, per-particle division)
};

// Everything a stage kernel needs, passed by value.
// Per-(step, stage) coefficients read from device memory by the stage kernels
// when pf_run replays a captured step block (the values the host would pass
// as kernel arguments otherwise).
struct StageCoef {
  BFieldCoef bf;
  double n2col, kn2col;
};

struct StageArgs {
  const StageCoef *coef_tab;  // non-null: coefficients at coef_tab[*step_ctr * 4 + stage - 1]
  const int *step_ctr;
  // particle arrays
  const double *x, *y, *z2, *px, *py, *gam, *chi;
  const double *kin[6];   // derivative used to form the stage state (stage > 1)
  double *kout[6];        // derivative written by this stage
  double *kacc[6];        // k2 (stage 2 out) / k2+k3 (stage 3 in/out) / read (stage 4)
  const double *k1[6];    // stage 4: k1
  double *ynext[6];       // stage 4: committed state
  int64_t np;
  double cstate;          // state = y + cstate * kin
  double h6;
  // field (inner window)
  const double *ar, *ai;  // stage field A_s
  unsigned long long *acc_lo_r, *acc_hi_r, *acc_lo_i, *acc_hi_i;
  int64_t nix, niy, npl;  // window dims and planes held
  int64_t nz2;
  int periodic;
  int one_d;
  double dx, dy, dz2, halfx, halfy, dV3;
  // physics
  double eta, kappa, rho, gamma_r, aw, n2col, sInv2rho, dxc, k2;
  double inv_eta, eta_k2, rho2, kn2col, inv_dx, inv_dy, inv_dz2, inv_dV3;
  int field_evolve, electrons_evolve, coupling;
  int fix_e;              // fixed-point scale exponent of the deposit
  int fix_maxexp;         // overflow guard: |contribution * 2^E| < 2^fix_maxexp
  int tile_ppb;           // dense mode: macroparticles per block (set at launch)
  BFieldCoef bf;
  unsigned int *status;
};

struct NodeArgs {
  int *step_ctr;              // non-null: stage 4 advances it once per step
  int64_t n;                  // window nodes
  unsigned long long *acc_lo_r, *acc_hi_r, *acc_lo_i, *acc_hi_i;
  double *wr, *wi;            // window field state (ac_rfield_in)
  double *asr, *asi;          // stage field
  double *d0r, *d0i;          // k1 of the field
  double *d12r, *d12i;        // k2 (then k2+k3) of the field
  double coef;                // hh or h
  double h6;
  int fix_e;
  const unsigned int *status;
};

// One unit of work of a batched launch: a range of macroparticles (or of
// window nodes) of one instance of the batch.
struct BatchTile {
  int32_t inst, pad;
  int64_t begin, end;
};

// Per-instance arguments of the batched periodic z2 wrap.
struct WrapArgs {
  double *z2[2];     // z2 of both particle buffers
  int64_t csteps0;   // cumulative steps before the block
  double lenz2;
  int redist, cur0, periodic, pad;
};

struct DiffPlan;  // FFT plan (fft.cu)

enum { PROF_STAGE = 0, PROF_NODES = 1, PROF_FFT = 2, PROF_DIFF = 3, PROF_OTHER = 4, PROF_N = 5 };

struct ProfEvent {
  cudaEvent_t a, b;
  int cls;
};

struct AdjCtx;  // adjoint checkpoints and state (adjoint.cu)
void pf_adj_destroy(AdjCtx *c);

struct pf_handle {
  pf_params p;
  int dev = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  int64_t launches = 0;

  // particles
  int64_t np = 0;
  int64_t cap = 0;
  bool particles_set = false;
  double *y[2][6] = {};       // double-buffered x, y, z2, px, py, gamma
  int cur = 0;
  double *chi = nullptr;
  float *chi_f = nullptr;  // FP32 copy of chi (mixed precision), set with the particles
  float4 *base4 = nullptr; // FP32 x, y, px, py of the step's start state (mixed; stage 1 writes it)
  double *k1[6] = {}, *ka[6] = {}, *kb[6] = {};
  int fix_e = 0, fix_maxexp = 126;
  double chi_max = 0.0;

  // field
  int64_t nouter = 0;         // nx*ny*nz2
  double *or_ = nullptr, *oi_ = nullptr;   // outer mesh
  int nix = 0, niy = 0;       // window
  int64_t npl = 0;            // planes held in the window (nz2 or nz2-1)
  int64_t nwin = 0, wcap = 0;
  double *wr = nullptr, *wi = nullptr;     // window field state
  double *asr = nullptr, *asi = nullptr;   // stage field
  double *d0r = nullptr, *d0i = nullptr, *d12r = nullptr, *d12i = nullptr;
  unsigned long long *acc = nullptr;       // 4 * wcap words
  bool window_valid = false;  // window holds the outer mesh's current values

  // z2 ordering of the macroparticles (pf_run, at the wrap cadence): slot k
  // holds the caller's macroparticle perm[k] while `permuted`
  int32_t *perm = nullptr;
  int *plane_off = nullptr;
  int64_t plane_cap = 0, last_sort = 0, last_check = 0;
  bool permuted = false, sort_z2 = true;


  // mixed precision: interleaved complex-float outer mesh and window arrays
  void *oc32 = nullptr;
  void *w32 = nullptr, *as32 = nullptr, *d0_32 = nullptr, *d12_32 = nullptr, *acc32 = nullptr;
  double *staging = nullptr;  // FP64 staging for field transfers (2 * nouter)
  double *wstage = nullptr;   // FP64 staging of the window field (2 * wstage_cap), mixed
  int64_t wstage_cap = 0;

  // diagnostics scratch
  double *diag = nullptr;
  size_t diag_cap = 0;
  double *lat_scratch = nullptr;  // partial sums of the chi-weighted means

  // snapshot of the particles and the window before an asynchronous step
  // block of pf_run (restored and replayed step by step if the block fails)
  void *snap = nullptr;
  size_t snap_cap = 0;

  AdjCtx *adj = nullptr;

  // graph replay of pf_run's step blocks: the captured block, what it was
  // captured for, and the coefficient table it reads
  cudaGraphExec_t gexec = nullptr;
  int g_len = 0, g_cur = -1;
  const void *g_key[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  void *coef_dev = nullptr;   // device table (StageCoef or its FP32 form)
  void *coef_host = nullptr;  // pinned host staging of the table
  size_t coef_cap = 0;
  int *step_ctr = nullptr;
  bool capturing = false;     // the step drivers emit table reads while set
  bool use_graphs = true;
  int launch_mode = 2;        // pf_set_launch_mode
  bool g_warm = false;        // an uncaptured block ran first (kernel attributes set)
  int64_t g_nlaunch = 0;      // kernels in the captured block

  // completed RK4 steps over the handle's life (the reference's iCsteps); the
  // z2 wrap cadence counts these
  int64_t csteps = 0;

  // taper state
  double n2col = 1.0, n2col0 = 1.0, undgrad = 0.0;
  // piecewise-linear taper profile alpha(z) over control points (empty: the
  // module's linear taper n2col0 + undgrad (z - sZFS))
  std::vector<double> prof_z, prof_a;

  // device scalars
  unsigned int *d_status = nullptr;
  double *d_red = nullptr;    // reduction scratch (window search)
  unsigned int *h_status = nullptr;  // pinned

  DiffPlan *diff = nullptr;
  // FP64 path: diffraction FFTs in paired-FP32 arithmetic (pf_set_fft_arithmetic)
  bool fft_pairs = false;

  // the host-array step (pf_rk4_step_host): a copy stream and its events
  cudaStream_t copy_stream = nullptr;
  std::vector<cudaEvent_t> copy_events;

  // optional per-kernel-class timing
  bool prof = false;
  std::vector<ProfEvent> prof_pending;
  std::vector<ProfEvent> prof_pool;
  double prof_ms[PROF_N] = {};
  int64_t prof_n[PROF_N] = {};
  int prof_open = -1;
};

// Record the start/end of a timed launch of class cls (no-op when disabled).
void pf_prof_begin(pf_handle *h, int cls);
void pf_prof_end(pf_handle *h);
// Accumulate the elapsed times of completed launches (after a stream sync).
void pf_prof_flush(pf_handle *h);

// fp64 RK4 step on the device; returns the device status word.
int pf_rk4_fp64(pf_handle *h, double szl, double hstep, unsigned int *status_out);
// the same step with the particles and the window field in host memory,
// copied in and out around it and overlapped with its kernels; returns the
// status word (the host arrays hold the step's input again when it is set)
int pf_rk4_fp64_host(pf_handle *h, double szl, double hstep, double *const host[6], double *wre,
                     double *wim, unsigned int *status_out);
int pf_rk4_mixed_host(pf_handle *h, double szl, double hstep, double *const host[6], double *wre,
                      double *wim, unsigned int *status_out);
// building blocks of the FP64 step for other drivers (the adjoint)
void pf_fill_stage_args(pf_handle *h, StageArgs &a, double h6);
int pf_launch_stage(pf_handle *h, int stage, StageArgs &a);   // k_stage<stage>
int pf_launch_nodes(pf_handle *h, int stage, NodeArgs &n);    // k_nodes<stage>
// stage-kernel pointers of stage s (1..4) for particle buffer cur
void pf_stage_pointers(pf_handle *h, StageArgs &a, int s, int cur);
// node-kernel arguments of the handle's window
void pf_fill_node_args(pf_handle *h, NodeArgs &n, double hstep);
// batched FP64 launches over (instance, range) tiles; dense-mode shared
// bytes of an instance's window (0: above the shared-memory limit)
cudaError_t pf_stage_batch(cudaStream_t st, int stage, bool tile, const StageArgs *args,
                           const BatchTile *tiles, int ntiles, int grid, int threads, size_t smem);
cudaError_t pf_nodes_batch(cudaStream_t st, int stage, const NodeArgs *args,
                           const BatchTile *tiles, int ntiles, int grid, int threads,
                           int *step_ctr);
cudaError_t pf_wrap_batch(cudaStream_t st, const WrapArgs *args, const BatchTile *tiles,
                          int ntiles, int grid, const int *step_ctr);
size_t pf_stage_tile_smem(const pf_handle *h);
// blocks of a kernel resident on the current device at once (grid < 0 of the
// batched launchers: a persistent grid)
int pf_resident_blocks(const void *kernel, int threads, size_t smem);
// SM count of the current device (cached per device ordinal)
int pf_sm_count();
constexpr int PF_FT_PPB = 8192;  // largest dense-mode tile of the FP64 stage
// batched mixed-precision launches (rk4_mixed.cu); the argument records are
// opaque to the callers
constexpr int PF_MX_THREADS = 512, PF_MX_PPT = 8;
size_t pf_mixed_stage_args_bytes();
size_t pf_mixed_node_args_bytes();
size_t pf_mixed_tile_smem(const pf_handle *h);
void pf_mixed_fill_stage(pf_handle *h, int stage, int cur, double hstep, int tile,
                         const void *coef_tab, const int *step_ctr, unsigned *status, void *out);
void pf_mixed_fill_nodes(pf_handle *h, int stage, double hstep, unsigned *status, void *out);
cudaError_t pf_mixed_stage_batch(cudaStream_t st, int stage, const void *args,
                                 const BatchTile *tiles, int ntiles, int grid, size_t smem);
cudaError_t pf_mixed_nodes_batch(cudaStream_t st, int stage, const void *args,
                                 const BatchTile *tiles, int ntiles, int grid, int threads,
                                 int *step_ctr);
// mixed-precision RK4 step
int pf_rk4_mixed(pf_handle *h, double szl, double hstep, unsigned int *status_out);
// fraction of the macroparticles whose deposit would miss their mixed stage
// block's shared tile (the z2 order a bunched beam loses within steps)
int pf_mixed_order_misses(pf_handle *h, double *frac);
// One stage of the mixed step on explicit arrays (the adjoint's recorded
// forward), with pf_rk4_mixed's stage roles: stage 1 writes kout (k1),
// stage 2 kacc (k2), stage 3 kout (k3) and kacc = kin + k3, stage 4 ynext =
// y + h/6 (k1 + k4 + 2 kacc).  Slope arrays hold FP32 values, except index 2
// (z2), which is FP64; the stage field is one float2 per window node, and
// the deposit goes to the handle's accumulator.
struct PfMixRec {
  const double *y[6];
  const void *as;
  void *kin[6], *kout[6], *kacc[6], *k1[6];
  double *ynext[6];
};
int pf_mixed_stage_rec(pf_handle *h, int stage, double hstep, double sz, const PfMixRec &r);
// the mixed stage kernel's constants for the handle (its adjoint uses them)
struct PfMixConst {
  double aw2g, g02, inv_eta, inv_dz2;
  double ser[7];
  float ser_r1, ser_r2, inv_dx_f, inv_dy_f, hx_dx, hy_dy, eta_f, inv_dV3, sInv2rho, dxc, eta_k2,
      rho2;
};
void pf_mixed_constants(pf_handle *h, PfMixConst *c);
// stage-coefficient table entries of one step (4 entries), FP64 and FP32 forms
void pf_step_coefficients(pf_handle *h, double szl, double hstep, StageCoef *out);
void pf_step_coefficients_f(pf_handle *h, double szl, double hstep, void *out);
size_t pf_step_coefficients_f_bytes();
// window management
int pf_window_from_particles(pf_handle *h, int *nix, int *niy);
int pf_outer_to_inner(pf_handle *h);
int pf_inner_to_outer(pf_handle *h);
// diffraction
int pf_diffract_outer(pf_handle *h, double dz);
// the outer mesh's diffraction (FP64 split, or complex float on a mixed
// handle) with the first and last transverse passes cut into ranges of z2
// planes [zcut[c], zcut[c + 1]): before(c) runs before the first pass reads
// range c, after(c) once the last pass has written it
int pf_diffract_outer_ranges(pf_handle *h, double dz, const std::vector<int64_t> &zcut,
                             const std::function<int(int)> &before,
                             const std::function<int(int)> &after);
// inner2Outer + diffraction + outer2Inner queued on the handle's stream
int pf_diffract_enqueue(pf_handle *h, double dz);
// save (restore) the particles and the window field of an asynchronous block
int pf_block_snapshot(pf_handle *h, bool save);

// The schedule of pf_run (UndSection's loop) for one handle.
struct RunSched {
  int32_t nsteps = 0, isteps4diff = 1, qdiffraction = 0;
  double hstep = 0.0;
  double dzds = 0.0;  // half diffraction step owed by the previous call
  int redist = 60;
  double *szl = nullptr;
  int32_t *steps_done = nullptr;
  bool sync = true;   // false: diffraction is queued without waiting
};
void pf_sched_init(pf_handle *h, RunSched &s, int32_t nsteps, int32_t isteps4diff,
                   int32_t qdiffraction, double hstep, double *szl, int32_t *steps_done);
int pf_sched_after_step(pf_handle *h, RunSched &s, int istep);
int pf_sched_eager_step(pf_handle *h, RunSched &s, int istep);
// adjoint of one FP64 diffraction step over dz on split outer-mesh arrays
int pf_diffract_adjoint_split(pf_handle *h, double *re, double *im, double dz);
// diffraction of an interleaved complex-float outer mesh (mixed precision)
int pf_diffract_outer_c32(pf_handle *h, void *outer, double dz);
// adjoint of one FP32 diffraction step on an interleaved complex-float outer
// mesh (the unique planes; the periodic mirror plane is not written)
int pf_diffract_adjoint_c32(pf_handle *h, void *outer, double dz);
void pf_diff_destroy(DiffPlan *d);

void pf_stage_coefficients(const pf_params &p, double sz, double n2col, int place,
                           BFieldCoef *bf);
void pf_taper_stage(pf_handle *h, double sz, double *n2col, int *place);
double pf_taper_profile_at(const std::vector<double> &z, const std::vector<double> &a, double sz);

// A failed call's error is also taken off the runtime's last-error state, so
// that an allocation failure, which leaves the context usable, is not
// reported again by the next launch check.
#define PF_CUDA(call)                                                     \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess) {                                              \
      (void)cudaGetLastError();                                           \
      h->err = std::string(#call) + ": " + cudaGetErrorString(e_);        \
      return PF_CUDA_ERR;                                                 \
    }                                                                     \
  } while (0)

#define PF_LAUNCHED(h)                                                    \
  do {                                                                    \
    (h)->launches++;                                                      \
    cudaError_t e_ = cudaGetLastError();                                  \
    if (e_ != cudaSuccess) {                                              \
      (h)->err = std::string("kernel launch: ") + cudaGetErrorString(e_); \
      return PF_CUDA_ERR;                                                 \
    }                                                                     \
  } while (0)
