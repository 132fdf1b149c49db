// Beam-line elements either side of the undulator modules, applied to the
// macroparticle state held on the device: drift, chicane (dispersion), quad
// point transform, energy modulation, the undulator entry/exit matching and
// the transverse re-centring, plus the per-module undulator set-up.
//
// Reference: puffin/lib/acc_lattice.f90 — disperse :420-463, driftSection
// :478-518, Quad :531-561, bModulation :575-585, correctTrans :601-623,
// matchOut :638-725, matchIn :743-828, initUndulator :848-895; offsets
// pxOffset / pyOffset / xOffSet_Array / yOffSet_Array
// (puffin/lib/undulator/init_conds.f90:68-223); the chi-weighted mean
// arr_mean_para_weighted (puffin/lib/utilities/base_functions.f90:552-573).
//
// Products that the reference adds to another term are formed with
// __dmul_rn so that the compiler contracts nothing into an FMA: these
// element maps then round exactly as the reference's sequential FP64 code,
// except for sin/cos, which are the CUDA library's.
#include <math.h>

#include "pf_internal.h"

namespace {

constexpr int kRedBlocks = 304;  // 2 x 152 SMs; fixed so sums are reproducible
constexpr int kRedThreads = 256;

inline unsigned grid_for(int64_t n, int threads) {
  const int64_t g = (n + threads - 1) / threads;
  return (unsigned)(g < 1 ? 1 : g);
}

// getP2 (gamma_to_p2.f90:84-85) in the reference's operation order
__device__ inline double p2_ref(double gam, double px, double py, double g0sq, double awsq,
                                double eta) {
  const double a = 1.0 / __dmul_rn(g0sq, __dmul_rn(gam, gam));
  const double b = 1.0 + __dmul_rn(awsq, __dmul_rn(px, px) + __dmul_rn(py, py));
  return ((1.0 / sqrt(1.0 - __dmul_rn(a, b))) - 1.0) / eta;
}

// driftSection: z2 += dz p2; x += (2 rho kappa / sqrt(eta) (1 + eta p2) / Gamma px) dz,
// y -= (... py) dz
__global__ void k_drift(double *x, double *y, double *z2, const double *px, const double *py,
                        const double *gam, int64_t n, double dz, double g0sq, double awsq,
                        double eta, double c2rk, int one_d) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double G = gam[i], PX = px[i], PY = py[i];
  const double p2 = p2_ref(G, PX, PY, g0sq, awsq, eta);
  z2[i] = z2[i] + __dmul_rn(dz, p2);
  if (!one_d) {
    const double q = __dmul_rn(c2rk, 1.0 + __dmul_rn(eta, p2)) / G;  // c2rk = 2 rho kappa / sqrt(eta)
    x[i] = x[i] + __dmul_rn(__dmul_rn(q, PX), dz);
    y[i] = y[i] - __dmul_rn(__dmul_rn(q, PY), dz);
  }
}

// disperse: z2 = z2 - 2 D (Gamma - 1) + slip
__global__ void k_chicane(double *z2, const double *gam, int64_t n, double disp2, double slip) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  z2[i] = (z2[i] - __dmul_rn(disp2, gam[i] - 1.0)) + slip;
}

// Quad: px += sqrt(eta)/(2 rho kappa) x / fx ; py -= sqrt(eta)/(2 rho kappa) y / fy
__global__ void k_quad(const double *x, const double *y, double *px, double *py, int64_t n,
                       double c, double qfx, double qfy) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  px[i] = px[i] + __dmul_rn(c, x[i]) / qfx;
  py[i] = py[i] - __dmul_rn(c, y[i]) / qfy;
}

// bModulation: Gamma += mag cos(k z2)
__global__ void k_modulation(const double *z2, double *gam, int64_t n, double mag, double k) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  gam[i] = gam[i] + __dmul_rn(mag, cos(__dmul_rn(k, z2[i])));
}

// matchIn (sign +1) / matchOut (sign -1).  Stage-uniform scalars from the host:
// pxo = pxOffset, pyo = pyOffset, cx = uy 4 kappa rho^2 / sqrt(eta) (and cy with
// ux), sn = sin(sz / 2 rho), cs = cos(sz / 2 rho).
struct MatchArgs {
  double *x, *y, *px, *py;
  const double *gam;
  int64_t n;
  int type;
  double sign;
  double pxo, pyo, kx2, ky2, eta_4rho2;
  double gamma_r, ncx, ncy, cx, cy, n2col, sn, cs;
};

__global__ void k_match(MatchArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double X = a.x[i], Y = a.y[i];
  double spx, spy;
  if (a.type == PF_UND_CURVED) {
    spx = (a.pxo - __dmul_rn(0.5 * a.kx2, __dmul_rn(X, X))) - __dmul_rn(0.5 * a.ky2, __dmul_rn(Y, Y));
    spy = -1.0 * (a.pyo - __dmul_rn(__dmul_rn(a.kx2, X), Y));
  } else if (a.type == PF_UND_PLANEPOLE) {
    spx = a.pxo - __dmul_rn(0.5 * a.eta_4rho2, __dmul_rn(X, X));
    spy = -1.0 * a.pyo;
  } else {
    spx = a.pxo;
    spy = -1.0 * a.pyo;
  }
  const double gj = a.gamma_r * a.gam[i];
  const double pp = __dmul_rn(spx, spx) + __dmul_rn(spy, spy);
  const double gj2 = __dmul_rn(gj, gj);
  const double tx = a.gamma_r / sqrt(gj2 - (1.0 + __dmul_rn(a.ncx, pp)));
  const double ty = a.gamma_r / sqrt(gj2 - (1.0 + __dmul_rn(a.ncy, pp)));
  const double sxo = -(((a.cx * tx) * a.n2col) * a.sn);
  const double syo = ((a.cy * ty) * a.n2col) * a.cs;
  if (a.sign > 0) {
    a.x[i] = X + sxo;
    a.y[i] = Y + syo;
    a.px[i] = a.px[i] + spx;
    a.py[i] = a.py[i] + spy;
  } else {
    a.x[i] = X - sxo;
    a.y[i] = Y - syo;
    a.px[i] = a.px[i] - spx;
    a.py[i] = a.py[i] - spy;
  }
}

// correctTrans, pass 1: per-block sums of chi, chi px, chi py, chi x, chi y
// over a fixed grid (reproducible: the same partition every call)
__global__ void __launch_bounds__(kRedThreads) k_wsum(const double *x, const double *y,
                                                      const double *px, const double *py,
                                                      const double *chi, int64_t n,
                                                      double *part) {
  __shared__ double s[5][kRedThreads];
  double a[5] = {0, 0, 0, 0, 0};
  for (int64_t i = (int64_t)blockIdx.x * kRedThreads + threadIdx.x; i < n;
       i += (int64_t)kRedBlocks * kRedThreads) {
    const double w = chi[i];
    a[0] += w;
    a[1] += w * px[i];
    a[2] += w * py[i];
    a[3] += w * x[i];
    a[4] += w * y[i];
  }
  for (int k = 0; k < 5; ++k) s[k][threadIdx.x] = a[k];
  __syncthreads();
  for (int st = kRedThreads / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int k = 0; k < 5; ++k) s[k][threadIdx.x] += s[k][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 5; ++k) part[(int64_t)k * kRedBlocks + blockIdx.x] = s[k][0];
}

// pass 2: one block folds the partials and forms the four means
__global__ void __launch_bounds__(kRedThreads) k_wmean(const double *part, double *mean) {
  __shared__ double s[5][kRedThreads];
  for (int k = 0; k < 5; ++k) {
    double v = 0.0;
    for (int b = threadIdx.x; b < kRedBlocks; b += kRedThreads) v += part[(int64_t)k * kRedBlocks + b];
    s[k][threadIdx.x] = v;
  }
  __syncthreads();
  for (int st = kRedThreads / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int k = 0; k < 5; ++k) s[k][threadIdx.x] += s[k][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 1; k < 5; ++k) mean[k - 1] = s[k][0] / s[0][0];
}

// pass 3: subtract the means
__global__ void k_center(double *x, double *y, double *px, double *py, int64_t n,
                         const double *mean) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  px[i] -= mean[0];
  py[i] -= mean[1];
  x[i] -= mean[2];
  y[i] -= mean[3];
}

__global__ void k_wrap(double *z2, int64_t n, double lenz2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) z2[i] = z2[i] - (floor(z2[i] / lenz2) * lenz2);
}

}  // namespace

static int lattice_ready(pf_handle *h) {
  if (!h) return PF_BAD_ARG;
  if (!h->particles_set) {
    h->err = "no macroparticles set";
    return PF_STATE;
  }
  cudaSetDevice(h->dev);
  return PF_OK;
}

extern "C" {

int pf_drift(pf_handle *h, double dz, int32_t qdiffraction) {
  int rc = lattice_ready(h);
  if (rc) return rc;
  const pf_params &p = h->p;
  double *const *s = h->y[h->cur];
  if (h->np > 0) {
    const double c2rk = 2.0 * p.rho * p.kappa / sqrt(p.eta);
    k_drift<<<grid_for(h->np, 256), 256, 0, h->stream>>>(
        s[0], s[1], s[2], s[3], s[4], s[5], h->np, dz, p.gamma_r * p.gamma_r, p.aw * p.aw, p.eta,
        c2rk, p.one_d);
    PF_LAUNCHED(h);
  }
  if (qdiffraction) return pf_diffract(h, dz);
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

int pf_chicane(pf_handle *h, double disp, double slip, double zbar, int32_t qdiffraction) {
  int rc = lattice_ready(h);
  if (rc) return rc;
  const pf_params &p = h->p;
  double *const *s = h->y[h->cur];
  if (h->np > 0) {
    k_chicane<<<grid_for(h->np, 256), 256, 0, h->stream>>>(s[2], s[5], h->np, 2.0 * disp, slip);
    PF_LAUNCHED(h);
  }
  if (qdiffraction && zbar > 0.0) {
    rc = pf_diffract(h, zbar);
    if (rc) return rc;
  }
  if (p.mesh_type == PF_MESH_PERIODIC && h->np > 0) {
    const double lenz2 = p.dz2 * (double)(p.nz2 - 1);
    k_wrap<<<grid_for(h->np, 256), 256, 0, h->stream>>>(s[2], h->np, lenz2);
    PF_LAUNCHED(h);
  }
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

int pf_quad(pf_handle *h, double qfx, double qfy) {
  int rc = lattice_ready(h);
  if (rc) return rc;
  if (qfx == 0.0 || qfy == 0.0) return PF_BAD_ARG;
  const pf_params &p = h->p;
  double *const *s = h->y[h->cur];
  if (!p.one_d && h->np > 0) {
    const double c = sqrt(p.eta) / (2.0 * p.rho * p.kappa);
    k_quad<<<grid_for(h->np, 256), 256, 0, h->stream>>>(s[0], s[1], s[3], s[4], h->np, c, qfx,
                                                         qfy);
    PF_LAUNCHED(h);
  }
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

int pf_modulation(pf_handle *h, double mag, double wavenum) {
  int rc = lattice_ready(h);
  if (rc) return rc;
  double *const *s = h->y[h->cur];
  if (h->np > 0) {
    k_modulation<<<grid_for(h->np, 256), 256, 0, h->stream>>>(s[2], s[5], h->np, mag, wavenum);
    PF_LAUNCHED(h);
  }
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

static int match(pf_handle *h, double sz, double sign) {
  int rc = lattice_ready(h);
  if (rc) return rc;
  if (h->np == 0) return PF_OK;
  const pf_params &p = h->p;
  double *const *s = h->y[h->cur];
  MatchArgs a;
  a.x = s[0];
  a.y = s[1];
  a.px = s[3];
  a.py = s[4];
  a.gam = s[5];
  a.n = h->np;
  a.type = p.und_type;
  a.sign = sign;
  const double ph = sz / (2.0 * p.rho);
  a.pxo = -((p.fy * h->n2col) * cos(ph));
  a.pyo = -((p.fx * h->n2col) * sin(ph));
  a.kx2 = p.kx_und * p.kx_und;
  a.ky2 = p.ky_und * p.ky_und;
  a.eta_4rho2 = p.eta / (4.0 * (p.rho * p.rho));
  a.gamma_r = p.gamma_r;
  a.ncx = p.aw * p.aw;
  a.ncy = 2.0 * (p.aw * p.aw) / (p.fx * p.fx + p.fy * p.fy);
  a.cx = ((p.fy * 4.0) * p.kappa) * (p.rho * p.rho) / sqrt(p.eta);
  a.cy = ((p.fx * 4.0) * p.kappa) * (p.rho * p.rho) / sqrt(p.eta);
  a.n2col = h->n2col;
  a.sn = sin(ph);
  a.cs = cos(ph);
  k_match<<<grid_for(h->np, 256), 256, 0, h->stream>>>(a);
  PF_LAUNCHED(h);
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

int pf_match_in(pf_handle *h, double sz) { return match(h, sz, 1.0); }
int pf_match_out(pf_handle *h, double sz) { return match(h, sz, -1.0); }

int pf_correct_trans(pf_handle *h) {
  int rc = lattice_ready(h);
  if (rc) return rc;
  if (h->np == 0) return PF_OK;
  double *const *s = h->y[h->cur];
  double *part = h->lat_scratch;
  if (!part) {
    PF_CUDA(cudaMalloc(&h->lat_scratch, sizeof(double) * (5 * kRedBlocks + 4)));
    part = h->lat_scratch;
  }
  k_wsum<<<kRedBlocks, kRedThreads, 0, h->stream>>>(s[0], s[1], s[3], s[4], h->chi, h->np, part);
  PF_LAUNCHED(h);
  k_wmean<<<1, kRedThreads, 0, h->stream>>>(part, part + 5 * kRedBlocks);
  PF_LAUNCHED(h);
  k_center<<<grid_for(h->np, 256), 256, 0, h->stream>>>(s[0], s[1], s[3], s[4], h->np,
                                                         part + 5 * kRedBlocks);
  PF_LAUNCHED(h);
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

int pf_init_undulator(pf_handle *h, int32_t und_type, double fx, double fy, double kbxsf,
                      double kbysf, double mf, double taper, int32_t nsteps, double hstep,
                      int32_t und_ends) {
  if (!h) return PF_BAD_ARG;
  if (und_type < PF_UND_PUFFIN || und_type > PF_UND_CURVED || nsteps < 0 || !(hstep > 0.0))
    return PF_BAD_ARG;
  pf_params &p = h->p;
  h->n2col0 = mf;
  h->n2col = mf;
  h->undgrad = taper;
  p.n2col0 = mf;
  p.undgrad = taper;
  p.und_type = und_type;
  p.fx = fx;
  p.fy = fy;
  p.kbxsf = kbxsf;
  p.kbysf = kbysf;
  p.und_ends = und_ends ? 1 : 0;
  const double pi = PF_PUFFIN_PI;
  if (und_ends) {
    p.szfs = 4.0 * pi * p.rho * 2.0;
    p.szfe = nsteps * hstep - 4.0 * pi * p.rho * 2.0;
  } else {
    p.szfs = 0.0;
    p.szfe = nsteps * hstep;
  }
  return PF_OK;
}

}  // extern "C"
