// Diffraction step: batched mixed-radix Stockham FFTs along x, y and z2
// (FP64 complex, unnormalised like FFTW's forward -1 / backward +1
// transforms), the free-space propagator and high-pass filter, and the
// absorbing boundary.
//
// Reference: DiffractionStep / MultiplyExp / AbsorptionStep
// (puffin/lib/diffraction/diffraction.f90:111-523), masks (masks.f90:50-430),
// k-values (transforms.f90:472-590), ffact (setup/setup.f90:334-346).
//
// Each FFT pass kernel loads a group of lines of one axis into shared
// memory (adjacent lines are adjacent in HBM, so the strided y and z2 axes are
// still read in full 32-byte sectors), runs every radix pass of the Stockham
// autosort between two shared-memory buffers and writes the lines back.  The
// propagator and the boundary damping are separable per axis
// (exp(i h (kx^2+ky^2)/2kz) = exp(i h kx^2/2kz) exp(i h ky^2/2kz)), so they
// are applied from two small (x,z2) and (y,z2) tables.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "pf_internal.h"

namespace {

struct cplx {
  double r, i;
};

__device__ __forceinline__ cplx cmul(cplx a, cplx b) {
  return cplx{a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r};
}

constexpr int MAX_PASSES = 16;
constexpr int MAX_RADIX = 64;

struct AxisPlan {
  int n;                 // transform length
  int npass;
  int radix[MAX_PASSES];
  int ns[MAX_PASSES];    // sub-transform size before the pass
  int twoff[MAX_PASSES]; // offset of the pass's twiddles (Ns*R complex each)
  int rootoff[MAX_PASSES];  // offset of the radix's R roots of unity
  int64_t stride;        // element stride along the axis
  int64_t inner;         // lines adjacent in memory (base = L % inner + (L / inner) * ostride)
  int64_t ostride;
  int64_t nlines;
  int lpb;               // lines per block
  cplx *tw_f, *tw_b;     // twiddles, forward and backward
  cplx *roots_f, *roots_b;
};

__device__ __forceinline__ int64_t line_base(const AxisPlan &p, int64_t L) {
  return (L % p.inner) + (L / p.inner) * p.ostride;
}

// One axis, all passes, lpb lines per block.  dir = 0 forward, 1 backward.
__global__ void __launch_bounds__(256) k_fft_axis(cplx *data, const AxisPlan p, int dir) {
  extern __shared__ cplx smem[];
  const int n = p.n;
  const int lpb = p.lpb;
  cplx *buf0 = smem;
  cplx *buf1 = smem + (size_t)lpb * n;
  const int64_t L0 = (int64_t)blockIdx.x * lpb;
  const int nl = (int)min((int64_t)lpb, p.nlines - L0);
  const int tid = threadIdx.x, nt = blockDim.x;

  // load: consecutive threads take consecutive lines (adjacent in memory)
  for (int t = tid; t < nl * n; t += nt) {
    int l, j;
    if (p.stride == 1) {
      l = t / n;
      j = t % n;
    } else {
      l = t % nl;
      j = t / nl;
    }
    buf0[l * n + j] = data[line_base(p, L0 + l) + (int64_t)j * p.stride];
  }
  __syncthreads();

  const cplx *tw = dir ? p.tw_b : p.tw_f;
  const cplx *roots = dir ? p.roots_b : p.roots_f;
  cplx *in = buf0, *out = buf1;
  for (int ps = 0; ps < p.npass; ++ps) {
    const int R = p.radix[ps];
    const int Ns = p.ns[ps];
    const int nb = n / R;
    const cplx *twp = tw + p.twoff[ps];
    const cplx *rt = roots + p.rootoff[ps];
    for (int t = tid; t < nl * nb; t += nt) {
      const int l = t / nb;
      const int j = t % nb;
      const int k = j % Ns;
      const cplx *src = in + l * n;
      cplx *dst = out + l * n;
      const int d = (j / Ns) * Ns * R + k;
      if (R == 2) {
        cplx v0 = src[j], v1 = cmul(src[j + nb], twp[k * 2 + 1]);
        dst[d] = cplx{v0.r + v1.r, v0.i + v1.i};
        dst[d + Ns] = cplx{v0.r - v1.r, v0.i - v1.i};
      } else if (R == 4) {
        cplx v0 = src[j];
        cplx v1 = cmul(src[j + nb], twp[k * 4 + 1]);
        cplx v2 = cmul(src[j + 2 * nb], twp[k * 4 + 2]);
        cplx v3 = cmul(src[j + 3 * nb], twp[k * 4 + 3]);
        cplx a0{v0.r + v2.r, v0.i + v2.i}, a1{v0.r - v2.r, v0.i - v2.i};
        cplx b0{v1.r + v3.r, v1.i + v3.i}, b1{v1.r - v3.r, v1.i - v3.i};
        // multiply b1 by -i (forward) or +i (backward)
        cplx b1r = dir ? cplx{-b1.i, b1.r} : cplx{b1.i, -b1.r};
        dst[d] = cplx{a0.r + b0.r, a0.i + b0.i};
        dst[d + Ns] = cplx{a1.r + b1r.r, a1.i + b1r.i};
        dst[d + 2 * Ns] = cplx{a0.r - b0.r, a0.i - b0.i};
        dst[d + 3 * Ns] = cplx{a1.r - b1r.r, a1.i - b1r.i};
      } else {
        // generic radix: X[q] = sum_r v[r] W_R^(r q)
        cplx v[MAX_RADIX];
        v[0] = src[j];
        for (int r = 1; r < R; ++r) v[r] = cmul(src[j + r * nb], twp[k * R + r]);
        for (int qq = 0; qq < R; ++qq) {
          cplx acc = v[0];
          int e = qq;
          for (int r = 1; r < R; ++r) {
            const cplx w = rt[e];
            acc.r += v[r].r * w.r - v[r].i * w.i;
            acc.i += v[r].r * w.i + v[r].i * w.r;
            e += qq;
            if (e >= R) e -= R;
          }
          dst[d + qq * Ns] = acc;
        }
      }
    }
    __syncthreads();
    cplx *tmp = in;
    in = out;
    out = tmp;
  }

  for (int t = tid; t < nl * n; t += nt) {
    int l, j;
    if (p.stride == 1) {
      l = t / n;
      j = t % n;
    } else {
      l = t % nl;
      j = t / nl;
    }
    data[line_base(p, L0 + l) + (int64_t)j * p.stride] = in[l * n + j];
  }
}

struct MulTables {
  const cplx *px, *py;     // propagator factors (x,z) and (y,z)
  const double *dxt, *dyt; // damping factors (x,z) and (y,z)
  const unsigned char *zflag;  // bit0: pass band, bit1: kz != 0
  const double *mask;      // transverse mask (y,x)
  const double *mz;        // z2 mask
  int nx, ny, nz;
  int qfilter;
  double ffact;
};

__global__ void k_pack(cplx *A, const double *re, const double *im, int64_t n) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) A[t] = cplx{re[t], im[t]};
}

__global__ void k_unpack(const cplx *A, double *re, double *im, int64_t n, int64_t mirror_plane,
                         int64_t plane) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  cplx v = A[t];
  re[t] = v.r;
  im[t] = v.i;
  if (mirror_plane >= 0 && t < plane) {
    re[mirror_plane * plane + t] = v.r;
    im[mirror_plane * plane + t] = v.i;
  }
}

// MultiplyExp (diffraction.f90:111-184)
__global__ void k_propagate(cplx *A, const MulTables T) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t n = (int64_t)T.nx * T.ny * T.nz;
  if (t >= n) return;
  int x = (int)(t % T.nx);
  int y = (int)((t / T.nx) % T.ny);
  int z = (int)(t / ((int64_t)T.nx * T.ny));
  unsigned char f = T.zflag[z];
  if (f & 1) {
    if (f & 2) {
      cplx e = cmul(T.px[(int64_t)z * T.nx + x], T.py[(int64_t)z * T.ny + y]);
      A[t] = cmul(e, A[t]);
    }
  } else if (T.qfilter) {
    A[t] = cplx{0.0, 0.0};
  }
}

// A /= ffact, then the absorbing-boundary split (diffraction.f90:454-470)
__global__ void k_norm_split(cplx *A, cplx *anb, const MulTables T) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t n = (int64_t)T.nx * T.ny * T.nz;
  if (t >= n) return;
  int64_t xy = t % ((int64_t)T.nx * T.ny);
  int z = (int)(t / ((int64_t)T.nx * T.ny));
  cplx a = A[t];
  a.r = a.r / T.ffact;
  a.i = a.i / T.ffact;
  double mk = T.mask[xy];
  double m = mk + T.mz[z] * (1.0 - mk);
  double nbm = 1.0 - m;
  anb[t] = cplx{nbm * a.r, nbm * a.i};
  A[t] = cplx{m * a.r, m * a.i};
}

// boundary damping (diffraction.f90:480-501)
__global__ void k_damp(cplx *A, const MulTables T) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t n = (int64_t)T.nx * T.ny * T.nz;
  if (t >= n) return;
  int x = (int)(t % T.nx);
  int y = (int)((t / T.nx) % T.ny);
  int z = (int)(t / ((int64_t)T.nx * T.ny));
  if (T.zflag[z] & 2) {
    double f = T.dxt[(int64_t)z * T.nx + x] * T.dyt[(int64_t)z * T.ny + y];
    cplx a = A[t];
    A[t] = cplx{f * a.r, f * a.i};
  }
}

// A = A/ffact + anb (diffraction.f90:513-517)
__global__ void k_norm_recombine(cplx *A, const cplx *anb, const MulTables T) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t n = (int64_t)T.nx * T.ny * T.nz;
  if (t >= n) return;
  cplx a = A[t], b = anb[t];
  A[t] = cplx{a.r / T.ffact + b.r, a.i / T.ffact + b.i};
}

// per-call tables: propagator and damping factors for step h
__global__ void k_tables(cplx *px, cplx *py, double *dxt, double *dyt, const double *kx,
                         const double *ky, const double *kz, int nx, int ny, int nz, double h,
                         double sbeta) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t nxz = (int64_t)nx * nz, nyz = (int64_t)ny * nz;
  if (t < nxz) {
    int z = (int)(t / nx), x = (int)(t % nx);
    double kzz = kz[z];
    double th = h * (kx[x] * kx[x]) / (2.0 * kzz);
    double s, c;
    sincos(th, &s, &c);
    px[t] = (kzz != 0.0) ? cplx{c, s} : cplx{1.0, 0.0};
    dxt[t] = (kzz != 0.0) ? exp(-h * sbeta * fabs(kx[x]) / sqrt(fabs(2.0 * kzz))) : 1.0;
  } else if (t < nxz + nyz) {
    t -= nxz;
    int z = (int)(t / ny), y = (int)(t % ny);
    double kzz = kz[z];
    double th = h * (ky[y] * ky[y]) / (2.0 * kzz);
    double s, c;
    sincos(th, &s, &c);
    py[t] = (kzz != 0.0) ? cplx{c, s} : cplx{1.0, 0.0};
    dyt[t] = (kzz != 0.0) ? exp(-h * sbeta * fabs(ky[y]) / sqrt(fabs(2.0 * kzz))) : 1.0;
  }
}

}  // namespace

struct DiffPlan {
  int nx = 0, ny = 0, nz = 0;
  int64_t n = 0;
  AxisPlan ax[3];
  size_t smem[3] = {0, 0, 0};
  cplx *A = nullptr, *anb = nullptr;
  cplx *tw = nullptr;          // all twiddles/roots (forward, backward) in one allocation
  cplx *px = nullptr, *py = nullptr;
  double *dxt = nullptr, *dyt = nullptr;
  double *kx = nullptr, *ky = nullptr, *kz = nullptr;
  double *mask = nullptr, *mz = nullptr;
  unsigned char *zflag = nullptr;
  double ffact = 1.0;
};

void pf_diff_destroy(DiffPlan *d) {
  if (!d) return;
  cudaFree(d->A);
  cudaFree(d->anb);
  cudaFree(d->tw);
  cudaFree(d->px);
  cudaFree(d->py);
  cudaFree(d->dxt);
  cudaFree(d->dyt);
  cudaFree(d->kx);
  cudaFree(d->ky);
  cudaFree(d->kz);
  cudaFree(d->mask);
  cudaFree(d->mz);
  cudaFree(d->zflag);
  delete d;
}

static std::vector<int> factorize(int n) {
  std::vector<int> f;
  while (n % 4 == 0) { f.push_back(4); n /= 4; }
  while (n % 2 == 0) { f.push_back(2); n /= 2; }
  for (int p = 3; n > 1; p += 2) {
    while (n % p == 0) { f.push_back(p); n /= p; }
  }
  return f;
}

// linspace (base_functions.f90:67-98)
static std::vector<double> linspace(double a, double b, int n) {
  std::vector<double> v(n);
  if (n == 1) { v[0] = a; return v; }
  double d = (b - a) / (double)(n - 1);
  for (int i = 0; i < n; ++i) v[i] = a + i * d;
  return v;
}

static double sq(double v) { return v * v; }

// Mask1D2 (masks.f90:266-302): the lower-end assignment is made second and
// wins where the two ends overlap.
static std::vector<double> mask1d2(const std::vector<double> &x, double dx, int nx, int nb) {
  const double pi = PF_PUFFIN_PI;
  std::vector<double> m(nx, 0.0);
  double lb = (nb - 1) * dx, x01 = x[nx - 1], x02 = x[0];
  for (int j = std::max(0, nx - nb); j < nx; ++j) m[j] = sq(cos(pi * (x[j] - x01) / (2.0 * lb)));
  for (int j = 0; j < std::min(nb, nx); ++j) m[j] = sq(cos(pi * (x[j] - x02) / (2.0 * lb)));
  for (int j = nb; j < nx - nb; ++j) m[j] = 0.0;
  return m;
}

// Maskf4 (masks.f90:329-361)
static std::vector<double> maskf4(const std::vector<double> &x, double dx, int nx, int nb) {
  const double pi = PF_PUFFIN_PI;
  std::vector<double> m(nx, 0.0);
  double lb = (nb - 1) * dx, x01 = x[std::max(0, nx - nb)], x02 = x[std::min(nb, nx) - 1];
  for (int j = std::max(0, nx - nb); j < nx; ++j) m[j] = sq(cos(pi * (x[j] - x01) / (2.0 * lb)));
  for (int j = 0; j < std::min(nb, nx); ++j) m[j] = sq(cos(pi * (x[j] - x02) / (2.0 * lb)));
  for (int j = nb; j < nx - nb; ++j) m[j] = 1.0;
  return m;
}

static int build_plan(pf_handle *h) {
  const pf_params &p = h->p;
  DiffPlan *d = new DiffPlan();
  h->diff = d;
  d->nx = p.nx;
  d->ny = p.ny;
  d->nz = (int)h->npl;
  d->n = (int64_t)d->nx * d->ny * d->nz;
  d->ffact = (double)p.nx * (double)p.ny * (double)d->nz;
  const int dims[3] = {d->nx, d->ny, d->nz};
  const int64_t strides[3] = {1, d->nx, (int64_t)d->nx * d->ny};

  std::vector<cplx> tab;  // forward block then backward block
  std::vector<cplx> tabb;
  int max_smem = 0;
  PF_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->dev));
  for (int a = 0; a < 3; ++a) {
    AxisPlan &ap = d->ax[a];
    memset(&ap, 0, sizeof(ap));
    ap.n = dims[a];
    ap.stride = strides[a];
    if (a == 0) {
      ap.inner = 1;
      ap.ostride = d->nx;
      ap.nlines = (int64_t)d->ny * d->nz;
    } else if (a == 1) {
      ap.inner = d->nx;
      ap.ostride = (int64_t)d->nx * d->ny;
      ap.nlines = (int64_t)d->nx * d->nz;
    } else {
      ap.inner = (int64_t)d->nx * d->ny;
      ap.ostride = 0;
      ap.nlines = (int64_t)d->nx * d->ny;
    }
    std::vector<int> f = factorize(ap.n);
    if ((int)f.size() > MAX_PASSES) {
      h->err = "FFT length has too many factors";
      return PF_BAD_ARG;
    }
    for (int r : f)
      if (r > MAX_RADIX) {
        h->err = "FFT length has a prime factor above 64";
        return PF_BAD_ARG;
      }
    ap.npass = (int)f.size();
    int ns = 1;
    for (int ps = 0; ps < ap.npass; ++ps) {
      int R = f[ps];
      ap.radix[ps] = R;
      ap.ns[ps] = ns;
      ap.twoff[ps] = (int)tab.size();
      for (int k = 0; k < ns; ++k)
        for (int r = 0; r < R; ++r) {
          double ang = -2.0 * PF_FULL_PI * (double)(k * r) / (double)(ns * R);
          tab.push_back(cplx{cos(ang), sin(ang)});
          tabb.push_back(cplx{cos(ang), -sin(ang)});
        }
      ap.rootoff[ps] = (int)tab.size();
      for (int r = 0; r < R; ++r) {
        double ang = -2.0 * PF_FULL_PI * (double)r / (double)R;
        tab.push_back(cplx{cos(ang), sin(ang)});
        tabb.push_back(cplx{cos(ang), -sin(ang)});
      }
      ns *= R;
    }
    // lines per block: enough lines for 32-byte sectors on the strided axes,
    // bounded by shared memory (two buffers)
    int lpb = (a == 0) ? std::max(1, 2048 / std::max(1, ap.n)) : 8;
    while (lpb > 1 && (size_t)2 * lpb * ap.n * sizeof(cplx) > (size_t)max_smem) lpb /= 2;
    if ((size_t)2 * lpb * ap.n * sizeof(cplx) > (size_t)max_smem) {
      h->err = "FFT line too long for shared memory";
      return PF_BAD_ARG;
    }
    ap.lpb = lpb;
    d->smem[a] = (size_t)2 * lpb * ap.n * sizeof(cplx);
  }
  size_t ntab = tab.size();
  PF_CUDA(cudaMalloc(&d->tw, 2 * ntab * sizeof(cplx)));
  PF_CUDA(cudaMemcpy(d->tw, tab.data(), ntab * sizeof(cplx), cudaMemcpyHostToDevice));
  PF_CUDA(cudaMemcpy(d->tw + ntab, tabb.data(), ntab * sizeof(cplx), cudaMemcpyHostToDevice));
  for (int a = 0; a < 3; ++a) {
    d->ax[a].tw_f = d->tw;
    d->ax[a].roots_f = d->tw;
    d->ax[a].tw_b = d->tw + ntab;
    d->ax[a].roots_b = d->tw + ntab;
  }
  PF_CUDA(cudaFuncSetAttribute(k_fft_axis, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));

  PF_CUDA(cudaMalloc(&d->A, d->n * sizeof(cplx)));
  PF_CUDA(cudaMalloc(&d->anb, d->n * sizeof(cplx)));
  PF_CUDA(cudaMalloc(&d->px, (size_t)d->nx * d->nz * sizeof(cplx)));
  PF_CUDA(cudaMalloc(&d->py, (size_t)d->ny * d->nz * sizeof(cplx)));
  PF_CUDA(cudaMalloc(&d->dxt, (size_t)d->nx * d->nz * sizeof(double)));
  PF_CUDA(cudaMalloc(&d->dyt, (size_t)d->ny * d->nz * sizeof(double)));

  // k-values (transforms.f90:472-590), full-precision pi
  auto kvals = [](int m, double len) {
    std::vector<double> k(m);
    int mx = (int)ceil((double)m / 2.0);
    for (int i = 0; i < m; ++i) k[i] = 2.0 * PF_FULL_PI * (double)(i >= mx ? i - m : i) / len;
    return k;
  };
  std::vector<double> kx = kvals(d->nx, (double)d->nx * p.dx);
  std::vector<double> ky = kvals(d->ny, (double)d->ny * p.dy);
  std::vector<double> kz = kvals(d->nz, (double)d->nz * p.dz2);
  PF_CUDA(cudaMalloc(&d->kx, kx.size() * sizeof(double)));
  PF_CUDA(cudaMalloc(&d->ky, ky.size() * sizeof(double)));
  PF_CUDA(cudaMalloc(&d->kz, kz.size() * sizeof(double)));
  PF_CUDA(cudaMemcpy(d->kx, kx.data(), kx.size() * sizeof(double), cudaMemcpyHostToDevice));
  PF_CUDA(cudaMemcpy(d->ky, ky.data(), ky.size() * sizeof(double), cudaMemcpyHostToDevice));
  PF_CUDA(cudaMemcpy(d->kz, kz.data(), kz.size() * sizeof(double), cudaMemcpyHostToDevice));

  // filter cutoff (diffraction.f90:138-139; sFilt from setup_calcs.f90:208-210)
  const double ppi = PF_PUFFIN_PI;
  double lenz2 = p.dz2 * p.nz2;
  double sfilt = lenz2 / (4 * ppi * p.rho) * p.sfilt_frac;
  double cutoff = 2.0 * ppi * sfilt / ((double)p.nz2 * p.dz2);
  if (p.mesh_type == PF_MESH_PERIODIC && p.sperwaves <= 1.1) cutoff = 0.0;
  std::vector<unsigned char> zf(d->nz);
  for (int z = 0; z < d->nz; ++z)
    zf[z] = (unsigned char)(((kz[z] > cutoff) || (kz[z] < -cutoff)) ? 1 : 0) |
            (unsigned char)((kz[z] != 0.0) ? 2 : 0);
  PF_CUDA(cudaMalloc(&d->zflag, zf.size()));
  PF_CUDA(cudaMemcpy(d->zflag, zf.data(), zf.size(), cudaMemcpyHostToDevice));

  // masks (masks.f90:50-189, 366-430)
  double lenx = (d->nx - 1) * p.dx, leny = (d->ny - 1) * p.dy;
  std::vector<double> xs = linspace(-lenx / 2, lenx / 2, d->nx);
  std::vector<double> ys = linspace(-leny / 2, leny / 2, d->ny);
  std::vector<double> maskx = mask1d2(xs, p.dx, d->nx, p.nbx);
  std::vector<double> masky = mask1d2(ys, p.dy, d->ny, p.nby);
  std::vector<double> maskx2 = maskf4(xs, p.dx, d->nx, p.nbx);
  std::vector<double> m2((size_t)d->nx * d->ny);
  for (int y = 0; y < d->ny; ++y)
    for (int x = 0; x < d->nx; ++x) m2[(size_t)y * d->nx + x] = 1.0 * maskx[x] + maskx2[x] * masky[y];
  std::vector<double> mzv(d->nz, 0.0);
  if (p.mesh_type != PF_MESH_PERIODIC) {
    double dx = p.dz2;
    std::vector<double> xz = linspace(0.0 * dx, (double)(d->nz - 1) * dx, d->nz);
    double lb = (p.nbz2 - 1) * dx;
    double lf = (p.nz2 - 1 * dx);  // getZ2Mask's own form (masks.f90:366-430)
    double x0 = lf - lb / 2.0;
    int fbn = p.nz2 - p.nbz2 + 1;
    for (int i = 0; i < d->nz; ++i)
      if (i + 1 >= fbn) mzv[i] = sq(cos(ppi * (xz[i] - x0) / lb));
  }
  PF_CUDA(cudaMalloc(&d->mask, m2.size() * sizeof(double)));
  PF_CUDA(cudaMalloc(&d->mz, mzv.size() * sizeof(double)));
  PF_CUDA(cudaMemcpy(d->mask, m2.data(), m2.size() * sizeof(double), cudaMemcpyHostToDevice));
  PF_CUDA(cudaMemcpy(d->mz, mzv.data(), mzv.size() * sizeof(double), cudaMemcpyHostToDevice));
  return PF_OK;
}

static int fft3(pf_handle *h, DiffPlan *d, int dir) {
  for (int a = 0; a < 3; ++a) {
    const AxisPlan &ap = d->ax[a];
    if (ap.n == 1) continue;
    int64_t blocks = (ap.nlines + ap.lpb - 1) / ap.lpb;
    pf_prof_begin(h, PROF_FFT);
    k_fft_axis<<<(unsigned)blocks, 256, d->smem[a], h->stream>>>(d->A, ap, dir);
    pf_prof_end(h);
    PF_LAUNCHED(h);
  }
  return PF_OK;
}

int pf_diffract_outer(pf_handle *h, double dz) {
  const pf_params &p = h->p;
  if (!h->diff) {
    int rc = build_plan(h);
    if (rc) return rc;
  }
  DiffPlan *d = h->diff;
  const int threads = 256;
  const unsigned g = (unsigned)((d->n + threads - 1) / threads);
  MulTables T;
  T.px = d->px;
  T.py = d->py;
  T.dxt = d->dxt;
  T.dyt = d->dyt;
  T.zflag = d->zflag;
  T.mask = d->mask;
  T.mz = d->mz;
  T.nx = d->nx;
  T.ny = d->ny;
  T.nz = d->nz;
  T.qfilter = p.qfilter;
  T.ffact = d->ffact;

  int64_t ntab = (int64_t)(d->nx + d->ny) * d->nz;
  pf_prof_begin(h, PROF_DIFF);
  k_tables<<<(unsigned)((ntab + threads - 1) / threads), threads, 0, h->stream>>>(
      d->px, d->py, d->dxt, d->dyt, d->kx, d->ky, d->kz, d->nx, d->ny, d->nz, dz, p.sbeta);
  pf_prof_end(h);
  PF_LAUNCHED(h);
  pf_prof_begin(h, PROF_DIFF);
  k_pack<<<g, threads, 0, h->stream>>>(d->A, h->or_, h->oi_, d->n);
  pf_prof_end(h);
  PF_LAUNCHED(h);
  int rc = fft3(h, d, 0);
  if (rc) return rc;
  pf_prof_begin(h, PROF_DIFF);
  k_propagate<<<g, threads, 0, h->stream>>>(d->A, T);
  pf_prof_end(h);
  PF_LAUNCHED(h);
  rc = fft3(h, d, 1);
  if (rc) return rc;
  pf_prof_begin(h, PROF_DIFF);
  k_norm_split<<<g, threads, 0, h->stream>>>(d->A, d->anb, T);
  pf_prof_end(h);
  PF_LAUNCHED(h);
  rc = fft3(h, d, 0);
  if (rc) return rc;
  pf_prof_begin(h, PROF_DIFF);
  k_damp<<<g, threads, 0, h->stream>>>(d->A, T);
  pf_prof_end(h);
  PF_LAUNCHED(h);
  rc = fft3(h, d, 1);
  if (rc) return rc;
  pf_prof_begin(h, PROF_DIFF);
  k_norm_recombine<<<g, threads, 0, h->stream>>>(d->A, d->anb, T);
  pf_prof_end(h);
  PF_LAUNCHED(h);
  const int64_t plane = (int64_t)d->nx * d->ny;
  const int64_t mirror = (p.mesh_type == PF_MESH_PERIODIC) ? (int64_t)d->nz : -1;
  pf_prof_begin(h, PROF_DIFF);
  k_unpack<<<g, threads, 0, h->stream>>>(d->A, h->or_, h->oi_, d->n, mirror, plane);
  pf_prof_end(h);
  PF_LAUNCHED(h);
  return PF_OK;
}
