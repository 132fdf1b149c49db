// On-device diagnostics of the run state: radiated power per z2 slice,
// bunching factor per slice, and the on-axis spectrum.
//
// Reference: gPower / fPower_1D / fPower_3D with m_trapz2D / m_trapz
// (puffin/lib/io/av_write.f90:112-276), the bunching sums of getSliceTwiss
// (av_write.f90:405-770, b1..b5 at :562-650) with the slice count of
// write_adapter.f90:110-112, and the spectrum of
// utilities/pyPlotting/plotSpecPow.py:58-95.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <vector>

#include "pf_internal.h"

namespace {

// one block per z2 plane: m_trapz along x for every row (one thread per row,
// accumulated in single precision as the reference's default-real m_trapz),
// then m_trapz along y over the row integrals
__global__ void k_power(const double *re, const double *im, const float2 *oc, int nx, int ny,
                        int64_t nz2, const double *xax, const double *yax, double *power) {
  extern __shared__ double cul[];
  const int64_t z = blockIdx.x;
  if (z >= nz2) return;
  const int64_t base = z * (int64_t)nx * ny;
  auto intens = [&](int64_t i) {
    double r, m;
    if (oc) {
      r = (double)oc[i].x;
      m = (double)oc[i].y;
    } else {
      r = re[i];
      m = im[i];
    }
    return r * r + m * m;
  };
  if (nx == 1 && ny == 1) {  // fPower_1D
    if (threadIdx.x == 0) power[z] = intens(base);
    return;
  }
  for (int iy = threadIdx.x; iy < ny; iy += blockDim.x) {
    float acc = 0.f;
    const int64_t row = base + (int64_t)iy * nx;
    double yi = intens(row);
    for (int i = 0; i < nx - 1; ++i) {
      const double yn = intens(row + i + 1);
      acc = (float)((double)acc + (xax[i + 1] - xax[i]) * (yn + yi) / 2.0);
      yi = yn;
    }
    cul[iy] = (double)acc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float acc = 0.f;
    for (int i = 0; i < ny - 1; ++i)
      acc = (float)((double)acc + (yax[i + 1] - yax[i]) * (cul[i + 1] + cul[i]) / 2.0);
    power[z] = (double)acc;
  }
}

// bunching at harmonic m with linear slice weights (av_write.f90:562-650).
// Macroparticles are ordered along z2, so a block's particles fall in a few
// consecutive slices: each block sums into shared bins from its lowest slice
// and adds the bins to HBM once; slices outside the bins go to HBM directly.
constexpr int BUNCH_BINS = 64;
__global__ void k_bunching(const double *z2, const double *chi, int64_t np, int harmonic,
                           double rho, double S, int nslices, int periodic, double *br,
                           double *bi, double *sd, unsigned int *status) {
  __shared__ double s_r[BUNCH_BINS], s_i[BUNCH_BINS], s_d[BUNCH_BINS];
  __shared__ int s_base;
  for (int t = threadIdx.x; t < BUNCH_BINS; t += blockDim.x) {
    s_r[t] = 0.0;
    s_i[t] = 0.0;
    s_d[t] = 0.0;
  }
  if (threadIdx.x == 0) s_base = INT_MAX;
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int is = 0;
  bool ok = false;
  double z = 0.0, c = 0.0;
  if (i < np) {
    z = z2[i];
    c = chi[i];
    is = (int)ceil(z / S);
    ok = true;
    if (periodic) {
      if (is >= nslices) is = is - (int)(floor((double)is / (double)nslices) * nslices) + 1;
      if (is < 1) ok = false;
    } else if (is > nslices || is < 1) {
      ok = false;
    }
    if (!ok) atomicOr(status, 1u);
    else atomicMin(&s_base, is - 1);
  }
  __syncthreads();
  const int base = s_base;
  // The z2-ordered macroparticles of a warp fall in one or two slices: their
  // contributions are summed across the warp first, one pass per distinct
  // slice (a butterfly over all 32 lanes of the members' values), and one
  // lane per slice adds the sums to the block's bins -- shared FP64 atomics
  // to one address from every lane would serialise.  Every lane of the warp
  // takes part (a macroparticle without a slice contributes nothing).
  auto add = [&](int slot, double vr, double vi, double vd) {
    const int lane = threadIdx.x & 31;
    unsigned todo = __ballot_sync(0xffffffffu, slot >= 0);
    while (todo) {
      const int leader = __ffs(todo) - 1;
      const int ls = __shfl_sync(0xffffffffu, slot, leader);
      const bool member = (slot == ls);
      double sr = member ? vr : 0.0, si = member ? vi : 0.0, sdv = member ? vd : 0.0;
      for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        si += __shfl_xor_sync(0xffffffffu, si, o);
        sdv += __shfl_xor_sync(0xffffffffu, sdv, o);
      }
      todo &= ~__ballot_sync(0xffffffffu, member);
      if (lane != leader) continue;
      const int b = ls - base;
      if (b >= 0 && b < BUNCH_BINS) {
        atomicAdd(s_r + b, sr);
        atomicAdd(s_i + b, si);
        if (sdv != 0.0) atomicAdd(s_d + b, sdv);
      } else {
        atomicAdd(br + ls, sr);
        atomicAdd(bi + ls, si);
        if (sdv != 0.0) atomicAdd(sd + ls, sdv);
      }
    }
  };
  double sn = 0.0, cs = 0.0, w0 = 0.0;
  if (ok) {
    const double ph = (double)harmonic * z / (2.0 * rho);
    sincos(ph, &sn, &cs);
    w0 = (is * S - z) / S;
  }
  add(ok ? is - 1 : -1, c * cs * w0, c * sn * w0, c);
  if (!periodic) {
    const double w1 = ok ? -((is - 1) * S - z) / S : 0.0;
    add(ok ? is : -1, c * cs * w1, c * sn * w1, 0.0);  // slice is+1 (the arrays hold nslices+1)
  }
  __syncthreads();
  if (base == INT_MAX) return;
  for (int t = threadIdx.x; t < BUNCH_BINS; t += blockDim.x) {
    const int slot = base + t;
    if (slot > nslices) break;
    if (s_r[t] != 0.0) atomicAdd(br + slot, s_r[t]);
    if (s_i[t] != 0.0) atomicAdd(bi + slot, s_i[t]);
    if (s_d[t] != 0.0) atomicAdd(sd + slot, s_d[t]);
  }
}

// one-sided |DFT|^2 of the on-axis field (plotSpecPow.py:83-95), direct sum
// with the roots of unity from a table (root index k z mod n)
__global__ void k_spectrum(const double *re, const double *im, const float2 *oc, int64_t stride,
                           int64_t off, int64_t n, int64_t nu, const double2 *roots, double *sx,
                           double *sy) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nu) return;
  double xr = 0.0, xi = 0.0, yr = 0.0, yi = 0.0;
  int64_t m = 0;
  for (int64_t z = 0; z < n; ++z) {
    const int64_t pos = off + z * stride;
    const double a = oc ? (double)oc[pos].x : re[pos];
    const double b = oc ? (double)oc[pos].y : im[pos];
    const double2 w = roots[m];  // (cos, -sin)(2 pi k z / n)
    xr = fma(a, w.x, xr);
    xi = fma(a, w.y, xi);
    yr = fma(b, w.x, yr);
    yi = fma(b, w.y, yi);
    m += k;
    if (m >= n) m -= n;
  }
  double px = xr * xr + xi * xi, py = yr * yr + yi * yi;
  // one-sided power: double every bin but DC (and the Nyquist bin of an even n)
  if (k > 0 && ((n % 2) == 1 || k < nu - 1)) {
    px *= 2.0;
    py *= 2.0;
  }
  sx[k] = px;
  sy[k] = py;
}

}  // namespace

static int diag_scratch(pf_handle *h, size_t doubles, double **out) {
  // the diagnostic buffers reuse one lazily grown device array
  static_assert(sizeof(double) == 8, "");
  if (h->diag_cap < doubles) {
    cudaFree(h->diag);
    h->diag = nullptr;
    h->diag_cap = 0;
    PF_CUDA(cudaMalloc(&h->diag, doubles * sizeof(double)));
    h->diag_cap = doubles;
  }
  *out = h->diag;
  return PF_OK;
}

extern "C" {

int64_t pf_num_slices(const pf_handle *h) {
  if (!h) return -1;
  const double pi = PF_PUFFIN_PI;
  const pf_params &p = h->p;
  if (p.mesh_type == PF_MESH_TEMPORAL)
    return (int64_t)ceil((p.dz2 * p.nz2) / (4 * pi * p.rho));
  return (int64_t)ceil((p.dz2 * (double)(p.nz2 - 1)) / (4 * pi * p.rho));
}

int pf_power(pf_handle *h, double *power, int64_t n) {
  if (!h || !power || n != h->p.nz2) return PF_BAD_ARG;
  cudaSetDevice(h->dev);
  int rc = pf_inner_to_outer(h);
  if (rc) return rc;
  const pf_params &p = h->p;
  double *d;
  rc = diag_scratch(h, (size_t)p.nz2 + p.nx + p.ny, &d);
  if (rc) return rc;
  // axes: linspace(-l/2, l/2, n) with l = d*(n-1) (av_write.f90:76-98)
  std::vector<double> ax((size_t)p.nx + p.ny);
  auto lin = [&](double len, int m, double *o) {
    if (m == 1) {
      o[0] = -len / 2.0;
      return;
    }
    const double dd = (len / 2.0 - (-len / 2.0)) / (double)(m - 1);
    for (int i = 0; i < m; ++i) o[i] = -len / 2.0 + i * dd;
  };
  lin(p.dx * (p.nx - 1), p.nx, ax.data());
  lin(p.dy * (p.ny - 1), p.ny, ax.data() + p.nx);
  PF_CUDA(cudaMemcpyAsync(d + p.nz2, ax.data(), ax.size() * sizeof(double), cudaMemcpyHostToDevice,
                          h->stream));
  const bool mixed = h->p.precision == PF_MIXED;
  k_power<<<(unsigned)p.nz2, 128, (size_t)p.ny * sizeof(double), h->stream>>>(
      mixed ? nullptr : h->or_, mixed ? nullptr : h->oi_, mixed ? (const float2 *)h->oc32 : nullptr,
      p.nx, p.ny, p.nz2, d + p.nz2, d + p.nz2 + p.nx, d);
  PF_LAUNCHED(h);
  PF_CUDA(cudaMemcpyAsync(power, d, sizeof(double) * p.nz2, cudaMemcpyDeviceToHost, h->stream));
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

int pf_bunching(pf_handle *h, int32_t harmonic, double *b, int64_t nslices) {
  if (!h || !b || harmonic < 1 || nslices != pf_num_slices(h)) return PF_BAD_ARG;
  cudaSetDevice(h->dev);
  const pf_params &p = h->p;
  double *d;
  const int64_t ns1 = nslices + 1;
  int rc = diag_scratch(h, (size_t)3 * ns1, &d);
  if (rc) return rc;
  PF_CUDA(cudaMemsetAsync(d, 0, sizeof(double) * 3 * ns1, h->stream));
  PF_CUDA(cudaMemsetAsync(h->d_status, 0, sizeof(unsigned int), h->stream));
  const double S = 4 * PF_PUFFIN_PI * p.rho;  // sliceSizeZ2
  if (h->np > 0) {
    k_bunching<<<(unsigned)((h->np + 255) / 256), 256, 0, h->stream>>>(
        h->y[h->cur][2], h->chi, h->np, harmonic, p.rho, S, (int)nslices,
        p.mesh_type == PF_MESH_PERIODIC, d, d + ns1, d + 2 * ns1, h->d_status);
    PF_LAUNCHED(h);
  }
  std::vector<double> hb((size_t)3 * ns1);
  PF_CUDA(cudaMemcpyAsync(hb.data(), d, sizeof(double) * 3 * ns1, cudaMemcpyDeviceToHost, h->stream));
  PF_CUDA(cudaMemcpyAsync(h->h_status, h->d_status, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                          h->stream));
  PF_CUDA(cudaStreamSynchronize(h->stream));
  if (*h->h_status) {
    h->err = "a macroparticle's z2 slice index is out of bounds (av_write.f90 slice computation)";
    return PF_OUT_OF_Z2;
  }
  for (int64_t s = 0; s < nslices; ++s) {
    const double r = hb[s], i = hb[ns1 + s], sd = hb[2 * ns1 + s];
    b[s] = (sd > 0.0) ? sqrt(r * r + i * i) / S : 0.0;
  }
  return PF_OK;
}

int pf_spectrum(pf_handle *h, double *sx, double *sy, int64_t nunique) {
  if (!h || !sx || !sy) return PF_BAD_ARG;
  const pf_params &p = h->p;
  const int64_t n = p.nz2;
  if (nunique != (n + 2) / 2) return PF_BAD_ARG;  // ceil((n+1)/2)
  cudaSetDevice(h->dev);
  int rc = pf_inner_to_outer(h);
  if (rc) return rc;
  double *d;
  rc = diag_scratch(h, (size_t)2 * nunique + 2 * (size_t)n, &d);
  if (rc) return rc;
  {
    std::vector<double> rt((size_t)2 * n);
    for (int64_t m = 0; m < n; ++m) {
      const double ang = 2.0 * M_PI * (double)m / (double)n;
      rt[2 * m] = cos(ang);
      rt[2 * m + 1] = -sin(ang);
    }
    PF_CUDA(cudaMemcpyAsync(d + 2 * nunique, rt.data(), rt.size() * sizeof(double),
                            cudaMemcpyHostToDevice, h->stream));
    PF_CUDA(cudaStreamSynchronize(h->stream));
  }
  const int64_t plane = (int64_t)p.nx * p.ny;
  const int64_t off = (int64_t)((p.nx - 1) / 2) + (int64_t)p.nx * ((p.ny - 1) / 2);
  const bool mixed = h->p.precision == PF_MIXED;
  k_spectrum<<<(unsigned)((nunique + 127) / 128), 128, 0, h->stream>>>(
      mixed ? nullptr : h->or_, mixed ? nullptr : h->oi_, mixed ? (const float2 *)h->oc32 : nullptr,
      plane, off, n, nunique, (const double2 *)(d + 2 * nunique), d, d + nunique);
  PF_LAUNCHED(h);
  PF_CUDA(cudaMemcpyAsync(sx, d, sizeof(double) * nunique, cudaMemcpyDeviceToHost, h->stream));
  PF_CUDA(cudaMemcpyAsync(sy, d + nunique, sizeof(double) * nunique, cudaMemcpyDeviceToHost,
                          h->stream));
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

}  // extern "C"
