// C ABI of puffgpu: handle life cycle, particle/field transfer, the inner
// transverse window, the periodic z2 wrap and the UndSection-style loop.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>

#include "pf_internal.h"

namespace {

typedef unsigned long long u64;

std::string g_err;

// Order-preserving map of doubles onto unsigned 64-bit integers.
__device__ __forceinline__ u64 ord_key(double v) {
  u64 b = (u64)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void k_minmax_xy(const double *x, const double *y, int64_t n, u64 *out) {
  // out[0] max x, out[1] min x (as keys), out[2] max y, out[3] min y
  u64 mx = 0, mnx = ~0ull, my = 0, mny = ~0ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    u64 kx = ord_key(x[i]), ky = ord_key(y[i]);
    mx = max(mx, kx);
    mnx = min(mnx, kx);
    my = max(my, ky);
    mny = min(mny, ky);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    mnx = min(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
    my = max(my, __shfl_xor_sync(0xffffffffu, my, o));
    mny = min(mny, __shfl_xor_sync(0xffffffffu, mny, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out + 0, mx);
    atomicMin(out + 1, mnx);
    atomicMax(out + 2, my);
    atomicMin(out + 3, mny);
  }
}

__global__ void k_absmax(const double *v, int64_t n, u64 *out) {
  u64 m = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    m = max(m, (u64)__double_as_longlong(fabs(v[i])));
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// outer2Inner / inner2Outer (para_field.f90:1352-1429): the window is
// centred, offset ((nx - nix)/2, (ny - niy)/2).
__global__ void k_window_copy(double *wr, double *wi, double *or_, double *oi, int nix, int niy,
                              int64_t npl, int nx, int ny, int64_t nz2, int to_outer,
                              int mirror) {
  const int64_t nw = (int64_t)nix * niy * npl;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nw) return;
  const int ix = (int)(t % nix);
  const int iy = (int)((t / nix) % niy);
  const int64_t iz = t / ((int64_t)nix * niy);
  const int ox = (nx - nix) / 2, oy = (ny - niy) / 2;
  const int64_t plane = (int64_t)nx * ny;
  const int64_t o = (ix + ox) + (int64_t)nx * (iy + oy) + plane * iz;
  if (to_outer) {
    or_[o] = wr[t];
    oi[o] = wi[t];
    if (mirror && iz == 0) {
      or_[o + plane * (nz2 - 1)] = wr[t];
      oi[o + plane * (nz2 - 1)] = wi[t];
    }
  } else {
    wr[t] = or_[o];
    wi[t] = oi[o];
  }
}

__global__ void k_window_copy_c32(float2 *w, float2 *o, int nix, int niy, int64_t npl, int nx,
                                  int ny, int64_t nz2, int to_outer, int mirror) {
  const int64_t nw = (int64_t)nix * niy * npl;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nw) return;
  const int ix = (int)(t % nix);
  const int iy = (int)((t / nix) % niy);
  const int64_t iz = t / ((int64_t)nix * niy);
  const int ox = (nx - nix) / 2, oy = (ny - niy) / 2;
  const int64_t plane = (int64_t)nx * ny;
  const int64_t oo = (ix + ox) + (int64_t)nx * (iy + oy) + plane * iz;
  if (to_outer) {
    o[oo] = w[t];
    if (mirror && iz == 0) o[oo + plane * (nz2 - 1)] = w[t];
  } else {
    w[t] = o[oo];
  }
}

// FP64 split field <-> interleaved complex float (mixed precision transfers)
__global__ void k_to_c32(float2 *o, const double *re, const double *im, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) o[t] = make_float2((float)re[t], (float)im[t]);
}

__global__ void k_to_f32(float *o, const double *v, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) o[t] = (float)v[t];
}

__global__ void k_from_c32(const float2 *o, double *re, double *im, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) {
    const float2 v = o[t];
    re[t] = (double)v.x;
    im[t] = (double)v.y;
  }
}

__global__ void k_mirror_plane_c32(float2 *o, int64_t plane, int64_t nz2) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < plane) o[plane * (nz2 - 1) + t] = o[t];
}

// Periodic wrap of z2 (para_field.f90:212-215)
__global__ void k_wrap_z2(double *z2, int64_t n, double lenz2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) z2[i] = z2[i] - (floor(z2[i] / lenz2) * lenz2);
}

__global__ void k_mirror_plane(double *re, double *im, int64_t plane, int64_t nz2) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < plane) {
    re[plane * (nz2 - 1) + t] = re[t];
    im[plane * (nz2 - 1) + t] = im[t];
  }
}

inline unsigned grid_for(int64_t n, int threads) {
  return (unsigned)std::max<int64_t>(1, (n + threads - 1) / threads);
}

}  // namespace

// ---------------------------------------------------------------------------
// per-kernel-class timing
void pf_prof_begin(pf_handle *h, int cls) {
  if (!h->prof) return;
  ProfEvent e;
  if (!h->prof_pool.empty()) {
    e = h->prof_pool.back();
    h->prof_pool.pop_back();
  } else {
    cudaEventCreate(&e.a);
    cudaEventCreate(&e.b);
  }
  e.cls = cls;
  cudaEventRecord(e.a, h->stream);
  h->prof_pending.push_back(e);
  h->prof_open = (int)h->prof_pending.size() - 1;
}

void pf_prof_end(pf_handle *h) {
  if (!h->prof || h->prof_open < 0) return;
  cudaEventRecord(h->prof_pending[h->prof_open].b, h->stream);
  h->prof_open = -1;
}

void pf_prof_flush(pf_handle *h) {
  if (h->prof_pending.empty()) return;
  for (ProfEvent &e : h->prof_pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(e.b) == cudaSuccess && cudaEventElapsedTime(&ms, e.a, e.b) == cudaSuccess) {
      h->prof_ms[e.cls] += ms;
      h->prof_n[e.cls] += 1;
    }
    h->prof_pool.push_back(e);
  }
  h->prof_pending.clear();
}

static void free_particles(pf_handle *h) {
  for (int b = 0; b < 2; ++b)
    for (int j = 0; j < 6; ++j) cudaFree(h->y[b][j]), h->y[b][j] = nullptr;
  for (int j = 0; j < 6; ++j) {
    cudaFree(h->k1[j]);
    cudaFree(h->ka[j]);
    cudaFree(h->kb[j]);
    h->k1[j] = h->ka[j] = h->kb[j] = nullptr;
  }
  cudaFree(h->chi);
  cudaFree(h->chi_f);
  cudaFree(h->base4);
  cudaFree(h->perm);
  h->chi = nullptr;
  h->chi_f = nullptr;
  h->base4 = nullptr;
  h->perm = nullptr;
  h->permuted = false;
  h->cap = 0;
}

static void free_window(pf_handle *h) {
  double **ptrs[] = {&h->wr, &h->wi, &h->asr, &h->asi, &h->d0r, &h->d0i, &h->d12r, &h->d12i};
  for (auto p : ptrs) {
    cudaFree(*p);
    *p = nullptr;
  }
  cudaFree(h->acc);
  h->acc = nullptr;
  void **c32[] = {&h->w32, &h->as32, &h->d0_32, &h->d12_32, &h->acc32};
  for (auto p : c32) {
    cudaFree(*p);
    *p = nullptr;
  }
  h->wcap = 0;
  h->nwin = 0;
  h->window_valid = false;
}

static int alloc_particles_raw(pf_handle *h, int64_t n) {
  const size_t b = sizeof(double) * (size_t)std::max<int64_t>(n, 1);
  for (int bb = 0; bb < 2; ++bb)
    for (int j = 0; j < 6; ++j) PF_CUDA(cudaMalloc(&h->y[bb][j], b));
  for (int j = 0; j < 6; ++j) {
    PF_CUDA(cudaMalloc(&h->k1[j], b));
    PF_CUDA(cudaMalloc(&h->ka[j], b));
    PF_CUDA(cudaMalloc(&h->kb[j], b));
  }
  PF_CUDA(cudaMalloc(&h->chi, b));
  if (h->p.precision == PF_MIXED) {
    PF_CUDA(cudaMalloc(&h->chi_f, sizeof(float) * (size_t)std::max<int64_t>(n, 1)));
    PF_CUDA(cudaMalloc(&h->base4, sizeof(float4) * (size_t)std::max<int64_t>(n, 1)));
  }
  return PF_OK;
}

// On an allocation failure the handle is left without particles (PF_STATE
// until the next successful pf_set_particles) and stays destroyable.
static int alloc_particles(pf_handle *h, int64_t n) {
  if (n <= h->cap) return PF_OK;
  free_particles(h);
  h->np = 0;
  h->particles_set = false;
  const int rc = alloc_particles_raw(h, n);
  if (rc) {
    free_particles(h);
    return rc;
  }
  h->cap = n;
  return PF_OK;
}

static int alloc_window_raw(pf_handle *h, int64_t nw) {
  const size_t b = sizeof(double) * (size_t)nw;
  if (h->p.precision == PF_MIXED) {
    void **c32[] = {&h->w32, &h->as32, &h->d0_32, &h->d12_32, &h->acc32};
    for (auto p : c32) PF_CUDA(cudaMalloc(p, b));  // float2 per node
    PF_CUDA(cudaMemsetAsync(h->acc32, 0, b, h->stream));
  } else {
    double **ptrs[] = {&h->wr, &h->wi, &h->asr, &h->asi, &h->d0r, &h->d0i, &h->d12r, &h->d12i};
    for (auto p : ptrs) PF_CUDA(cudaMalloc(p, b));
    PF_CUDA(cudaMalloc(&h->acc, 4 * b));
    PF_CUDA(cudaMemsetAsync(h->acc, 0, 4 * b, h->stream));
  }
  return PF_OK;
}

// On an allocation failure the handle is left without a window (PF_STATE
// until the particles are set again) and stays destroyable.
static int alloc_window(pf_handle *h, int nix, int niy) {
  const int64_t nw = (int64_t)nix * niy * h->npl;
  if (nw > h->wcap) {
    free_window(h);
    const int rc = alloc_window_raw(h, nw);
    if (rc) {
      free_window(h);
      return rc;
    }
    h->wcap = nw;
  }
  h->nix = nix;
  h->niy = niy;
  h->nwin = nw;
  return PF_OK;
}

int pf_outer_to_inner(pf_handle *h) {
  if (h->nwin == 0) return PF_OK;
  if (h->p.precision == PF_MIXED) {
    k_window_copy_c32<<<grid_for(h->nwin, 256), 256, 0, h->stream>>>(
        (float2 *)h->w32, (float2 *)h->oc32, h->nix, h->niy, h->npl, h->p.nx, h->p.ny, h->p.nz2,
        0, 0);
    PF_LAUNCHED(h);
    h->window_valid = true;
    return PF_OK;
  }
  k_window_copy<<<grid_for(h->nwin, 256), 256, 0, h->stream>>>(
      h->wr, h->wi, h->or_, h->oi_, h->nix, h->niy, h->npl, h->p.nx, h->p.ny, h->p.nz2, 0, 0);
  PF_LAUNCHED(h);
  h->window_valid = true;
  return PF_OK;
}

int pf_inner_to_outer(pf_handle *h) {
  if (h->nwin == 0 || !h->window_valid) return PF_OK;
  const int mirror = (h->p.mesh_type == PF_MESH_PERIODIC);
  if (h->p.precision == PF_MIXED) {
    k_window_copy_c32<<<grid_for(h->nwin, 256), 256, 0, h->stream>>>(
        (float2 *)h->w32, (float2 *)h->oc32, h->nix, h->niy, h->npl, h->p.nx, h->p.ny, h->p.nz2,
        1, mirror);
    PF_LAUNCHED(h);
    return PF_OK;
  }
  k_window_copy<<<grid_for(h->nwin, 256), 256, 0, h->stream>>>(
      h->wr, h->wi, h->or_, h->oi_, h->nix, h->niy, h->npl, h->p.nx, h->p.ny, h->p.nz2, 1,
      mirror);
  PF_LAUNCHED(h);
  return PF_OK;
}

// getInNode (para_field.f90:1432-1508)
int pf_window_from_particles(pf_handle *h, int *nix, int *niy) {
  const pf_params &p = h->p;
  if (p.nx * p.ny == 1) {
    *nix = 1;
    *niy = 1;
    return PF_OK;
  }
  int ix, iy;
  if (h->np > 0) {
    u64 init[4] = {0ull, ~0ull, 0ull, ~0ull};
    u64 *d = (u64 *)h->d_red;
    PF_CUDA(cudaMemcpyAsync(d, init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    k_minmax_xy<<<std::min<unsigned>(grid_for(h->np, 256), 4096), 256, 0, h->stream>>>(
        h->y[h->cur][0], h->y[h->cur][1], h->np, d);
    PF_LAUNCHED(h);
    u64 r[4];
    PF_CUDA(cudaMemcpyAsync(r, d, sizeof(r), cudaMemcpyDeviceToHost, h->stream));
    PF_CUDA(cudaStreamSynchronize(h->stream));
    auto unkey = [](u64 k) {
      u64 b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
      double v;
      memcpy(&v, &b, sizeof(v));
      return v;
    };
    double smaxx = fabs(unkey(r[0])), sminx = fabs(unkey(r[1]));
    double smaxy = fabs(unkey(r[2])), sminy = fabs(unkey(r[3]));
    if (!(std::isfinite(smaxx) && std::isfinite(sminx) && std::isfinite(smaxy) &&
          std::isfinite(sminy))) {
      h->err = "a macroparticle's transverse position is not finite";
      return PF_NOT_FINITE;
    }
    if (!(std::max(smaxx, sminx) / p.dx < 1.0e9 && std::max(smaxy, sminy) / p.dy < 1.0e9)) {
      h->err = "transverse grid not large enough for the inner window";
      return PF_OUT_OF_WINDOW;
    }
    long imaxx = (long)ceil(smaxx / p.dx), iminx = (long)floor(sminx / p.dx);
    long imaxy = (long)ceil(smaxy / p.dy), iminy = (long)floor(sminy / p.dy);
    ix = (int)((std::max(imaxx, iminx) + 3) * 2);
    iy = (int)((std::max(imaxy, iminy) + 3) * 2);
  } else {
    ix = iy = 2;
  }
  if ((p.nx % 2) != (ix % 2)) ix += 1;
  if ((p.ny % 2) != (iy % 2)) iy += 1;
  if (ix > p.nx || iy > p.ny) {
    h->err = "transverse grid not large enough for the inner window (nspinDX=" +
             std::to_string(ix) + ", nspinDY=" + std::to_string(iy) + ")";
    return PF_OUT_OF_WINDOW;
  }
  *nix = ix;
  *niy = iy;
  return PF_OK;
}

static int set_window(pf_handle *h, int nix, int niy) {
  int rc = pf_inner_to_outer(h);
  if (rc) return rc;
  h->window_valid = false;
  rc = alloc_window(h, nix, niy);
  if (rc) return rc;
  return pf_outer_to_inner(h);
}

// grow_only: keep the current window while it is at least as large as the
// one the particles need
static int choose_window(pf_handle *h, bool grow_only) {
  int nix = h->p.nix, niy = h->p.niy;
  if (nix <= 0 || niy <= 0) {
    int rc = pf_window_from_particles(h, &nix, &niy);
    if (rc) return rc;
  }
  if (nix > h->p.nx || niy > h->p.ny || nix < 1 || niy < 1) {
    h->err = "inner window larger than the mesh";
    return PF_BAD_ARG;
  }
  if (grow_only && h->nwin > 0 && nix <= h->nix && niy <= h->niy) return PF_OK;
  return set_window(h, nix, niy);
}

static int status_to_rc(unsigned int st) { return pf_status_of(st); }

// ---------------------------------------------------------------------------
extern "C" {

int pf_abi_version(void) { return PUFFGPU_ABI_VERSION; }

void pf_default_params(pf_params *p) {
  memset(p, 0, sizeof(*p));
  p->rho = 0.01;
  p->aw = 1.0;
  p->gamma_r = 100.0;
  p->fx = 1.0;
  p->fy = 1.0;
  p->szfe = 1.0e30;
  p->n2col0 = 1.0;
  p->dx = p->dy = p->dz2 = 1.0;
  p->sbeta = 1.0;
  p->sfilt_frac = (double)0.3f;
  p->sperwaves = -1.0;
  p->und_type = PF_UND_PUFFIN;
  p->mesh_type = PF_MESH_TEMPORAL;
  p->nx = p->ny = 1;
  p->nz2 = 2;
  p->nbx = p->nby = 16;
  p->nbz2 = 37;
  p->field_evolve = p->electrons_evolve = p->coupling = 1;
  p->qfilter = 1;
  p->redist_every = 60;
  p->precision = PF_FP64;
}

const char *pf_last_error(const pf_handle *h) { return h ? h->err.c_str() : g_err.c_str(); }

int pf_create(const pf_params *p, pf_handle **out) {
  if (!p || !out) return PF_BAD_ARG;
  *out = nullptr;
  if (p->nx < 1 || p->ny < 1 || p->nz2 < 2 || p->dz2 <= 0.0 || p->dx <= 0.0 || p->dy <= 0.0 ||
      p->rho <= 0.0 || p->eta <= 0.0 || p->gamma_r <= 0.0) {
    g_err = "pf_create: invalid mesh or physics constants";
    return PF_BAD_ARG;
  }
  if (p->one_d && (p->nx != 1 || p->ny != 1)) {
    g_err = "pf_create: one_d requires nx = ny = 1";
    return PF_BAD_ARG;
  }
  if (p->precision != PF_FP64 && p->precision != PF_MIXED) {
    g_err = "pf_create: precision must be PF_FP64 or PF_MIXED";
    return PF_BAD_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    g_err = "pf_create: no CUDA device";
    return PF_NO_DEVICE;
  }
  if (p->device < 0 || p->device >= ndev) {
    g_err = "pf_create: bad device ordinal";
    return PF_BAD_ARG;
  }
  pf_handle *h = new pf_handle();
  h->p = *p;
  h->dev = p->device;
  h->n2col = p->n2col0;
  h->n2col0 = p->n2col0;
  h->undgrad = p->undgrad;
  h->npl = (p->mesh_type == PF_MESH_PERIODIC) ? p->nz2 - 1 : p->nz2;
  h->fft_pairs = (p->precision == PF_FP64);  // pf_set_fft_arithmetic: paired FP32 by default
  h->nouter = (int64_t)p->nx * p->ny * p->nz2;
  auto fail = [&](cudaError_t e, const char *what) {
    (void)cudaGetLastError();  // an allocation failure leaves the context usable
    g_err = std::string("pf_create: ") + what + ": " + cudaGetErrorString(e);
    pf_destroy(h);
    return PF_CUDA_ERR;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(h->dev)) != cudaSuccess) return fail(e, "cudaSetDevice");
  if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return fail(e, "stream");
  h->own_stream = true;
  if ((e = cudaMalloc(&h->d_status, 64)) != cudaSuccess) return fail(e, "status");
  if ((e = cudaMalloc(&h->d_red, 64)) != cudaSuccess) return fail(e, "reduction scratch");
  if ((e = cudaMallocHost(&h->h_status, 64)) != cudaSuccess) return fail(e, "pinned status");
  if (p->precision == PF_MIXED) {
    if ((e = cudaMalloc(&h->oc32, sizeof(float2) * h->nouter)) != cudaSuccess) return fail(e, "field");
    cudaMemsetAsync(h->oc32, 0, sizeof(float2) * h->nouter, h->stream);
  } else {
    if ((e = cudaMalloc(&h->or_, sizeof(double) * h->nouter)) != cudaSuccess) return fail(e, "field");
    if ((e = cudaMalloc(&h->oi_, sizeof(double) * h->nouter)) != cudaSuccess) return fail(e, "field");
    cudaMemsetAsync(h->or_, 0, sizeof(double) * h->nouter, h->stream);
    cudaMemsetAsync(h->oi_, 0, sizeof(double) * h->nouter, h->stream);
  }
  cudaMemsetAsync(h->d_status, 0, 64, h->stream);
  if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return fail(e, "sync");
  *out = h;
  return PF_OK;
}

int pf_destroy(pf_handle *h) {
  if (!h) return PF_OK;
  cudaSetDevice(h->dev);
  if (h->stream) cudaStreamSynchronize(h->stream);
  pf_prof_flush(h);
  for (ProfEvent &e : h->prof_pool) {
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
  for (cudaEvent_t e : h->copy_events) cudaEventDestroy(e);
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  free_particles(h);
  free_window(h);
  pf_diff_destroy(h->diff);
  cudaFree(h->or_);
  cudaFree(h->oi_);
  cudaFree(h->oc32);
  cudaFree(h->staging);
  cudaFree(h->wstage);
  cudaFree(h->diag);
  cudaFree(h->lat_scratch);
  cudaFree(h->snap);
  cudaFree(h->plane_off);
  pf_adj_destroy(h->adj);
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  cudaFree(h->coef_dev);
  if (h->coef_host) cudaFreeHost(h->coef_host);
  cudaFree(h->step_ctr);
  cudaFree(h->d_status);
  cudaFree(h->d_red);
  if (h->h_status) cudaFreeHost(h->h_status);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return PF_OK;
}

__global__ void k_unpermute(const double *src, const int32_t *perm, double *dst, int64_t n);

// chi (and its FP32 copy) of a z2-ordered handle back in the caller's
// order, for new particle arrays in that order that keep chi
static int unpermute_chi(pf_handle *h) {
  const int64_t n = h->np;
  k_unpermute<<<grid_for(n, 256), 256, 0, h->stream>>>(h->chi, h->perm, h->kb[0], n);
  PF_LAUNCHED(h);
  PF_CUDA(cudaMemcpyAsync(h->chi, h->kb[0], sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice,
                          h->stream));
  if (h->chi_f) {
    k_to_f32<<<grid_for(n, 256), 256, 0, h->stream>>>(h->chi_f, h->chi, n);
    PF_LAUNCHED(h);
  }
  return PF_OK;
}

static int set_particles_impl(pf_handle *h, int64_t n, const double *const src[7],
                              cudaMemcpyKind kind) {
  if (!h || n < 0) return PF_BAD_ARG;
  for (int j = 0; j < 6; ++j)
    if (n > 0 && !src[j]) return PF_BAD_ARG;
  // chi == NULL keeps the handle's chi (and its fixed-point scale): only for
  // the same macroparticles, as a driver that hands the state in every step
  // passes them (rk4par never changes chi)
  const bool keep_chi = (src[6] == nullptr);
  if (n > 0 && keep_chi && !(h->particles_set && n == h->np)) {
    h->err = "pf_set_particles: chi may be NULL only to keep the current macroparticles' chi";
    return PF_BAD_ARG;
  }
  cudaSetDevice(h->dev);
  int rc = alloc_particles(h, n);
  if (rc) return rc;
  if (h->permuted && src[6] == nullptr && n > 0 && n == h->np) {
    rc = unpermute_chi(h);  // the kept chi goes back to the caller's order
    if (rc) return rc;
  }
  h->permuted = false;
  h->np = n;
  h->particles_set = true;
  const size_t b = sizeof(double) * (size_t)n;
  if (n > 0) {
    for (int j = 0; j < 6; ++j)
      PF_CUDA(cudaMemcpyAsync(h->y[h->cur][j], src[j], b, kind, h->stream));
    if (!keep_chi) {
      PF_CUDA(cudaMemcpyAsync(h->chi, src[6], b, kind, h->stream));
      if (h->chi_f) {
        k_to_f32<<<grid_for(n, 256), 256, 0, h->stream>>>(h->chi_f, h->chi, n);
        PF_LAUNCHED(h);
      }
    }
  }
  if (keep_chi && n > 0) return choose_window(h, true);
  // fixed-point scale of the deposit from max |chi| / dV3
  double chimax = 0.0;
  if (n > 0) {
    u64 *d = (u64 *)h->d_red;
    PF_CUDA(cudaMemsetAsync(d, 0, sizeof(u64), h->stream));
    k_absmax<<<std::min<unsigned>(grid_for(n, 256), 4096), 256, 0, h->stream>>>(h->chi, n, d);
    PF_LAUNCHED(h);
    u64 r;
    PF_CUDA(cudaMemcpyAsync(&r, d, sizeof(r), cudaMemcpyDeviceToHost, h->stream));
    PF_CUDA(cudaStreamSynchronize(h->stream));
    memcpy(&chimax, &r, sizeof(r));
  }
  h->chi_max = chimax;
  int lg = 0;
  while ((int64_t(1) << lg) < 2 * n + 2) ++lg;
  h->fix_maxexp = 126 - lg;
  const double smax = chimax / (h->p.dx * h->p.dy * h->p.dz2);
  const int e_s = (smax > 0.0 && isfinite(smax)) ? ilogb(smax) + 1 : 0;
  h->fix_e = h->fix_maxexp - 16 - e_s;
  // getInNode for the first particles; afterwards the window only grows here
  // (the reference recomputes it at redistribution, pf_redistribute), so a
  // driver that hands the state in every step keeps one window
  return choose_window(h, true);
}

int pf_set_particles(pf_handle *h, int64_t n, const double *x, const double *y,
                     const double *z2, const double *px, const double *py,
                     const double *gam, const double *chi) {
  const double *s[7] = {x, y, z2, px, py, gam, chi};
  return set_particles_impl(h, n, s, cudaMemcpyHostToDevice);
}

int pf_set_particles_dev(pf_handle *h, int64_t n, const double *x, const double *y,
                         const double *z2, const double *px, const double *py,
                         const double *gam, const double *chi) {
  const double *s[7] = {x, y, z2, px, py, gam, chi};
  return set_particles_impl(h, n, s, cudaMemcpyDeviceToDevice);
}

// ---------------------------------------------------------------------------
// z2 ordering: a counting sort of the macroparticles over the z2 planes (the
// FEL bunching spreads runs of consecutive macroparticles over many planes,
// which defeats the stage kernels' block tiles); the caller's order is kept
// in perm and restored by pf_get_particles.
__device__ __forceinline__ int sort_plane(double z2, double inv_dz2, int npl, int periodic) {
  const double f = floor(z2 * inv_dz2);
  int p = (fabs(f) < 2.0e9) ? (int)f : 0;
  if (periodic) {
    p %= npl;
    if (p < 0) p += npl;
  }
  return min(max(p, 0), npl - 1);
}

__global__ void k_iota32(int32_t *p, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) p[t] = (int32_t)t;
}

// Stable counting sort over the z2 planes.  The macroparticles are cut into
// chunks of consecutive slots, one warp per chunk: (1) each chunk counts its
// planes; (2) an exclusive scan of the counts in (plane, chunk) order gives
// every chunk the first slot of each plane it holds; (3) each chunk writes its
// macroparticles in order, a warp-wide rank among equal planes per round of
// 32.  Slots keep their relative order within a plane, so the result depends
// only on the input order: the same every run.
constexpr int SORT_SCAN_TILE = 4096;  // ints per block of the scan

__global__ void __launch_bounds__(32) k_chunk_count(const double *z2, int64_t n, int64_t chunk,
                                                    double inv_dz2, int npl, int periodic,
                                                    int *tab, int64_t nchunks) {
  extern __shared__ int hist[];
  const int64_t c = blockIdx.x;
  for (int k = threadIdx.x; k < npl; k += 32) hist[k] = 0;
  __syncwarp();
  const int64_t i0 = c * chunk, i1 = min(n, i0 + chunk);
  for (int64_t i = i0 + threadIdx.x; i < i1; i += 32)
    atomicAdd(hist + sort_plane(z2[i], inv_dz2, npl, periodic), 1);
  __syncwarp();
  for (int k = threadIdx.x; k < npl; k += 32) tab[(int64_t)k * nchunks + c] = hist[k];
}

// exclusive scan of 4096-int tiles in place; tile totals to sums[blockIdx.x]
__global__ void __launch_bounds__(256) k_scan_tiles(int *v, int64_t n, int *sums) {
  __shared__ int warp_tot[8];
  const int64_t base = (int64_t)blockIdx.x * SORT_SCAN_TILE + (int64_t)threadIdx.x * 16;
  int x[16];
  int run = 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    x[k] = (base + k < n) ? v[base + k] : 0;
    run += x[k];
  }
  // exclusive scan of the per-thread totals across the block
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = run;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_tot[w] = inc;
  __syncthreads();
  int woff = 0, tot = 0;
  for (int k = 0; k < 8; ++k) {
    if (k < w) woff += warp_tot[k];
    tot += warp_tot[k];
  }
  int acc = woff + inc - run;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    if (base + k < n) v[base + k] = acc;
    acc += x[k];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// exclusive scan of the tile totals (one block, in order)
__global__ void __launch_bounds__(1024) k_scan_sums(int *sums, int m) {
  __shared__ int carry;
  __shared__ int warp_tot[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int b = 0; b < m; b += 1024) {
    const int i = b + threadIdx.x;
    const int x = (i < m) ? sums[i] : 0;
    int inc = x;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    int woff = 0, tot = 0;
    for (int k = 0; k < 32; ++k) {
      if (k < w) woff += warp_tot[k];
      tot += warp_tot[k];
    }
    if (i < m) sums[i] = carry + woff + inc - x;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) k_scan_add(int *v, int64_t n, const int *sums) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] += sums[i / SORT_SCAN_TILE];
}

struct SortArrays {
  const double *src[7];
  double *dst[7];
  const int32_t *perm_src;
  int32_t *perm_dst;
};

__global__ void __launch_bounds__(32) k_chunk_scatter(const SortArrays a, int64_t n, int64_t chunk,
                                                      double inv_dz2, int npl, int periodic,
                                                      const int *tab, int64_t nchunks) {
  extern __shared__ int run[];
  const int64_t c = blockIdx.x;
  for (int k = threadIdx.x; k < npl; k += 32) run[k] = tab[(int64_t)k * nchunks + c];
  __syncwarp();
  const int lane = threadIdx.x;
  const unsigned lt = (1u << lane) - 1u;
  const int64_t i0 = c * chunk, i1 = min(n, i0 + chunk);
  for (int64_t r = i0; r < i1; r += 32) {
    const int64_t t = r + lane;
    const bool on = t < i1;
    const unsigned act = __ballot_sync(0xffffffffu, on);
    int pos = 0, p = 0;
    unsigned peers = 0;
    if (on) {
      p = sort_plane(a.src[2][t], inv_dz2, npl, periodic);
      peers = __match_any_sync(act, p);
      pos = run[p] + __popc(peers & lt);
    }
    __syncwarp();
    if (on && lane == 31 - __clz(peers)) run[p] += __popc(peers);  // the group's last lane
    __syncwarp();
    if (on) {
#pragma unroll
      for (int j = 0; j < 7; ++j) a.dst[j][pos] = a.src[j][t];
      a.perm_dst[pos] = a.perm_src[t];
    }
  }
}

__global__ void k_unpermute(const double *src, const int32_t *perm, double *dst, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) dst[perm[t]] = src[t];
}

// Between steps only: the slope arrays (k1, ka) and the other state buffer
// are free then and hold the sorted copy, which is copied back in place (the
// arrays keep their addresses, so captured step blocks stay valid).
int pf_sort_z2(pf_handle *h) {
  if (!h->sort_z2 || h->np < ((int64_t)1 << 15) || h->p.one_d || h->npl < 2) return PF_OK;
  if (h->np >= ((int64_t)1 << 31)) return PF_OK;
  const int npl = (int)h->npl;
  if ((size_t)npl * sizeof(int) > (size_t)200 * 1024) return PF_OK;  // plane table per warp
  const int periodic = (h->p.mesh_type == PF_MESH_PERIODIC);
  const double inv_dz2 = 1.0 / h->p.dz2;
  const int64_t n = h->np;
  // chunks of at least 1024 slots, about 4096 of them, the count table
  // (npl x chunks ints) at most 64 MB
  int64_t chunk = std::max<int64_t>(1024, (n + 4095) / 4096);
  while ((n + chunk - 1) / chunk * (int64_t)npl > ((int64_t)16 << 20)) chunk *= 2;
  const int64_t nchunks = (n + chunk - 1) / chunk;
  const int64_t ntab = nchunks * npl;
  const int64_t ntiles = (ntab + SORT_SCAN_TILE - 1) / SORT_SCAN_TILE;
  const size_t need = (size_t)(ntab + ntiles);
  if (!h->perm) PF_CUDA(cudaMalloc(&h->perm, sizeof(int32_t) * (size_t)h->cap));
  if (h->plane_cap < (int64_t)need) {
    cudaFree(h->plane_off);
    h->plane_off = nullptr;
    PF_CUDA(cudaMalloc(&h->plane_off, sizeof(int) * need));
    h->plane_cap = (int64_t)need;
  }
  if (!h->permuted) {
    k_iota32<<<grid_for(n, 256), 256, 0, h->stream>>>(h->perm, n);
    PF_LAUNCHED(h);
  }
  const size_t smem = sizeof(int) * (size_t)npl;
  static PfDeviceOnce attr_once;  // the attribute is per device
  PF_CUDA(pf_device_once(attr_once, [] {
    cudaError_t e = cudaFuncSetAttribute(k_chunk_count, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         200 * 1024);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_chunk_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               200 * 1024);
    return e;
  }));
  int *tab = h->plane_off, *sums = h->plane_off + ntab;
  k_chunk_count<<<(unsigned)nchunks, 32, smem, h->stream>>>(h->y[h->cur][2], n, chunk, inv_dz2,
                                                            npl, periodic, tab, nchunks);
  PF_LAUNCHED(h);
  k_scan_tiles<<<(unsigned)ntiles, 256, 0, h->stream>>>(tab, ntab, sums);
  PF_LAUNCHED(h);
  k_scan_sums<<<1, 1024, 0, h->stream>>>(sums, (int)ntiles);
  PF_LAUNCHED(h);
  k_scan_add<<<grid_for(ntab, 256), 256, 0, h->stream>>>(tab, ntab, sums);
  PF_LAUNCHED(h);
  SortArrays a;
  const int nxt = 1 - h->cur;
  for (int j = 0; j < 6; ++j) {
    a.src[j] = h->y[h->cur][j];
    a.dst[j] = h->y[nxt][j];
  }
  a.src[6] = h->chi;
  a.dst[6] = h->k1[0];
  a.perm_src = h->perm;
  a.perm_dst = reinterpret_cast<int32_t *>(h->ka[0]);
  k_chunk_scatter<<<(unsigned)nchunks, 32, smem, h->stream>>>(a, n, chunk, inv_dz2, npl, periodic,
                                                              tab, nchunks);
  PF_LAUNCHED(h);
  const size_t b = sizeof(double) * (size_t)n;
  for (int j = 0; j < 6; ++j)
    PF_CUDA(cudaMemcpyAsync(h->y[h->cur][j], h->y[nxt][j], b, cudaMemcpyDeviceToDevice, h->stream));
  PF_CUDA(cudaMemcpyAsync(h->chi, h->k1[0], b, cudaMemcpyDeviceToDevice, h->stream));
  PF_CUDA(cudaMemcpyAsync(h->perm, h->ka[0], sizeof(int32_t) * (size_t)n,
                          cudaMemcpyDeviceToDevice, h->stream));
  if (h->chi_f) {
    k_to_f32<<<grid_for(n, 256), 256, 0, h->stream>>>(h->chi_f, h->chi, n);
    PF_LAUNCHED(h);
  }
  h->permuted = true;
  return PF_OK;
}

static int get_particles_impl(pf_handle *h, double *const dst[7], cudaMemcpyKind kind) {
  if (!h) return PF_BAD_ARG;
  cudaSetDevice(h->dev);
  const size_t b = sizeof(double) * (size_t)h->np;
  if (h->np > 0) {
    for (int j = 0; j < 7; ++j) {
      if (!dst[j]) continue;
      const double *src = (j < 6) ? h->y[h->cur][j] : h->chi;
      if (h->permuted) {  // back to the caller's order through a free slope array
        k_unpermute<<<grid_for(h->np, 256), 256, 0, h->stream>>>(src, h->perm, h->kb[0], h->np);
        PF_LAUNCHED(h);
        src = h->kb[0];
      }
      PF_CUDA(cudaMemcpyAsync(dst[j], src, b, kind, h->stream));
    }
  }
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

int pf_get_particles(pf_handle *h, double *x, double *y, double *z2, double *px, double *py,
                     double *gam, double *chi) {
  double *d[7] = {x, y, z2, px, py, gam, chi};
  return get_particles_impl(h, d, cudaMemcpyDeviceToHost);
}

int pf_get_particles_dev(pf_handle *h, double *x, double *y, double *z2, double *px, double *py,
                         double *gam, double *chi) {
  double *d[7] = {x, y, z2, px, py, gam, chi};
  return get_particles_impl(h, d, cudaMemcpyDeviceToDevice);
}

int64_t pf_num_particles(const pf_handle *h) { return h ? h->np : -1; }

static int set_field_impl(pf_handle *h, const double *re, const double *im, cudaMemcpyKind kind) {
  if (!h || !re || !im) return PF_BAD_ARG;
  cudaSetDevice(h->dev);
  const size_t b = sizeof(double) * (size_t)h->nouter;
  const int64_t plane = (int64_t)h->p.nx * h->p.ny;
  if (h->p.precision == PF_MIXED) {
    if (!h->staging) PF_CUDA(cudaMalloc(&h->staging, 2 * b));
    PF_CUDA(cudaMemcpyAsync(h->staging, re, b, kind, h->stream));
    PF_CUDA(cudaMemcpyAsync(h->staging + h->nouter, im, b, kind, h->stream));
    k_to_c32<<<grid_for(h->nouter, 256), 256, 0, h->stream>>>((float2 *)h->oc32, h->staging,
                                                             h->staging + h->nouter, h->nouter);
    PF_LAUNCHED(h);
    if (h->p.mesh_type == PF_MESH_PERIODIC) {
      k_mirror_plane_c32<<<grid_for(plane, 256), 256, 0, h->stream>>>((float2 *)h->oc32, plane,
                                                                     h->p.nz2);
      PF_LAUNCHED(h);
    }
  } else {
    PF_CUDA(cudaMemcpyAsync(h->or_, re, b, kind, h->stream));
    PF_CUDA(cudaMemcpyAsync(h->oi_, im, b, kind, h->stream));
    if (h->p.mesh_type == PF_MESH_PERIODIC) {  // pupd8: the head plane wins
      k_mirror_plane<<<grid_for(plane, 256), 256, 0, h->stream>>>(h->or_, h->oi_, plane, h->p.nz2);
      PF_LAUNCHED(h);
    }
  }
  if (h->nwin > 0) {
    int rc = pf_outer_to_inner(h);
    if (rc) return rc;
  }
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

int pf_set_field(pf_handle *h, const double *re, const double *im) {
  return set_field_impl(h, re, im, cudaMemcpyHostToDevice);
}
int pf_set_field_dev(pf_handle *h, const double *re, const double *im) {
  return set_field_impl(h, re, im, cudaMemcpyDeviceToDevice);
}

static int get_field_impl(pf_handle *h, double *re, double *im, cudaMemcpyKind kind) {
  if (!h || !re || !im) return PF_BAD_ARG;
  cudaSetDevice(h->dev);
  int rc = pf_inner_to_outer(h);
  if (rc) return rc;
  const size_t b = sizeof(double) * (size_t)h->nouter;
  if (h->p.precision == PF_MIXED) {
    if (!h->staging) PF_CUDA(cudaMalloc(&h->staging, 2 * b));
    k_from_c32<<<grid_for(h->nouter, 256), 256, 0, h->stream>>>(
        (const float2 *)h->oc32, h->staging, h->staging + h->nouter, h->nouter);
    PF_LAUNCHED(h);
    PF_CUDA(cudaMemcpyAsync(re, h->staging, b, kind, h->stream));
    PF_CUDA(cudaMemcpyAsync(im, h->staging + h->nouter, b, kind, h->stream));
  } else {
    PF_CUDA(cudaMemcpyAsync(re, h->or_, b, kind, h->stream));
    PF_CUDA(cudaMemcpyAsync(im, h->oi_, b, kind, h->stream));
  }
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

int pf_get_field(pf_handle *h, double *re, double *im) {
  return get_field_impl(h, re, im, cudaMemcpyDeviceToHost);
}
int pf_get_field_dev(pf_handle *h, double *re, double *im) {
  return get_field_impl(h, re, im, cudaMemcpyDeviceToDevice);
}

// the inner-window field (ac_rfield_in / ac_ifield_in) in outer2Inner's layout
static int set_window_field_impl(pf_handle *h, const double *re, const double *im,
                                 cudaMemcpyKind kind) {
  if (!h || !re || !im) return PF_BAD_ARG;
  if (h->nwin == 0) {
    h->err = "pf_set_window_field: no inner window (particles not set)";
    return PF_STATE;
  }
  cudaSetDevice(h->dev);
  const size_t b = sizeof(double) * (size_t)h->nwin;
  if (h->p.precision == PF_MIXED) {
    if (!h->staging) PF_CUDA(cudaMalloc(&h->staging, 2 * sizeof(double) * (size_t)h->nouter));
    PF_CUDA(cudaMemcpyAsync(h->staging, re, b, kind, h->stream));
    PF_CUDA(cudaMemcpyAsync(h->staging + h->nwin, im, b, kind, h->stream));
    k_to_c32<<<grid_for(h->nwin, 256), 256, 0, h->stream>>>((float2 *)h->w32, h->staging,
                                                           h->staging + h->nwin, h->nwin);
    PF_LAUNCHED(h);
  } else {
    PF_CUDA(cudaMemcpyAsync(h->wr, re, b, kind, h->stream));
    PF_CUDA(cudaMemcpyAsync(h->wi, im, b, kind, h->stream));
  }
  h->window_valid = true;
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

static int get_window_field_impl(pf_handle *h, double *re, double *im, cudaMemcpyKind kind) {
  if (!h || !re || !im) return PF_BAD_ARG;
  if (h->nwin == 0) {
    h->err = "pf_get_window_field: no inner window (particles not set)";
    return PF_STATE;
  }
  cudaSetDevice(h->dev);
  const size_t b = sizeof(double) * (size_t)h->nwin;
  if (h->p.precision == PF_MIXED) {
    if (!h->staging) PF_CUDA(cudaMalloc(&h->staging, 2 * sizeof(double) * (size_t)h->nouter));
    k_from_c32<<<grid_for(h->nwin, 256), 256, 0, h->stream>>>(
        (const float2 *)h->w32, h->staging, h->staging + h->nwin, h->nwin);
    PF_LAUNCHED(h);
    PF_CUDA(cudaMemcpyAsync(re, h->staging, b, kind, h->stream));
    PF_CUDA(cudaMemcpyAsync(im, h->staging + h->nwin, b, kind, h->stream));
  } else {
    PF_CUDA(cudaMemcpyAsync(re, h->wr, b, kind, h->stream));
    PF_CUDA(cudaMemcpyAsync(im, h->wi, b, kind, h->stream));
  }
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

int pf_set_window_field(pf_handle *h, const double *re, const double *im) {
  return set_window_field_impl(h, re, im, cudaMemcpyHostToDevice);
}
int pf_get_window_field(pf_handle *h, double *re, double *im) {
  return get_window_field_impl(h, re, im, cudaMemcpyDeviceToHost);
}
int pf_set_window_field_dev(pf_handle *h, const double *re, const double *im) {
  return set_window_field_impl(h, re, im, cudaMemcpyDeviceToDevice);
}
int pf_get_window_field_dev(pf_handle *h, double *re, double *im) {
  return get_window_field_impl(h, re, im, cudaMemcpyDeviceToDevice);
}

int64_t pf_window_nodes(const pf_handle *h) { return h ? h->nwin : -1; }

int pf_set_taper(pf_handle *h, double n2col, double n2col0, double undgrad) {
  if (!h) return PF_BAD_ARG;
  h->n2col = n2col;
  h->n2col0 = n2col0;
  h->undgrad = undgrad;
  return PF_OK;
}

int pf_get_taper(const pf_handle *h, double *n2col, double *n2col0, double *undgrad) {
  if (!h) return PF_BAD_ARG;
  if (n2col) *n2col = h->n2col;
  if (n2col0) *n2col0 = h->n2col0;
  if (undgrad) *undgrad = h->undgrad;
  return PF_OK;
}

int pf_get_window(const pf_handle *h, int32_t *nix, int32_t *niy) {
  if (!h) return PF_BAD_ARG;
  if (nix) *nix = h->nix;
  if (niy) *niy = h->niy;
  return PF_OK;
}

int pf_rk4_step(pf_handle *h, double szl, double hstep) {
  if (!h) return PF_BAD_ARG;
  if (!h->particles_set || h->nwin == 0) {
    h->err = "pf_rk4_step: particles not set";
    return PF_STATE;
  }
  cudaSetDevice(h->dev);
  unsigned int st = 0;
  int rc = (h->p.precision == PF_MIXED) ? pf_rk4_mixed(h, szl, hstep, &st)
                                         : pf_rk4_fp64(h, szl, hstep, &st);
  if (rc) return rc;
  rc = status_to_rc(st);
  if (rc == PF_OUT_OF_Z2) h->err = "a macroparticle's z2 node lies outside the temporal mesh";
  if (rc == PF_OUT_OF_WINDOW) h->err = "a macroparticle left the inner transverse window";
  if (rc == PF_OVERFLOW) h->err = "deposit contribution beyond the fixed-point range";
  if (rc == PF_NOT_FINITE) h->err = "a non-finite value in a macroparticle's state or in the field";
  return rc;
}

int pf_rk4_step_host(pf_handle *h, double szl, double hstep, double *x, double *y, double *z2,
                     double *px, double *py, double *gam, double *wre, double *wim) {
  if (!h || !x || !y || !z2 || !px || !py || !gam || !wre || !wim) return PF_BAD_ARG;
  if (!h->particles_set || h->nwin == 0 || h->np == 0) {
    h->err = "pf_rk4_step_host: particles not set";
    return PF_STATE;
  }
  cudaSetDevice(h->dev);
  // the arrays come in the caller's order: a z2-ordered handle's chi
  // follows them back
  if (h->permuted) {
    const int rc = unpermute_chi(h);
    if (rc) return rc;
    h->permuted = false;
  }
  double *const host[6] = {x, y, z2, px, py, gam};
  unsigned int st = 0;
  int rc = (h->p.precision == PF_MIXED) ? pf_rk4_mixed_host(h, szl, hstep, host, wre, wim, &st)
                                         : pf_rk4_fp64_host(h, szl, hstep, host, wre, wim, &st);
  if (rc) return rc;
  h->window_valid = true;
  rc = status_to_rc(st);
  if (rc == PF_OUT_OF_Z2) h->err = "a macroparticle's z2 node lies outside the temporal mesh";
  if (rc == PF_OUT_OF_WINDOW) h->err = "a macroparticle left the inner transverse window";
  if (rc == PF_OVERFLOW) h->err = "deposit contribution beyond the fixed-point range";
  if (rc == PF_NOT_FINITE) h->err = "a non-finite value in a macroparticle's state or in the field";
  return rc;
}

// inner2Outer + diffractIM + outer2Inner with the driver's arrays in host
// memory: the outer field and the window field go in by ranges of z2 planes
// on the copy stream, each range's window planes are copied into it and the
// first transverse passes run on it as it arrives; the last transverse
// passes write the outer field range by range, the range's window planes
// are taken from it, and the range goes out while the next is computed.  On
// a mixed handle the FP64 arrays are converted to and from the complex-float
// fields on the device (the outer field through the staging buffer, the
// window through its own).
int pf_diffract_host(pf_handle *h, double dz, double *ore, double *oim, double *wre,
                     double *wim) {
  if (!h || !ore || !oim) return PF_BAD_ARG;
  // the driver's window arrays are the window state whenever there is one
  const bool win = h->nwin > 0;
  if (win && (!wre || !wim)) return PF_BAD_ARG;
  cudaSetDevice(h->dev);
  const pf_params &p = h->p;
  const bool mixed = (p.precision == PF_MIXED);
  const bool periodic = (p.mesh_type == PF_MESH_PERIODIC);
  const int64_t plane = (int64_t)p.nx * p.ny, no = h->nouter;
  const int64_t nzf = periodic ? p.nz2 - 1 : p.nz2;  // planes the transforms run over
  // eight ranges of z2 planes (ranges graded down to 1/20 of the planes at
  // the ends measured no different)
  const int64_t n8 = std::max<int64_t>(1, std::min<int64_t>(8, nzf));
  std::vector<int64_t> zcut;
  for (int64_t c = 0; c <= n8; ++c) zcut.push_back(nzf * c / n8);
  const int nch = (int)zcut.size() - 1;
  if (!h->copy_stream) PF_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
  while ((int)h->copy_events.size() < 2 * nch + 1) {
    cudaEvent_t e;
    PF_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    h->copy_events.push_back(e);
  }
  // mixed: the FP64 outer field passes through the staging buffer (re then
  // im, nouter each) and the window through its own, converted on the device
  if (mixed && !h->staging) PF_CUDA(cudaMalloc(&h->staging, 2 * sizeof(double) * (size_t)no));
  if (mixed && win && h->wstage_cap < h->nwin) {
    cudaFree(h->wstage);
    h->wstage = nullptr;
    h->wstage_cap = 0;
    PF_CUDA(cudaMalloc(&h->wstage, 2 * sizeof(double) * (size_t)h->nwin));
    h->wstage_cap = h->nwin;
  }
  double *dre = mixed ? h->staging : h->or_, *dim = mixed ? h->staging + no : h->oi_;
  // the window's FP64 planes on the device (the window state itself, or its staging)
  double *wdr = mixed ? h->wstage : h->wr, *wdi = mixed ? h->wstage + h->nwin : h->wi;
  float2 *oc = (float2 *)h->oc32, *w32 = (float2 *)h->w32;
  cudaEvent_t *ev_in = h->copy_events.data(), *ev_out = ev_in + nch, ev_end = ev_in[2 * nch];
  cudaStream_t cs = h->copy_stream, st = h->stream;
  // window planes [z0, z0 + nz): wplane * nz values from wplane * z0 on
  const int64_t wplane = (int64_t)h->nix * h->niy;
  // in by ranges on the copy stream: the outer field's planes and the
  // window's planes of each range
  for (int c = 0; c < nch; ++c) {
    const size_t off = (size_t)(zcut[c] * plane), n = (size_t)((zcut[c + 1] - zcut[c]) * plane);
    PF_CUDA(cudaMemcpyAsync(dre + off, ore + off, n * sizeof(double), cudaMemcpyHostToDevice, cs));
    PF_CUDA(cudaMemcpyAsync(dim + off, oim + off, n * sizeof(double), cudaMemcpyHostToDevice, cs));
    if (win) {
      const size_t wo = (size_t)(zcut[c] * wplane), wn = (size_t)((zcut[c + 1] - zcut[c]) * wplane);
      PF_CUDA(cudaMemcpyAsync(wdr + wo, wre + wo, wn * sizeof(double), cudaMemcpyHostToDevice, cs));
      PF_CUDA(cudaMemcpyAsync(wdi + wo, wim + wo, wn * sizeof(double), cudaMemcpyHostToDevice, cs));
    }
    PF_CUDA(cudaEventRecord(ev_in[c], cs));
  }
  auto before = [&](int c) -> int {
    PF_CUDA(cudaStreamWaitEvent(st, ev_in[c], 0));
    const int64_t z0 = zcut[c], nz = zcut[c + 1] - zcut[c];
    if (mixed) {
      k_to_c32<<<grid_for(nz * plane, 256), 256, 0, st>>>(oc + z0 * plane, dre + z0 * plane,
                                                           dim + z0 * plane, nz * plane);
      PF_LAUNCHED(h);
      if (win) {
        k_to_c32<<<grid_for(nz * wplane, 256), 256, 0, st>>>(w32 + z0 * wplane, wdr + z0 * wplane,
                                                              wdi + z0 * wplane, nz * wplane);
        PF_LAUNCHED(h);
      }
    }
    if (win) {  // inner2Outer of the range's planes (range 0 also writes the mirror plane)
      const int mirror = (periodic && c == 0) ? 1 : 0;
      if (mixed)
        k_window_copy_c32<<<grid_for(wplane * nz, 256), 256, 0, st>>>(
            w32 + z0 * wplane, oc + z0 * plane, h->nix, h->niy, nz, p.nx, p.ny, p.nz2, 1, mirror);
      else
        k_window_copy<<<grid_for(wplane * nz, 256), 256, 0, st>>>(
            h->wr + z0 * wplane, h->wi + z0 * wplane, h->or_ + z0 * plane, h->oi_ + z0 * plane,
            h->nix, h->niy, nz, p.nx, p.ny, p.nz2, 1, mirror);
      PF_LAUNCHED(h);
    }
    return PF_OK;
  };
  auto after = [&](int c) -> int {
    const int64_t z0 = zcut[c], nz = zcut[c + 1] - zcut[c];
    if (win) {  // outer2Inner of the range's planes
      if (mixed) {
        k_window_copy_c32<<<grid_for(wplane * nz, 256), 256, 0, st>>>(
            w32 + z0 * wplane, oc + z0 * plane, h->nix, h->niy, nz, p.nx, p.ny, p.nz2, 0, 0);
        PF_LAUNCHED(h);
        k_from_c32<<<grid_for(nz * wplane, 256), 256, 0, st>>>(w32 + z0 * wplane, wdr + z0 * wplane,
                                                                wdi + z0 * wplane, nz * wplane);
      } else {
        k_window_copy<<<grid_for(wplane * nz, 256), 256, 0, st>>>(
            h->wr + z0 * wplane, h->wi + z0 * wplane, h->or_ + z0 * plane, h->oi_ + z0 * plane,
            h->nix, h->niy, nz, p.nx, p.ny, p.nz2, 0, 0);
      }
      PF_LAUNCHED(h);
    }
    if (mixed) {
      k_from_c32<<<grid_for(nz * plane, 256), 256, 0, st>>>(oc + z0 * plane, dre + z0 * plane,
                                                             dim + z0 * plane, nz * plane);
      PF_LAUNCHED(h);
      if (periodic && c == 0) {
        const int64_t mo = (p.nz2 - 1) * plane;
        k_from_c32<<<grid_for(plane, 256), 256, 0, st>>>(oc + mo, dre + mo, dim + mo, plane);
        PF_LAUNCHED(h);
      }
    }
    PF_CUDA(cudaEventRecord(ev_out[c], st));
    PF_CUDA(cudaStreamWaitEvent(cs, ev_out[c], 0));
    const size_t off = (size_t)(z0 * plane), n = (size_t)(nz * plane);
    PF_CUDA(cudaMemcpyAsync(ore + off, dre + off, n * sizeof(double), cudaMemcpyDeviceToHost, cs));
    PF_CUDA(cudaMemcpyAsync(oim + off, dim + off, n * sizeof(double), cudaMemcpyDeviceToHost, cs));
    if (periodic && c == 0) {  // the mirror plane, written with plane 0
      const size_t mo = (size_t)((p.nz2 - 1) * plane);
      PF_CUDA(cudaMemcpyAsync(ore + mo, dre + mo, (size_t)plane * sizeof(double),
                              cudaMemcpyDeviceToHost, cs));
      PF_CUDA(cudaMemcpyAsync(oim + mo, dim + mo, (size_t)plane * sizeof(double),
                              cudaMemcpyDeviceToHost, cs));
    }
    if (win) {
      const size_t wo = (size_t)(z0 * wplane), wn = (size_t)(nz * wplane);
      PF_CUDA(cudaMemcpyAsync(wre + wo, wdr + wo, wn * sizeof(double), cudaMemcpyDeviceToHost, cs));
      PF_CUDA(cudaMemcpyAsync(wim + wo, wdi + wo, wn * sizeof(double), cudaMemcpyDeviceToHost, cs));
    }
    return PF_OK;
  };
  int rc = pf_diffract_outer_ranges(h, dz, zcut, before, after);
  if (rc) {
    cudaStreamSynchronize(cs);
    cudaStreamSynchronize(st);
    return rc;
  }
  if (win) h->window_valid = true;
  PF_CUDA(cudaEventRecord(ev_end, st));
  PF_CUDA(cudaStreamWaitEvent(cs, ev_end, 0));
  PF_CUDA(cudaStreamSynchronize(cs));
  pf_prof_flush(h);
  return PF_OK;
}

int pf_wrap_z2(pf_handle *h) {
  if (!h) return PF_BAD_ARG;
  if (h->p.mesh_type != PF_MESH_PERIODIC || h->np == 0) return PF_OK;
  cudaSetDevice(h->dev);
  const double lenz2 = h->p.dz2 * (double)(h->p.nz2 - 1);
  k_wrap_z2<<<grid_for(h->np, 256), 256, 0, h->stream>>>(h->y[h->cur][2], h->np, lenz2);
  PF_LAUNCHED(h);
  return PF_OK;
}

int pf_redistribute(pf_handle *h) {
  if (!h) return PF_BAD_ARG;
  cudaSetDevice(h->dev);
  int rc = pf_inner_to_outer(h);
  if (rc) return rc;
  int nix, niy;
  rc = pf_window_from_particles(h, &nix, &niy);
  if (rc) return rc;
  rc = pf_wrap_z2(h);
  if (rc) return rc;
  h->window_valid = false;
  rc = alloc_window(h, nix, niy);
  if (rc) return rc;
  rc = pf_outer_to_inner(h);
  if (rc) return rc;
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

}  // extern "C"

int pf_diffract_enqueue(pf_handle *h, double dz) {
  int rc = pf_inner_to_outer(h);
  if (rc) return rc;
  rc = (h->p.precision == PF_MIXED) ? pf_diffract_outer_c32(h, h->oc32, dz)
                                     : pf_diffract_outer(h, dz);
  if (rc) return rc;
  if (h->nwin > 0) {
    rc = pf_outer_to_inner(h);
    if (rc) return rc;
  }
  return PF_OK;
}

extern "C" {

int pf_diffract(pf_handle *h, double dz) {
  if (!h) return PF_BAD_ARG;
  cudaSetDevice(h->dev);
  const int rc = pf_diffract_enqueue(h, dz);
  if (rc) return rc;
  PF_CUDA(cudaStreamSynchronize(h->stream));
  pf_prof_flush(h);
  return PF_OK;
}

}  // extern "C"

// Bytes of the state an asynchronous block can change: the current particle
// buffers and the window field.
static size_t block_state_bytes(const pf_handle *h, size_t *wbytes) {
  *wbytes = (h->p.precision == PF_MIXED) ? (size_t)h->nwin * 2 * sizeof(float)
                                         : (size_t)h->nwin * 2 * sizeof(double);
  return (size_t)6 * h->np * sizeof(double) + *wbytes;
}

// Copy the block state to (save) or from (restore) the snapshot buffer.
int pf_block_snapshot(pf_handle *h, bool save) {
  size_t wb;
  const size_t need = block_state_bytes(h, &wb);
  if (save && h->snap_cap < need) {
    cudaFree(h->snap);
    h->snap = nullptr;
    h->snap_cap = 0;
    PF_CUDA(cudaMalloc(&h->snap, need));
    h->snap_cap = need;
  }
  char *s = (char *)h->snap;
  const size_t pb = (size_t)h->np * sizeof(double);
  for (int j = 0; j < 6; ++j) {
    char *dst = save ? s + j * pb : (char *)h->y[h->cur][j];
    const char *src = save ? (const char *)h->y[h->cur][j] : s + j * pb;
    PF_CUDA(cudaMemcpyAsync(dst, src, pb, cudaMemcpyDeviceToDevice, h->stream));
  }
  char *ws = s + 6 * pb;
  if (h->p.precision == PF_MIXED) {
    PF_CUDA(cudaMemcpyAsync(save ? ws : (char *)h->w32, save ? (const char *)h->w32 : ws, wb,
                            cudaMemcpyDeviceToDevice, h->stream));
  } else {
    const size_t half = wb / 2;
    PF_CUDA(cudaMemcpyAsync(save ? ws : (char *)h->wr, save ? (const char *)h->wr : ws, half,
                            cudaMemcpyDeviceToDevice, h->stream));
    PF_CUDA(cudaMemcpyAsync(save ? ws + half : (char *)h->wi,
                            save ? (const char *)h->wi : ws + half, half,
                            cudaMemcpyDeviceToDevice, h->stream));
  }
  return PF_OK;
}

// A block of len RK4 steps (len even, no wrap inside) as one CUDA-graph
// launch.  The graph is captured once per (block length, buffers) and
// replayed; the per-(step, stage) coefficients reach the kernels through a
// device table uploaded before each launch, indexed by a device step counter
// that the last node kernel of every step advances.  *szl advances to the
// block's last step (whose position update, diffraction and wrap the caller
// does after the status check).
static int run_block_graph(pf_handle *h, int len, double hstep, double *szl) {
  const bool mixed = (h->p.precision == PF_MIXED);
  const size_t entry = mixed ? pf_step_coefficients_f_bytes() : 4 * sizeof(StageCoef);
  const size_t bytes = entry * (size_t)len;
  if (h->coef_cap < bytes) {
    cudaFree(h->coef_dev);
    if (h->coef_host) cudaFreeHost(h->coef_host);
    h->coef_dev = h->coef_host = nullptr;
    h->coef_cap = 0;
    PF_CUDA(cudaMalloc(&h->coef_dev, bytes));
    PF_CUDA(cudaMallocHost(&h->coef_host, bytes));
    h->coef_cap = bytes;
    if (h->gexec) {  // the captured graph reads the old table
      cudaGraphExecDestroy(h->gexec);
      h->gexec = nullptr;
    }
  }
  if (!h->step_ctr) PF_CUDA(cudaMalloc(&h->step_ctr, sizeof(int)));
  const void *key[6] = {h->y[0][0], h->y[1][0], mixed ? h->w32 : (const void *)h->wr,
                        (const void *)(intptr_t)h->np, (const void *)(intptr_t)h->nwin,
                        (const void *)(intptr_t)(h->nix * 65536 + h->niy)};
  bool same = h->gexec && h->g_len == len && h->g_cur == h->cur;
  for (int k = 0; k < 6; ++k) same = same && (h->g_key[k] == key[k]);
  const double szl0 = *szl;
  if (!same) {
    if (h->gexec) {
      cudaGraphExecDestroy(h->gexec);
      h->gexec = nullptr;
    }
    // capture: the drivers' host-side work runs (taper state and buffer
    // parity advance), so both are restored afterwards
    const double n2col = h->n2col, n2col0 = h->n2col0, undgrad = h->undgrad;
    const int cur = h->cur;
    const int64_t launches = h->launches;
    cudaGraph_t g = nullptr;
    PF_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    h->capturing = true;
    int rc = PF_OK;
    double z = szl0;
    for (int k = 0; k < len && rc == PF_OK; ++k) {
      unsigned int *none = nullptr;
      rc = mixed ? pf_rk4_mixed(h, z, hstep, none) : pf_rk4_fp64(h, z, hstep, none);
      z = z + hstep;
    }
    h->capturing = false;
    const cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
    h->g_nlaunch = h->launches - launches;
    h->launches = launches;
    h->n2col = n2col;
    h->n2col0 = n2col0;
    h->undgrad = undgrad;
    h->cur = cur;
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ce != cudaSuccess) {
      h->err = std::string("step-block capture: ") + cudaGetErrorString(ce);
      if (g) cudaGraphDestroy(g);
      return PF_CUDA_ERR;
    }
    const cudaError_t ie = cudaGraphInstantiate(&h->gexec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      h->gexec = nullptr;
      h->err = std::string("step-block graph: ") + cudaGetErrorString(ie);
      return PF_CUDA_ERR;
    }
    h->g_len = len;
    h->g_cur = h->cur;
    for (int k = 0; k < 6; ++k) h->g_key[k] = key[k];
  }
  // this block's coefficients (the taper state advances as the steps do)
  double z = szl0;
  for (int k = 0; k < len; ++k) {
    char *dst = (char *)h->coef_host + entry * (size_t)k;
    if (mixed) pf_step_coefficients_f(h, z, hstep, dst);
    else pf_step_coefficients(h, z, hstep, (StageCoef *)dst);
    if (k < len - 1) z = z + hstep;
  }
  *szl = z;
  PF_CUDA(cudaMemcpyAsync(h->coef_dev, h->coef_host, bytes, cudaMemcpyHostToDevice, h->stream));
  PF_CUDA(cudaMemsetAsync(h->step_ctr, 0, sizeof(int), h->stream));
  PF_CUDA(cudaGraphLaunch(h->gexec, h->stream));
  h->launches += h->g_nlaunch;
  return PF_OK;
}

void pf_sched_init(pf_handle *h, RunSched &s, int32_t nsteps, int32_t isteps4diff,
                   int32_t qdiffraction, double hstep, double *szl, int32_t *steps_done) {
  s.nsteps = nsteps;
  s.isteps4diff = isteps4diff;
  s.qdiffraction = qdiffraction;
  s.hstep = hstep;
  s.dzds = qdiffraction ? (double)isteps4diff * hstep / 2.0 : 0.0;
  s.redist = h->p.redist_every > 0 ? h->p.redist_every : 60;
  s.szl = szl;
  s.steps_done = steps_done;
  s.sync = true;
}

// What follows step istep of UndSection's loop (undulator.f90:214-330): the
// position, the diffraction of the step's end (the half step owed plus the
// next half step), the cumulative count and the periodic wrap.
int pf_sched_after_step(pf_handle *h, RunSched &s, int istep) {
  *s.szl = *s.szl + s.hstep;
  if (s.qdiffraction && (istep % s.isteps4diff == 0 || istep == s.nsteps)) {
    const double dzdf = s.dzds;
    if (istep == s.nsteps) s.dzds = 0.0;
    else if (istep + s.isteps4diff <= s.nsteps) s.dzds = (double)s.isteps4diff * s.hstep / 2;
    else s.dzds = (double)(s.nsteps - istep) * s.hstep / 2;
    const int r = s.sync ? pf_diffract(h, dzdf + s.dzds) : pf_diffract_enqueue(h, dzdf + s.dzds);
    if (r) return r;
  }
  h->csteps++;
  if (h->csteps % s.redist == 0) {
    const int r = pf_wrap_z2(h);
    if (r) return r;
  }
  // re-order at the wrap cadence, and (mixed precision, whose stage kernel
  // deposits through a shared tile of a few z2 planes per block) sooner when
  // more than 2 % of the macroparticles would miss their block's tile: a
  // bunched beam near saturation loses its z2 order within a few steps.
  // Checked after every block of steps, or every fourth step of a run that
  // goes step by step.
  const int64_t since = h->csteps - h->last_sort;
  bool disordered = false;
  if (h->sort_z2 && h->p.precision == PF_MIXED && since > 0 && h->np >= ((int64_t)1 << 15) &&
      (h->csteps - h->last_check >= 4 || h->csteps < h->last_check)) {
    h->last_check = h->csteps;
    double frac = 0.0;
    const int r = pf_mixed_order_misses(h, &frac);
    if (r) return r;
    disordered = frac > 0.02;
  }
  if (since >= s.redist || since < 0 || disordered) {
    const int r = pf_sort_z2(h);
    if (r) return r;
    h->last_sort = h->csteps;
  }
  if (s.steps_done) *s.steps_done = istep;
  return PF_OK;
}

// One step with the reference's window retries (undulator.f90:196-212).
int pf_sched_eager_step(pf_handle *h, RunSched &s, int istep) {
  int tries = 0;
  for (;;) {
    int r = pf_rk4_step(h, *s.szl, s.hstep);
    if (r == PF_OK) break;
    if (r != PF_OUT_OF_WINDOW || ++tries > 3) return r;
    r = pf_redistribute(h);  // getInNode + getLocalFieldIndices
    if (r) return r;
  }
  return pf_sched_after_step(h, s, istep);
}

extern "C" {

int pf_run(pf_handle *h, int32_t nsteps, int32_t isteps4diff, int32_t qdiffraction,
           double hstep, double *szl, int32_t *steps_done) {
  if (!h || !szl || nsteps < 0 || (qdiffraction && isteps4diff < 1)) return PF_BAD_ARG;
  if (steps_done) *steps_done = 0;
  if (nsteps > 0 && (!h->particles_set || h->nwin == 0)) {
    h->err = "pf_run: particles not set";
    return PF_STATE;
  }
  cudaSetDevice(h->dev);
  RunSched sc;
  pf_sched_init(h, sc, nsteps, isteps4diff, qdiffraction, hstep, szl, steps_done);
  int rc;
  if (qdiffraction) {
    rc = pf_diffract(h, sc.dzds);
    if (rc) return rc;
  }
  const int redist = sc.redist;
  // Steps between two diffraction calls run as one asynchronous block: the
  // kernels of every step are queued without a host round trip and the status
  // word is read once at the end (a failed step makes the rest of the block a
  // no-op).  If it failed, the state saved before the block is restored and
  // the block is replayed step by step with the reference's retries.  Used
  // when the saved state is small (launch-bound problems); larger problems
  // gain nothing from it and run step by step.
  size_t wb;
  const bool async_blocks = h->launch_mode >= 1 && block_state_bytes(h, &wb) <= ((size_t)256 << 20);
  int istep = 1;
  while (istep <= nsteps) {
    // the block ends at the next diffraction step (or after 16 steps)
    int last = qdiffraction ? std::min<int>(nsteps, ((istep - 1) / isteps4diff + 1) * isteps4diff)
                            : std::min<int>(nsteps, istep + 15);
    if (!async_blocks || last == istep) {
      rc = pf_sched_eager_step(h, sc, istep);
      if (rc) return rc;
      ++istep;
      continue;
    }
    // asynchronous block istep..last; its last step's diffraction runs after
    // the status check
    const double szl0 = *szl, n2col = h->n2col, n2col0 = h->n2col0, undgrad = h->undgrad;
    const int64_t csteps0 = h->csteps;
    const int cur0 = h->cur;
    rc = pf_block_snapshot(h, true);
    if (rc) return rc;
    PF_CUDA(cudaMemsetAsync(h->d_status, 0, sizeof(unsigned int), h->stream));
    const int len = last - istep + 1;
    bool wrap_inside = false;
    for (int k = 1; k < len; ++k) wrap_inside |= ((csteps0 + k) % redist == 0);
    if (h->use_graphs && !h->prof && h->g_warm && len == isteps4diff && len % 2 == 0 &&
        !wrap_inside) {
      rc = run_block_graph(h, len, hstep, szl);
      if (rc) return rc;
      h->csteps += len - 1;
    } else {
      for (int k = istep; k <= last; ++k) {
        unsigned int *none = nullptr;
        rc = (h->p.precision == PF_MIXED) ? pf_rk4_mixed(h, *szl, hstep, none)
                                          : pf_rk4_fp64(h, *szl, hstep, none);
        if (rc) return rc;
        if (k < last) {
          *szl = *szl + hstep;
          h->csteps++;
          if (h->csteps % redist == 0) {
            rc = pf_wrap_z2(h);
            if (rc) return rc;
          }
        }
      }
      h->g_warm = true;  // kernel attributes are set: later blocks may be captured
    }
    PF_CUDA(cudaMemcpyAsync(h->h_status, h->d_status, sizeof(unsigned int),
                            cudaMemcpyDeviceToHost, h->stream));
    PF_CUDA(cudaStreamSynchronize(h->stream));
    pf_prof_flush(h);
    if (*h->h_status == 0u) {
      rc = pf_sched_after_step(h, sc, last);  // last step's position, diffraction and wrap
      if (rc) return rc;
      istep = last + 1;
      continue;
    }
    // replay the block step by step from the saved state
    h->cur = cur0;
    rc = pf_block_snapshot(h, false);
    if (rc) return rc;
    *szl = szl0;
    h->n2col = n2col;
    h->n2col0 = n2col0;
    h->undgrad = undgrad;
    h->csteps = csteps0;
    for (int k = istep; k <= last; ++k) {
      rc = pf_sched_eager_step(h, sc, k);
      if (rc) return rc;
    }
    istep = last + 1;
  }
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

int pf_set_taper_profile(pf_handle *h, int32_t n, const double *z, const double *alpha) {
  if (!h || n < 0 || (n > 0 && (!z || !alpha)) || n == 1) return PF_BAD_ARG;
  for (int32_t k = 1; k < n; ++k)
    if (!(z[k] > z[k - 1])) {
      h->err = "taper profile abscissae must increase";
      return PF_BAD_ARG;
    }
  h->prof_z.assign(z, z + n);
  h->prof_a.assign(alpha, alpha + n);
  if (n > 0) h->n2col = h->n2col0 = alpha[0];
  return PF_OK;
}

int pf_set_fft_arithmetic(pf_handle *h, int32_t mode) {
  if (!h || (mode != PF_FFT_FP64 && mode != PF_FFT_PAIRED_FP32)) return PF_BAD_ARG;
  if (h->p.precision == PF_MIXED) {
    h->err = "pf_set_fft_arithmetic: the mixed-precision path transforms in FP32";
    return PF_BAD_ARG;
  }
  h->fft_pairs = (mode == PF_FFT_PAIRED_FP32);
  return PF_OK;
}

int pf_set_launch_mode(pf_handle *h, int32_t mode) {
  if (!h || mode < 0 || mode > 2) return PF_BAD_ARG;
  h->launch_mode = mode;
  h->use_graphs = (mode == 2);
  return PF_OK;
}

int64_t pf_step_count(const pf_handle *h) { return h ? h->csteps : -1; }

int pf_set_step_count(pf_handle *h, int64_t csteps) {
  if (!h || csteps < 0) return PF_BAD_ARG;
  h->csteps = csteps;
  return PF_OK;
}

int pf_sync(pf_handle *h) {
  if (!h) return PF_BAD_ARG;
  cudaSetDevice(h->dev);
  PF_CUDA(cudaStreamSynchronize(h->stream));
  return PF_OK;
}

int64_t pf_kernel_launches(const pf_handle *h) { return h ? h->launches : -1; }

void *pf_get_stream(const pf_handle *h) { return h ? (void *)h->stream : nullptr; }

int pf_profile(pf_handle *h, int32_t enable) {
  if (!h) return PF_BAD_ARG;
  cudaSetDevice(h->dev);
  PF_CUDA(cudaStreamSynchronize(h->stream));
  pf_prof_flush(h);
  for (int c = 0; c < PROF_N; ++c) {
    h->prof_ms[c] = 0.0;
    h->prof_n[c] = 0;
  }
  h->prof = enable != 0;
  return PF_OK;
}

int pf_profile_read(pf_handle *h, int32_t cls, double *ms_total, int64_t *launches) {
  if (!h || cls < 0 || cls >= PROF_N) return PF_BAD_ARG;
  cudaSetDevice(h->dev);
  PF_CUDA(cudaStreamSynchronize(h->stream));
  pf_prof_flush(h);
  if (ms_total) *ms_total = h->prof_ms[cls];
  if (launches) *launches = h->prof_n[cls];
  return PF_OK;
}

}  // extern "C"
