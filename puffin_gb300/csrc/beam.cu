// Quiet-start beam generation on the device: Halton-sequence beamlets per
// z2 slice with Poisson shot noise, from a seeded counter-based random
// generator (the reference seeds from the clock).
//
// Reference: getSeqs / genHSeq / halton / projectRSeq / interp1
// (puffin/lib/macroparticle_generation/mp_sequences.f90:126-433), the
// beamlet loop of the sequence branch (MPfDists.f90:406-620) and applyNoise /
// addxDev (noise.f90:25-80).  Per slice k (centre z2m(k), width dz2, Ne(k)
// electrons) the same nseq sequence points are placed: x = xseq(j) xsig(k) +
// xm(k) (likewise y, px, py, gamma; Halton bases 2, 3, 5, 11, 7 projected on a
// unit Gaussian through the inverse CDF tabulated on 2000 points in [-4, 4]),
// z2 = z2m(k) + (halton13(j) - 1/2) dz2, and each beamlet represents
// Nk = Ne(k)/nseq electrons.  The shot noise draws Nk' ~ Poisson(Nk) and,
// when Nk' > 0, moves z2 by (u - 1/2) dz2 / sqrt(Nk') with u uniform.
//
// The sequences (nseq values per dimension) are computed on the host; the
// device expands them over the slices and draws the noise, one thread per
// macroparticle.  Random numbers: SplitMix64 finalisation of
// (seed, particle index, draw index) -> 53-bit uniforms; normals by
// Box-Muller; Poisson by Knuth's product method for a mean below 12 (draws
// 2..61 of the particle) and the rounded normal approximation
// mean + sqrt(mean) N(0,1) above (draws 0, 1); the jitter uses draw 63.
#include <math.h>
#include <string.h>

#include <vector>

#include "pf_internal.h"

namespace {

__host__ __device__ inline unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// uniform in (0, 1): draw d of particle i
__device__ inline double uniform01(unsigned long long seed, long long i, int d) {
  const unsigned long long r =
      mix64(seed ^ mix64((unsigned long long)i * 64ull + (unsigned long long)d));
  return ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

struct GenArgs {
  int64_t nslices, nseq;
  const double *seq;   // 6 x nseq: x, y, px, py, gamma (unit Gaussian), z2 offset (in dz2)
  const double *z2m, *ne, *mean, *sig;  // per slice; mean/sig: 5 per slice
  double dz2;
  int noise;
  unsigned long long seed;
  double chi_per_electron;
  double *x, *y, *z2, *px, *py, *gam, *chi;
};

__global__ void k_generate(const GenArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nslices * a.nseq) return;
  const int64_t k = i / a.nseq, j = i - k * a.nseq;
  const double *m = a.mean + 5 * k, *s = a.sig + 5 * k;
  double *out[5] = {a.x, a.y, a.px, a.py, a.gam};
#pragma unroll
  for (int d = 0; d < 5; ++d) out[d][i] = __dadd_rn(__dmul_rn(a.seq[d * a.nseq + j], s[d]), m[d]);
  double z = __dadd_rn(a.seq[5 * a.nseq + j], a.z2m[k]);
  double nk = a.ne[k] / (double)a.nseq;
  if (a.noise) {
    // Poisson(nk)
    double pk;
    if (nk < 12.0) {
      const double L = exp(-nk);
      double p = 1.0;
      int c = 0;
      for (int it = 0; it < 60; ++it) {  // P(count >= 60) < 1e-20 for a mean below 12
        p *= uniform01(a.seed, i, 2 + it);
        if (p <= L) break;
        ++c;
      }
      pk = (double)c;
    } else {
      const double u1 = uniform01(a.seed, i, 0), u2 = uniform01(a.seed, i, 1);
      const double g = sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
      pk = floor(nk + sqrt(nk) * g + 0.5);
    }
    if (pk > 0.0) {
      nk = pk;
      const double u = uniform01(a.seed, i, 63);
      z = z + (u - 0.5) * a.dz2 / sqrt(nk);
    }
  }
  a.z2[i] = z;
  a.chi[i] = nk * a.chi_per_electron;
}

}  // namespace

// halton(ind, base) (mp_sequences.f90:286-305)
static double halton(long long ind, int base) {
  double ft = 1.0, y = 0.0;
  long long it = ind;
  while (it > 0) {
    ft = ft / (double)base;
    y = y + ft * (double)(it % base);
    it = it / base;
  }
  return y;
}

// projectRSeq + interp1 (mp_sequences.f90:318-433): the inverse of the
// Gaussian CDF by linear interpolation on 2000 points in [-4, 4]
static void project_gauss(std::vector<double> &seq) {
  const int n = 2000;
  std::vector<double> yf(n), cdf(n);
  const double d = (4.0 - (-4.0)) / (double)(n - 1);
  for (int i = 0; i < n; ++i) {
    yf[i] = -4.0 + i * d;
    cdf[i] = 0.5 * (1.0 + erf(yf[i] / sqrt(2.0)));
  }
  for (double &v : seq) {
    double r;
    if (v > cdf[0] && v < cdf[n - 1]) {
      int ic = 0;
      while (v > cdf[ic]) ++ic;
      const int ifl = ic, ifu = ic + 1;
      const double dx = cdf[ifu] - cdf[ifl], locx = v - cdf[ifl];
      r = yf[ifl] * (1.0 - locx / dx);
      r = r + yf[ifu] * locx / dx;
    } else if (v <= cdf[0]) {
      r = yf[0];
    } else {
      r = yf[n - 1];
    }
    v = r;
  }
}

extern "C" {

int pf_generate_beam(pf_handle *h, int64_t nslices, const double *z2m, const double *ne,
                     double dz2, int32_t nseq, const double *mean, const double *sig,
                     int32_t noise, uint64_t seed, double chi_per_electron) {
  if (!h || nslices < 1 || nseq < 1 || !z2m || !ne || !mean || !sig || !(dz2 > 0.0))
    return PF_BAD_ARG;
  cudaSetDevice(h->dev);
  const int64_t n = nslices * nseq;
  // the six sequences of length nseq (getSeqs, Halton branch)
  const int bases[6] = {2, 3, 5, 11, 7, 13};
  std::vector<double> seq((size_t)6 * nseq);
  for (int d = 0; d < 6; ++d) {
    std::vector<double> v((size_t)nseq);
    for (int j = 0; j < nseq; ++j) v[j] = halton(j + 1, bases[d]);
    if (d < 5) project_gauss(v);
    else
      for (double &z : v) z = (z - 0.5) * dz2;
    memcpy(seq.data() + (size_t)d * nseq, v.data(), sizeof(double) * nseq);
  }
  // device staging: sequences, slice data, the 7 particle arrays
  const size_t bytes = sizeof(double) * (seq.size() + 12 * (size_t)nslices + 7 * (size_t)n);
  char *buf = nullptr;
  PF_CUDA(cudaMalloc(&buf, bytes));
  double *d = (double *)buf;
  GenArgs a;
  memset(&a, 0, sizeof(a));
  a.nslices = nslices;
  a.nseq = nseq;
  a.seq = d;
  a.z2m = d + seq.size();
  a.ne = a.z2m + nslices;
  a.mean = a.ne + nslices;
  a.sig = a.mean + 5 * nslices;
  double *p = (double *)a.sig + 5 * nslices;
  a.x = p;
  a.y = p + n;
  a.z2 = p + 2 * n;
  a.px = p + 3 * n;
  a.py = p + 4 * n;
  a.gam = p + 5 * n;
  a.chi = p + 6 * n;
  a.dz2 = dz2;
  a.noise = noise;
  a.seed = seed;
  a.chi_per_electron = chi_per_electron;
  int rc = PF_OK;
  if (cudaMemcpyAsync(d, seq.data(), sizeof(double) * seq.size(), cudaMemcpyHostToDevice,
                      h->stream) != cudaSuccess ||
      cudaMemcpyAsync((void *)a.z2m, z2m, sizeof(double) * nslices, cudaMemcpyDefault,
                      h->stream) != cudaSuccess ||
      cudaMemcpyAsync((void *)a.ne, ne, sizeof(double) * nslices, cudaMemcpyDefault,
                      h->stream) != cudaSuccess ||
      cudaMemcpyAsync((void *)a.mean, mean, sizeof(double) * 5 * nslices, cudaMemcpyDefault,
                      h->stream) != cudaSuccess ||
      cudaMemcpyAsync((void *)a.sig, sig, sizeof(double) * 5 * nslices, cudaMemcpyDefault,
                      h->stream) != cudaSuccess) {
    h->err = "pf_generate_beam: copy of the inputs failed";
    rc = PF_CUDA_ERR;
  }
  if (rc == PF_OK) {
    k_generate<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(a);
    if (cudaGetLastError() != cudaSuccess) {
      h->err = "pf_generate_beam: launch failed";
      rc = PF_CUDA_ERR;
    } else {
      h->launches++;
    }
  }
  if (rc == PF_OK)
    rc = pf_set_particles_dev(h, n, a.x, a.y, a.z2, a.px, a.py, a.gam, a.chi);
  cudaStreamSynchronize(h->stream);
  cudaFree(buf);
  return rc;
}

}  // extern "C"
