// Diffraction step: batched mixed-radix Stockham FFTs along x, y and z2
// (FP64 complex, unnormalised like FFTW's forward -1 / backward +1
// transforms), the free-space propagator and high-pass filter, and the
// absorbing boundary.
//
// Reference: DiffractionStep / MultiplyExp / AbsorptionStep
// (puffin/lib/diffraction/diffraction.f90:111-523), masks (masks.f90:50-430),
// k-values (transforms.f90:472-590), ffact (setup/setup.f90:334-346).
//
// One diffraction call is nine line passes, each one read and one write of
// the mesh:
//   1 x fwd (reads the split re/im field)   2 y fwd
//   3 z fwd * propagator/filter * z inv     4 y inv
//   5 x inv, /ffact, mask split (writes A_nb), x fwd
//   6 y fwd   7 z fwd * boundary damping * z inv   8 y inv
//   9 x inv, /ffact, + A_nb (writes the split re/im field and the periodic
//     mirror plane)
// A block loads `lpb` lines of one axis into shared memory (adjacent lines
// are adjacent in HBM, so the strided y and z2 axes read whole 32-byte sectors
// when lpb >= 2) and runs every radix pass there between two buffers.
// Radices 2, 4 and 8 are explicit butterflies; odd primes use the symmetric
// real-cos/real-sin form of the DFT (half the multiplies of the direct sum)
// with the roots of unity in constant memory, fully unrolled so every root is
// an immediate constant-bank operand.  The propagator and the damping are
// separable per axis, exp(i h (kx^2+ky^2)/2kz) = exp(i h kx^2/2kz)
// exp(i h ky^2/2kz), and are applied from (x, z2) and (y, z2) tables.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <functional>
#include <string>
#include <vector>

#include "dd_real.cuh"
#include "pf_internal.h"

#define FFT_T double
#define FFT_IO double
#define FFT_NS fft64
#define FFT_REAL_IS_FLOAT 0
#include "fft_kernels.cuh"
#undef FFT_T
#undef FFT_IO
#undef FFT_NS
#undef FFT_REAL_IS_FLOAT
// the FP64 field transformed in paired-FP32 arithmetic (dd_real.cuh)
#define FFT_T pf_dd
#define FFT_IO double
#define FFT_NS fftdd
#define FFT_REAL_IS_FLOAT 0
#include "fft_kernels.cuh"
#undef FFT_T
#undef FFT_IO
#undef FFT_NS
#undef FFT_REAL_IS_FLOAT
#define FFT_T float
#define FFT_IO float
#define FFT_NS fft32
#define FFT_REAL_IS_FLOAT 1
#include "fft_kernels.cuh"
#undef FFT_T
#undef FFT_IO
#undef FFT_NS
#undef FFT_REAL_IS_FLOAT

struct DiffPlan {
  fft64::Plan *p64 = nullptr;
  fftdd::Plan *pdd = nullptr;
  fft32::Plan *p32 = nullptr;
};

void pf_diff_destroy(DiffPlan *d) {
  if (!d) return;
  if (d->p64) fft64::destroy(d->p64);
  if (d->pdd) fftdd::destroy(d->pdd);
  if (d->p32) fft32::destroy(d->p32);
  delete d;
}

int pf_diffract_outer(pf_handle *h, double dz) {
  if (!h->diff) h->diff = new DiffPlan();
  if (h->fft_pairs) return fftdd::diffract(h, h->diff->pdd, h->or_, h->oi_, nullptr, dz);
  return fft64::diffract(h, h->diff->p64, h->or_, h->oi_, nullptr, dz);
}

int pf_diffract_outer_c32(pf_handle *h, void *outer, double dz) {
  if (!h->diff) h->diff = new DiffPlan();
  return fft32::diffract(h, h->diff->p32, nullptr, nullptr, (fft32::cplx *)outer, dz);
}

int pf_diffract_outer_ranges(pf_handle *h, double dz, const std::vector<int64_t> &zcut,
                             const std::function<int(int)> &before,
                             const std::function<int(int)> &after) {
  if (!h->diff) h->diff = new DiffPlan();
  if (h->p.precision == PF_MIXED)
    return fft32::diffract_ranges(h, h->diff->p32, nullptr, nullptr, (fft32::cplx *)h->oc32, dz,
                                  zcut, before, after);
  if (h->fft_pairs)
    return fftdd::diffract_ranges(h, h->diff->pdd, h->or_, h->oi_, nullptr, dz, zcut, before,
                                  after);
  return fft64::diffract_ranges(h, h->diff->p64, h->or_, h->oi_, nullptr, dz, zcut, before,
                                after);
}

int pf_diffract_adjoint_split(pf_handle *h, double *re, double *im, double dz) {
  if (!h->diff) h->diff = new DiffPlan();
  return fft64::diffract_adjoint(h, h->diff->p64, re, im, nullptr, dz);
}

int pf_diffract_adjoint_c32(pf_handle *h, void *outer, double dz) {
  if (!h->diff) h->diff = new DiffPlan();
  return fft32::diffract_adjoint(h, h->diff->p32, nullptr, nullptr, (fft32::cplx *)outer, dz);
}
