#include <type_traits>
// FFT diffraction kernels and host plan, instantiated once per real type
// (included by fft.cu with FFT_T = double / float and FFT_NS = fft64 / fft32).

namespace FFT_NS {

typedef FFT_T real;
typedef FFT_IO io_real;  // element type of the split re/im field in HBM
constexpr bool REAL_IS_DD = std::is_same<real, pf_dd>::value;
typedef pf_acc_of<real>::type acc;  // sums of products in the odd-prime butterflies

__device__ __forceinline__ double to_io(double v) { return v; }
__device__ __forceinline__ float to_io(float v) { return v; }
__device__ __forceinline__ double to_io(pf_dd v) { return dd_to_double(v); }
__device__ __forceinline__ double conv_in(double v, double *) { return v; }
__device__ __forceinline__ float conv_in(float v, float *) { return v; }
__device__ __forceinline__ pf_dd conv_in(double v, pf_dd *) { return dd_from_double(v); }
__device__ __forceinline__ real from_io(io_real v) { return conv_in(v, (real *)nullptr); }


struct cplx {
  real r, i;
};

__device__ __forceinline__ cplx cmul(cplx a, cplx b) {
  return cplx{a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r};
}
__device__ __forceinline__ cplx cadd(cplx a, cplx b) { return cplx{a.r + b.r, a.i + b.i}; }
__device__ __forceinline__ cplx csub(cplx a, cplx b) { return cplx{a.r - b.r, a.i - b.i}; }

constexpr int MAX_PASSES = 16;
constexpr int NTHREADS = 256;

// odd prime radices with unrolled butterflies; offsets into c_roots
constexpr int ODD_R[] = {3, 5, 7, 11, 13, 17, 43};
constexpr int N_ODD = 7;
__host__ __device__ constexpr int root_off(int R) {
  int off = 0;
  for (int q = 0; q < N_ODD; ++q) {
    if (ODD_R[q] == R) return off;
    off += ODD_R[q];
  }
  return -1;
}
constexpr int ROOTS_TOTAL = 3 + 5 + 7 + 11 + 13 + 17 + 43;
__constant__ cplx c_roots[ROOTS_TOTAL];  // (cos, sin)(2 pi m / R)


struct AxisPlan {
  int n;
  int npass;
  int radix[MAX_PASSES];
  int ns[MAX_PASSES];
  int twoff[MAX_PASSES];
  int64_t stride;   // element stride along the axis
  int64_t inner;    // base(L) = L % inner + (L / inner) * ostride
  int64_t ostride;
  int64_t nlines;   // the line kernel runs lines [line0, nlines)
  int64_t line0;
  int lpb;
  int axis;         // 0 x, 1 y, 2 z
  int pfa;          // 1: n = 129 = 3 * 43 as a prime-factor transform (k_fft)
};

struct MulTables {
  const cplx *px, *py;         // propagator factors (x,z) and (y,z)
  const real *dxt, *dyt;       // damping factors (x,z) and (y,z)
  const unsigned char *zflag;  // bit0: pass band, bit1: kz != 0
  const real *mask;            // transverse mask (y,x)
  const real *mz;              // z2 mask
  int nx, ny, nz;
  int qfilter;
  real ffact;
};

enum { MID_NONE = 0, MID_PROP = 1, MID_DAMP = 2, MID_SPLIT = 3, MID_RECOMB = 4,
       // adjoint of the diffraction step (see diffract_adjoint)
       MID_ADJ_SPLIT = 5, MID_ADJ_RECOMB = 6, MID_SCALE = 7 };

struct FftArgs {
  cplx *A;
  cplx *anb;
  const io_real *re_in, *im_in;  // split input (first pass)
  io_real *re_out, *im_out;      // split output (last pass)
  const cplx *tw_f, *tw_b;      // per-pass twiddles, forward and backward
  AxisPlan ax;
  AxisPlan ay;   // the y axis, for the transverse-plane kernel (ax is then x)
  MulTables T;
  int dir;       // direction of the first transform: 0 forward, 1 backward
  int mid;       // MID_*: operation after the first transform
  int second;    // run the opposite transform after the mid operation
  int load_split, store_split;
  int mirror;    // periodic: also write plane nz (mirror of plane 0) of the output
  // four-step z2 transform: w_N^(b k1) at [k1 * N2 + b], forward and backward
  const cplx *tw4f, *tw4b;
  int z0;        // the transverse-plane kernel runs planes z0 + blockIdx.x
};

__device__ __forceinline__ int64_t line_base(const AxisPlan &p, int64_t L) {
  return (L % p.inner) + (L / p.inner) * p.ostride;
}

// Asynchronous global -> shared copies (cp.async): a thread issues all of its
// loads of a line group or plane before waiting once, so the whole block's
// reads are in flight together.
template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(sa), "l"(gmem), "n"(BYTES)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// element pos of the pass input into shared slot dst
__device__ __forceinline__ void load_async(cplx *dst, const FftArgs &a, int64_t pos) {
  if (a.load_split) {
    static_assert(sizeof(io_real) == sizeof(real), "a split element fills its slot");
    cp_async<sizeof(io_real)>(&dst->r, a.re_in + pos);
    cp_async<sizeof(io_real)>(&dst->i, a.im_in + pos);
  } else {
    cp_async<sizeof(cplx)>(dst, a.A + pos);
  }
}

// Paired-FP32 arithmetic: a slot filled from the split FP64 field holds the
// FP64 bits; the thread that loaded it converts it in place after the wait.
__device__ __forceinline__ void fix_loaded(cplx *slot, const FftArgs &a) {
  if constexpr (REAL_IS_DD) {
    if (a.load_split) {
      const double r = *reinterpret_cast<const double *>(&slot->r);
      const double i = *reinterpret_cast<const double *>(&slot->i);
      slot->r = conv_in(r, (real *)nullptr);
      slot->i = conv_in(i, (real *)nullptr);
    }
  }
}

// ---- butterflies -------------------------------------------------------------
template <bool INV>
__device__ __forceinline__ cplx mul_mi(cplx b) {  // b * (-i) forward, b * (+i) backward
  return INV ? cplx{-b.i, b.r} : cplx{b.i, -b.r};
}

template <bool INV>
__device__ __forceinline__ void dft4(cplx &x0, cplx &x1, cplx &x2, cplx &x3) {
  const cplx a0 = cadd(x0, x2), a1 = csub(x0, x2);
  const cplx b0 = cadd(x1, x3), b1 = mul_mi<INV>(csub(x1, x3));
  x0 = cadd(a0, b0);
  x2 = csub(a0, b0);
  x1 = cadd(a1, b1);
  x3 = csub(a1, b1);
}

// DFT of v[0..R) written to dst[0], dst[ds], ..., dst[(R-1) ds].
template <int R, bool INV>
__device__ __forceinline__ void dft_store(cplx *v, cplx *dst, int ds) {
  if constexpr (R == 2) {
    dst[0] = cadd(v[0], v[1]);
    dst[ds] = csub(v[0], v[1]);
  } else if constexpr (R == 4) {
    dft4<INV>(v[0], v[1], v[2], v[3]);
#pragma unroll
    for (int r = 0; r < 4; ++r) dst[r * ds] = v[r];
  } else if constexpr (R == 8) {
    cplx e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    cplx o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<INV>(e0, e1, e2, e3);
    dft4<INV>(o0, o1, o2, o3);
    const real s = (real)0.70710678118654752440;
    // W8^1 = (s, -s) forward, (s, s) backward; W8^2 = -i / +i; W8^3 = (-s, -s) / (-s, s)
    const cplx t1 = INV ? cplx{s * (o1.r - o1.i), s * (o1.r + o1.i)}
                        : cplx{s * (o1.r + o1.i), s * (o1.i - o1.r)};
    const cplx t2 = mul_mi<INV>(o2);
    const cplx t3 = INV ? cplx{-s * (o3.r + o3.i), s * (o3.r - o3.i)}
                        : cplx{s * (o3.i - o3.r), -s * (o3.r + o3.i)};
    dst[0] = cadd(e0, o0);
    dst[4 * ds] = csub(e0, o0);
    dst[ds] = cadd(e1, t1);
    dst[5 * ds] = csub(e1, t1);
    dst[2 * ds] = cadd(e2, t2);
    dst[6 * ds] = csub(e2, t2);
    dst[3 * ds] = cadd(e3, t3);
    dst[7 * ds] = csub(e3, t3);
  }
}

// DFT of v[0..R) in place, outputs in natural order (R = 2, 4, 8).
template <int R, bool INV>
__device__ __forceinline__ void dft_regs(cplx *v) {
  if constexpr (R == 2) {
    const cplx a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if constexpr (R == 4) {
    dft4<INV>(v[0], v[1], v[2], v[3]);
  } else if constexpr (R == 8) {
    cplx e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    cplx o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<INV>(e0, e1, e2, e3);
    dft4<INV>(o0, o1, o2, o3);
    const real s = (real)0.70710678118654752440;
    const cplx t1 = INV ? cplx{s * (o1.r - o1.i), s * (o1.r + o1.i)}
                        : cplx{s * (o1.r + o1.i), s * (o1.i - o1.r)};
    const cplx t2 = mul_mi<INV>(o2);
    const cplx t3 = INV ? cplx{-s * (o3.r + o3.i), s * (o3.r - o3.i)}
                        : cplx{s * (o3.i - o3.r), -s * (o3.r + o3.i)};
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, t1);
    v[5] = csub(e1, t1);
    v[2] = cadd(e2, t2);
    v[6] = csub(e2, t2);
    v[3] = cadd(e3, t3);
    v[7] = csub(e3, t3);
  }
}

// Threads that share one odd-prime butterfly (each computes a subset of the
// output pairs), so a pass over few long butterflies still fills the block.
__host__ __device__ constexpr int odd_groups(int R) {
  return R >= 43 ? 7 : (R >= 17 ? 4 : (R >= 13 ? 3 : (R >= 11 ? 5 : 1)));
}

// Odd prime radix: X[q] = x0 + sum_j a_j cos(2 pi jq/R) -/+ i sum_j b_j sin(2 pi jq/R)
// with a_j = v_j + v_{R-j}, b_j = v_j - v_{R-j} formed as the inputs arrive,
// so only (R-1) complex values are live.  Thread g of the G sharing the
// butterfly writes X[0] (g = 0) and the pairs q = g+1, g+1+G, ...
template <int R, bool INV>
__device__ __forceinline__ void odd_butterfly(const cplx *src, int nb, const cplx *twk, bool twiddle,
                                              cplx *dst, int ds, int g) {
  constexpr int H = (R - 1) / 2;
  constexpr int G = odd_groups(R);
  constexpr int OFF = root_off(R);
  static_assert(OFF >= 0, "radix without an unrolled butterfly");
  cplx a[H], b[H];
  const cplx x0 = src[0];
  cplx s0 = x0;
#pragma unroll
  for (int j = 1; j <= H; ++j) {
    cplx u = src[j * nb], w = src[(R - j) * nb];
    if (twiddle) {
      u = cmul(u, twk[j]);
      w = cmul(w, twk[R - j]);
    }
    a[j - 1] = cadd(u, w);
    b[j - 1] = csub(u, w);
    s0 = cadd(s0, a[j - 1]);
  }
  if (g == 0) dst[0] = s0;
  // the root index m = j*q mod R is uniform across the threads of a group
#pragma unroll 1
  for (int q = g + 1; q <= H; q += G) {
    acc Cr = acc_start(x0.r), Ci = acc_start(x0.i);
    acc Sr = acc_start((real)0), Si = acc_start((real)0);
    int m = 0;
#pragma unroll
    for (int j = 1; j <= H; ++j) {
      m += q;
      if (m >= R) m -= R;
      const real c = c_roots[OFF + m].r;
      const real sn = c_roots[OFF + m].i;
      acc_fma(Cr, a[j - 1].r, c);
      acc_fma(Ci, a[j - 1].i, c);
      acc_fma(Sr, b[j - 1].r, sn);
      acc_fma(Si, b[j - 1].i, sn);
    }
    const cplx C{acc_end(Cr), acc_end(Ci)}, S{acc_end(Sr), acc_end(Si)};
    if (!INV) {
      dst[q * ds] = cplx{C.r + S.i, C.i - S.r};
      dst[(R - q) * ds] = cplx{C.r - S.i, C.i + S.r};
    } else {
      dst[q * ds] = cplx{C.r - S.i, C.i + S.r};
      dst[(R - q) * ds] = cplx{C.r + S.i, C.i - S.r};
    }
  }
}

// Odd prime radix shared by G > 1 threads per butterfly: the G threads first
// form a_j, b_j together into shared scratch (stride R complex per butterfly,
// which keeps the groups of a warp on distinct banks), then each computes its
// output pairs reading them back.  Only a handful of registers stay live.
template <int R, bool INV>
__device__ __forceinline__ void odd_pass_shared(const cplx *in, cplx *out, int n, int nl, int Ns,
                                                const cplx *tw, cplx *scratch) {
  constexpr int H = (R - 1) / 2;
  constexpr int G = odd_groups(R);
  constexpr int OFF = root_off(R);
  constexpr int BPR = NTHREADS / G;  // butterflies per round
  const int nb = n / R;
  const int nbt = nl * nb;
  const int btl = threadIdx.x / G, g = threadIdx.x - (threadIdx.x / G) * G;
  for (int base = 0; base < nbt; base += BPR) {
    const int bt = base + btl;
    const bool act = (btl < BPR) && (bt < nbt);
    int l = 0, j = 0, k = 0;
    cplx *ab = scratch + btl * R;
    if (act) {
      l = bt / nb;
      j = bt - l * nb;
      k = j % Ns;
      const cplx *src = in + l * n + j;
      const cplx *twk = tw + k * R;
      for (int jj = g + 1; jj <= H; jj += G) {
        cplx u = src[jj * nb], w = src[(R - jj) * nb];
        if (Ns > 1) {
          u = cmul(u, twk[jj]);
          w = cmul(w, twk[R - jj]);
        }
        ab[jj - 1] = cadd(u, w);
        ab[H + jj - 1] = csub(u, w);
      }
    }
    __syncthreads();
    if (act) {
      const cplx x0 = in[l * n + j];
      cplx *dst = out + l * n + (j / Ns) * Ns * R + k;
      if (g == 0) {
        cplx s0 = x0;
#pragma unroll
        for (int jj = 0; jj < H; ++jj) s0 = cadd(s0, ab[jj]);
        dst[0] = s0;
      }
#pragma unroll 1
      for (int q = g + 1; q <= H; q += G) {
        acc Cr = acc_start(x0.r), Ci = acc_start(x0.i);
        acc Sr = acc_start((real)0), Si = acc_start((real)0);
        int m = 0;
#pragma unroll
        for (int jj = 1; jj <= H; ++jj) {
          m += q;
          if (m >= R) m -= R;
          const real c = c_roots[OFF + m].r;
          const real sn = c_roots[OFF + m].i;
          const cplx av = ab[jj - 1], bv = ab[H + jj - 1];
          acc_fma(Cr, av.r, c);
          acc_fma(Ci, av.i, c);
          acc_fma(Sr, bv.r, sn);
          acc_fma(Si, bv.i, sn);
        }
        const cplx C{acc_end(Cr), acc_end(Ci)}, S{acc_end(Sr), acc_end(Si)};
        if (!INV) {
          dst[q * Ns] = cplx{C.r + S.i, C.i - S.r};
          dst[(R - q) * Ns] = cplx{C.r - S.i, C.i + S.r};
        } else {
          dst[q * Ns] = cplx{C.r - S.i, C.i + S.r};
          dst[(R - q) * Ns] = cplx{C.r + S.i, C.i - S.r};
        }
      }
    }
    __syncthreads();
  }
}

// scratch (complex values) an odd radix needs in odd_pass_shared
__host__ __device__ constexpr int odd_scratch(int R) {
  return odd_groups(R) > 1 ? (NTHREADS / odd_groups(R)) * R : 0;
}

// One Stockham pass of radix R from `in` to `out` over nl lines of length n.
template <int R, bool INV>
__device__ __forceinline__ void stockham_pass(const cplx *in, cplx *out, int n, int nl, int Ns,
                                              const cplx *tw, cplx *scratch) {
  const int nb = n / R;
  if constexpr (R == 2 || R == 4 || R == 8) {
    const int total = nl * nb;
    for (int t = threadIdx.x; t < total; t += NTHREADS) {
      const int l = t / nb, j = t - l * nb;
      const int k = j % Ns;
      const cplx *src = in + l * n + j;
      cplx *dst = out + l * n + (j / Ns) * Ns * R + k;
      cplx v[R];
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = src[r * nb];
      if (Ns > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) v[r] = cmul(v[r], tw[k * R + r]);
      }
      dft_store<R, INV>(v, dst, Ns);
    }
  } else if constexpr (odd_groups(R) > 1) {
    odd_pass_shared<R, INV>(in, out, n, nl, Ns, tw, scratch);
  } else {
    const int total = nl * nb;
    for (int t = threadIdx.x; t < total; t += NTHREADS) {
      const int l = t / nb, j = t - l * nb;
      const int k = j % Ns;
      odd_butterfly<R, INV>(in + l * n + j, nb, tw + k * R, Ns > 1,
                            out + l * n + (j / Ns) * Ns * R + k, Ns, 0);
    }
  }
}

// n = 129 = 3 * 43 as a prime-factor (Good-Thomas) transform: input
// element (n1, n2) at (43 n1 + 3 n2) mod 129, output (k1, k2) at
// (43 k1 + 87 k2) mod 129 (87 = 3 * (3^-1 mod 43)), so that the 3-point and
// 43-point DFTs need no twiddle factors between them (the mixed-radix form
// multiplies 126 values per line by twiddles).  Pass 1: the 43 three-point
// DFTs over n1, written as Y[k1][n2] at k1 * 43 + n2.
template <bool INV>
__device__ __forceinline__ void pfa129_pass3(const cplx *in, cplx *out, int nl) {
  const real c = c_roots[root_off(3) + 1].r, sn = c_roots[root_off(3) + 1].i;
  for (int t = threadIdx.x; t < nl * 43; t += NTHREADS) {
    const int l = t / 43, n2 = t - l * 43;
    const cplx *src = in + l * 129;
    const int i0 = 3 * n2;
    int i1 = i0 + 43, i2 = i0 + 86;
    if (i1 >= 129) i1 -= 129;
    if (i2 >= 129) i2 -= 129;
    const cplx x0 = src[i0], u = src[i1], w = src[i2];
    const cplx av = cadd(u, w), bv = csub(u, w);
    cplx C = x0;
    C.r = fma(av.r, c, C.r);
    C.i = fma(av.i, c, C.i);
    const cplx S{bv.r * sn, bv.i * sn};
    cplx *dst = out + l * 129 + n2;
    dst[0] = cadd(x0, av);
    if (!INV) {
      dst[43] = cplx{C.r + S.i, C.i - S.r};
      dst[86] = cplx{C.r - S.i, C.i + S.r};
    } else {
      dst[43] = cplx{C.r - S.i, C.i + S.r};
      dst[86] = cplx{C.r + S.i, C.i - S.r};
    }
  }
}

// Pass 2: the three 43-point DFTs over n2 (contiguous inputs Y[k1][.]),
// outputs to (43 k1 + 87 k2) mod 129; the butterfly shared by odd_groups(43)
// threads as in odd_pass_shared.
template <bool INV>
__device__ __forceinline__ void pfa129_pass43(const cplx *in, cplx *out, int nl, cplx *scratch) {
  constexpr int R = 43, H = 21;
  constexpr int G = odd_groups(R);
  constexpr int OFF = root_off(R);
  constexpr int BPR = NTHREADS / G;
  const int nbt = nl * 3;
  const int btl = threadIdx.x / G, g = threadIdx.x - (threadIdx.x / G) * G;
  for (int base = 0; base < nbt; base += BPR) {
    const int bt = base + btl;
    const bool act = (btl < BPR) && (bt < nbt);
    int l = 0, j = 0;
    cplx *ab = scratch + btl * R;
    if (act) {
      l = bt / 3;
      j = bt - l * 3;
      const cplx *src = in + l * 129 + j * 43;
      for (int jj = g + 1; jj <= H; jj += G) {
        const cplx u = src[jj], w = src[R - jj];
        ab[jj - 1] = cadd(u, w);
        ab[H + jj - 1] = csub(u, w);
      }
    }
    __syncthreads();
    if (act) {
      const cplx x0 = in[l * 129 + j * 43];
      cplx *dst = out + l * 129;
      const int k0 = 43 * j;
      if (g == 0) {
        cplx s0 = x0;
#pragma unroll
        for (int jj = 0; jj < H; ++jj) s0 = cadd(s0, ab[jj]);
        dst[k0] = s0;
      }
#pragma unroll 1
      for (int q = g + 1; q <= H; q += G) {
        acc Cr = acc_start(x0.r), Ci = acc_start(x0.i);
        acc Sr = acc_start((real)0), Si = acc_start((real)0);
        int m = 0;
#pragma unroll
        for (int jj = 1; jj <= H; ++jj) {
          m += q;
          if (m >= R) m -= R;
          const real c = c_roots[OFF + m].r;
          const real sn = c_roots[OFF + m].i;
          const cplx av = ab[jj - 1], bv = ab[H + jj - 1];
          acc_fma(Cr, av.r, c);
          acc_fma(Ci, av.i, c);
          acc_fma(Sr, bv.r, sn);
          acc_fma(Si, bv.i, sn);
        }
        const cplx C{acc_end(Cr), acc_end(Ci)}, S{acc_end(Sr), acc_end(Si)};
        const int kq = (k0 + 87 * q) % 129, kr = (k0 + 87 * (R - q)) % 129;
        if (!INV) {
          dst[kq] = cplx{C.r + S.i, C.i - S.r};
          dst[kr] = cplx{C.r - S.i, C.i + S.r};
        } else {
          dst[kq] = cplx{C.r - S.i, C.i + S.r};
          dst[kr] = cplx{C.r + S.i, C.i - S.r};
        }
      }
    }
    __syncthreads();
  }
}

// All passes of one transform; returns the buffer that holds the result.
template <bool INV>
__device__ __noinline__ cplx *transform(cplx *buf0, cplx *buf1, cplx *scratch, const AxisPlan &p,
                                        int nl, const cplx *tw) {
  cplx *in = buf0, *out = buf1;
  if (p.pfa) {
    pfa129_pass3<INV>(in, out, nl);
    __syncthreads();
    pfa129_pass43<INV>(out, in, nl, scratch);
    __syncthreads();
    return in;
  }
  for (int ps = 0; ps < p.npass; ++ps) {
    const int R = p.radix[ps], Ns = p.ns[ps];
    const cplx *twp = tw + p.twoff[ps];
    switch (R) {
      case 2: stockham_pass<2, INV>(in, out, p.n, nl, Ns, twp, scratch); break;
      case 4: stockham_pass<4, INV>(in, out, p.n, nl, Ns, twp, scratch); break;
      case 8: stockham_pass<8, INV>(in, out, p.n, nl, Ns, twp, scratch); break;
      case 3: stockham_pass<3, INV>(in, out, p.n, nl, Ns, twp, scratch); break;
      case 5: stockham_pass<5, INV>(in, out, p.n, nl, Ns, twp, scratch); break;
      case 7: stockham_pass<7, INV>(in, out, p.n, nl, Ns, twp, scratch); break;
      case 11: stockham_pass<11, INV>(in, out, p.n, nl, Ns, twp, scratch); break;
      case 13: stockham_pass<13, INV>(in, out, p.n, nl, Ns, twp, scratch); break;
      case 17: stockham_pass<17, INV>(in, out, p.n, nl, Ns, twp, scratch); break;
      case 43: stockham_pass<43, INV>(in, out, p.n, nl, Ns, twp, scratch); break;
      default: break;  // excluded when the plan is built
    }
    __syncthreads();
    cplx *tmp = in;
    in = out;
    out = tmp;
  }
  return in;
}

__device__ __forceinline__ cplx *run_transform(cplx *b0, cplx *b1, cplx *scratch, const FftArgs &a,
                                               int nl, int inv) {
  return inv ? transform<true>(b0, b1, scratch, a.ax, nl, a.tw_b)
             : transform<false>(b0, b1, scratch, a.ax, nl, a.tw_f);
}

// element coordinates (x, y, z) of element j of line L along the plan's axis
__device__ __forceinline__ void coords(const AxisPlan &p, const MulTables &T, int64_t L, int j,
                                       int &x, int &y, int &z) {
  if (p.axis == 0) {
    x = j;
    y = (int)(L % T.ny);
    z = (int)(L / T.ny);
  } else if (p.axis == 1) {
    x = (int)(L % T.nx);
    y = j;
    z = (int)(L / T.nx);
  } else {
    x = (int)(L % T.nx);
    y = (int)(L / T.nx);
    z = j;
  }
}

__device__ __forceinline__ cplx mid_op(const FftArgs &a, int64_t pos, int x, int y, int z, cplx v) {
  const MulTables &T = a.T;
  if (a.mid == MID_PROP) {  // MultiplyExp (diffraction.f90:155-176)
    const unsigned char f = T.zflag[z];
    if (f & 1) {
      if (f & 2) v = cmul(cmul(T.px[(int64_t)z * T.nx + x], T.py[(int64_t)z * T.ny + y]), v);
    } else if (T.qfilter) {
      v = cplx{(real)0, (real)0};
    }
  } else if (a.mid == MID_DAMP) {  // AbsorptionStep damping (diffraction.f90:480-501)
    if (T.zflag[z] & 2) {
      const real f = T.dxt[(int64_t)z * T.nx + x] * T.dyt[(int64_t)z * T.ny + y];
      v = cplx{f * v.r, f * v.i};
    }
  } else if (a.mid == MID_SPLIT) {  // /ffact then mask split (diffraction.f90:310, 454-470)
    v = cplx{v.r / T.ffact, v.i / T.ffact};
    const real mk = T.mask[(int64_t)y * T.nx + x];
    const real m = mk + T.mz[z] * ((real)1 - mk);
    const real nbm = (real)1 - m;
    a.anb[pos] = cplx{nbm * v.r, nbm * v.i};
    v = cplx{m * v.r, m * v.i};
  } else if (a.mid == MID_RECOMB) {  // /ffact then + A_nb (diffraction.f90:513-517)
    const cplx b = a.anb[pos];
    v = cplx{v.r / T.ffact + b.r, v.i / T.ffact + b.i};
  } else if (a.mid == MID_ADJ_SPLIT) {  // keep (1 - m) v for the adjoint recombine
    const real mk = T.mask[(int64_t)y * T.nx + x];
    const real nbm = (real)1 - (mk + T.mz[z] * ((real)1 - mk));
    a.anb[pos] = cplx{nbm * v.r, nbm * v.i};
  } else if (a.mid == MID_ADJ_RECOMB) {  // m (v / ffact) + (1 - m) v0
    const real mk = T.mask[(int64_t)y * T.nx + x];
    const real m = mk + T.mz[z] * ((real)1 - mk);
    const cplx b = a.anb[pos];
    v = cplx{m * (v.r / T.ffact) + b.r, m * (v.i / T.ffact) + b.i};
  } else if (a.mid == MID_SCALE) {
    v = cplx{v.r / T.ffact, v.i / T.ffact};
  }
  return v;
}

__device__ __forceinline__ void store(const FftArgs &a, int64_t pos, cplx v) {
  if (a.store_split) {
    const io_real vr = to_io(v.r), vi = to_io(v.i);
    a.re_out[pos] = vr;
    a.im_out[pos] = vi;
    if (a.mirror) {
      const int64_t plane = (int64_t)a.T.nx * a.T.ny;
      if (pos < plane) {
        a.re_out[pos + plane * a.T.nz] = vr;
        a.im_out[pos + plane * a.T.nz] = vi;
      }
    }
  } else {
    a.A[pos] = v;
    if (a.mirror) {  // the complex output is the outer mesh itself
      const int64_t plane = (int64_t)a.T.nx * a.T.ny;
      if (pos < plane) a.A[pos + plane * a.T.nz] = v;
    }
  }
}

// resident blocks per SM of the line kernel: 3 for the 8-byte reals (FP64
// and paired FP32, 80 registers; the paired form spills a few words, and
// measured 8 % slower at two blocks and 128 registers, 2 % slower at four
// blocks, 64 registers and 7 lines per block), 1 for FP32
constexpr int KFFT_MINB = (sizeof(real) == 8) ? 3 : 1;
__global__ void __launch_bounds__(NTHREADS, KFFT_MINB) k_fft(const FftArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx *smem_all = reinterpret_cast<cplx *>(smem_raw);
  const AxisPlan &p = a.ax;
  const int n = p.n;
  const int64_t L0 = p.line0 + (int64_t)blockIdx.x * p.lpb;
  const int nl = (int)min((int64_t)p.lpb, p.nlines - L0);
  const int tid = threadIdx.x;
  cplx *smem = smem_all;
  cplx *other = smem_all + (size_t)p.lpb * n;
  cplx *scratch = smem_all + (size_t)2 * p.lpb * n;

  // load: consecutive threads take consecutive lines (adjacent in memory)
  for (int t = tid; t < nl * n; t += NTHREADS) {
    int l, j;
    if (p.stride == 1) {
      l = t / n;
      j = t - l * n;
    } else {
      l = t % nl;
      j = t / nl;
    }
    const int64_t pos = line_base(p, L0 + l) + (int64_t)j * p.stride;
    load_async(smem + l * n + j, a, pos);
  }
  cp_async_wait_all();
  if constexpr (REAL_IS_DD) {
    for (int t = tid; t < nl * n; t += NTHREADS) {
      const int l = (p.stride == 1) ? t / n : t % nl, j = (p.stride == 1) ? t - (t / n) * n : t / nl;
      fix_loaded(smem + l * n + j, a);
    }
  }
  __syncthreads();
  {
    cplx *res = run_transform(smem, other, scratch, a, nl, a.dir);
    if (res != smem) {
      other = smem;
      smem = res;
    }
  }

  if (a.mid != MID_NONE) {
    for (int t = tid; t < nl * n; t += NTHREADS) {
      const int l = t / n, j = t - l * n;
      int x, y, z;
      coords(p, a.T, L0 + l, j, x, y, z);
      const int64_t pos = line_base(p, L0 + l) + (int64_t)j * p.stride;
      smem[t] = mid_op(a, pos, x, y, z, smem[t]);
    }
    __syncthreads();
    if (a.second) {
      cplx *res = run_transform(smem, other, scratch, a, nl, !a.dir);
      if (res != smem) {
        other = smem;
        smem = res;
      }
    }
  }

  for (int t = tid; t < nl * n; t += NTHREADS) {
    int l, j;
    if (p.stride == 1) {
      l = t / n;
      j = t - l * n;
    } else {
      l = t % nl;
      j = t / nl;
    }
    const int64_t pos = line_base(p, L0 + l) + (int64_t)j * p.stride;
    store(a, pos, smem[l * n + j]);
  }
}

// Element-wise form of a pass whose axis has length 1 (no transform): the
// load/store conversion and the split / recombine operations still apply.
__global__ void k_elementwise(const FftArgs a) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const MulTables &T = a.T;
  const int64_t n = (int64_t)T.nx * T.ny * T.nz;
  if (t >= n) return;
  const int x = (int)(t % T.nx), y = (int)((t / T.nx) % T.ny);
  const int z = (int)(t / ((int64_t)T.nx * T.ny));
  cplx v = a.load_split ? cplx{from_io(a.re_in[t]), from_io(a.im_in[t])} : a.A[t];
  v = mid_op(a, t, x, y, z, v);
  store(a, t, v);
}

// ---- in-place kernels specialised per transform length ------------------------
// The transverse-plane kernel (a whole nx*ny plane per block: the x and y
// transforms of one pass over HBM) and the four-step z2 kernels (G adjacent
// z2 lines per block, so that the strided z2 axis is read in whole 256-byte
// segments) hold their data in a single shared buffer.  A pass stages the
// inputs of each thread's butterflies in registers, the block syncs, and the
// outputs overwrite the inputs.  Lengths, radices and line counts are
// template constants, so each pass is straight-line code with constant index
// arithmetic; the host picks an instantiation for the mesh, and meshes
// without one use the two-buffer line kernel above.  Element j of line l sits
// at buf[l * ls + j * es].
constexpr int PT = 512;  // threads of the in-place kernels

// the host's factorisation (factorize below): eights, fours, twos, odd primes
__host__ __device__ constexpr int fac_count(int n) {
  int c = 0;
  while (n % 8 == 0) { n /= 8; ++c; }
  while (n % 4 == 0) { n /= 4; ++c; }
  while (n % 2 == 0) { n /= 2; ++c; }
  for (int p = 3; n > 1; p += 2)
    while (n % p == 0) { n /= p; ++c; }
  return c;
}
__host__ __device__ constexpr int fac_radix(int n, int k) {
  int c = 0;
  while (n % 8 == 0) { if (c++ == k) return 8; n /= 8; }
  while (n % 4 == 0) { if (c++ == k) return 4; n /= 4; }
  while (n % 2 == 0) { if (c++ == k) return 2; n /= 2; }
  for (int p = 3; n > 1; p += 2)
    while (n % p == 0) { if (c++ == k) return p; n /= p; }
  return 1;
}
__host__ __device__ constexpr int fac_ns(int n, int k) {
  int ns = 1;
  for (int q = 0; q < k; ++q) ns *= fac_radix(n, q);
  return ns;
}

// Shared-memory slot of logical element i: the XOR swizzle spreads the
// strided accesses of the Stockham passes (stride R*NS elements) over all
// banks; every access to the in-place buffer goes through it.
__device__ __forceinline__ int sw(int i) {
  return (sizeof(real) == 4) ? (i ^ ((i >> 4) & 15)) : (i ^ ((i >> 3) & 7));
}

// LM (line-major thread order): consecutive threads take adjacent lines at
// the same butterfly and the slots are not swizzled.  A warp's accesses are
// then to slots ls apart, which no two lanes of a 128-byte wavefront share a
// bank on when ls is 1 (interleaved lines) or odd.  Else consecutive threads
// take consecutive butterflies of a line and the XOR swizzle spreads their
// strided accesses (about two wavefronts per ideal one remain).
// element-wise operation applied to the outputs of a transform's last pass
// (line l, element e of the line), in place of a separate pass over shared
// memory; NoPost leaves them
struct NoPost {
  __device__ __forceinline__ cplx operator()(int, int, cplx v) const { return v; }
};

template <int N, int NL, int R, int NS, bool INV, bool LM = false, class Post = NoPost>
__device__ __forceinline__ void ip_pass(cplx *buf, int nl, int ls, int es, const cplx *tw,
                                        const Post &post = Post()) {
  constexpr int NB = N / R;
  constexpr int MAXB = (NL * NB + PT - 1) / PT;
  const int total = LM ? NL * NB : nl * NB;
  auto slot = [](int i) { return LM ? i : sw(i); };
  int obase[MAXB];
  if constexpr (R == 2 || R == 4 || R == 8) {
    cplx v[MAXB][R];
    int lb[MAXB], eb[MAXB];
#pragma unroll
    for (int b = 0; b < MAXB; ++b) {
      const int t = threadIdx.x + b * PT;
      obase[b] = -1;
      const int l = LM ? t % NL : t / NB, j = LM ? t / NL : t - (t / NB) * NB;
      if (t < total && (!LM || l < nl)) {
        const int k = j % NS;
        const int src = l * ls + j * es;
#pragma unroll
        for (int r = 0; r < R; ++r) v[b][r] = buf[slot(src + r * NB * es)];
        if constexpr (NS > 1) {
#pragma unroll
          for (int r = 1; r < R; ++r) v[b][r] = cmul(v[b][r], tw[k * R + r]);
        }
        lb[b] = l;
        eb[b] = (j / NS) * NS * R + k;
        obase[b] = l * ls + eb[b] * es;
      }
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < MAXB; ++b) {
      if (obase[b] < 0) continue;
      dft_regs<R, INV>(v[b]);
#pragma unroll
      for (int r = 0; r < R; ++r)
        buf[slot(obase[b] + r * NS * es)] = post(lb[b], eb[b] + r * NS, v[b][r]);
    }
    __syncthreads();
  } else {
    static_assert(std::is_same<Post, NoPost>::value, "output operations on radix 2, 4, 8 passes only");
    constexpr int H = (R - 1) / 2;
    constexpr int OFF = root_off(R);
    static_assert(OFF >= 0, "radix without an unrolled butterfly");
    cplx x0[MAXB], av[MAXB][H], bv[MAXB][H];
#pragma unroll
    for (int b = 0; b < MAXB; ++b) {
      const int t = threadIdx.x + b * PT;
      obase[b] = -1;
      const int l = LM ? t % NL : t / NB, j = LM ? t / NL : t - (t / NB) * NB;
      if (t < total && (!LM || l < nl)) {
        const int k = j % NS;
        const int src = l * ls + j * es;
        x0[b] = buf[slot(src)];
#pragma unroll
        for (int q = 1; q <= H; ++q) {
          cplx u = buf[slot(src + q * NB * es)], w = buf[slot(src + (R - q) * NB * es)];
          if constexpr (NS > 1) {
            u = cmul(u, tw[k * R + q]);
            w = cmul(w, tw[k * R + R - q]);
          }
          av[b][q - 1] = cadd(u, w);
          bv[b][q - 1] = csub(u, w);
        }
        obase[b] = l * ls + ((j / NS) * NS * R + k) * es;
      }
    }
    __syncthreads();
    const int ds = NS * es;
#pragma unroll
    for (int b = 0; b < MAXB; ++b) {
      if (obase[b] < 0) continue;
      const int o = obase[b];
      cplx s0 = x0[b];
#pragma unroll
      for (int q = 0; q < H; ++q) s0 = cadd(s0, av[b][q]);
      buf[slot(o)] = s0;
      // every thread runs the same (q, j) sequence: the root is an immediate
      // constant-bank operand
#pragma unroll
      for (int q = 1; q <= H; ++q) {
        acc Cr = acc_start(x0[b].r), Ci = acc_start(x0[b].i);
        acc Sr = acc_start((real)0), Si = acc_start((real)0);
#pragma unroll
        for (int j = 1; j <= H; ++j) {
          const int m = (j * q) % R;
          const real c = c_roots[OFF + m].r;
          const real sn = c_roots[OFF + m].i;
          acc_fma(Cr, av[b][j - 1].r, c);
          acc_fma(Ci, av[b][j - 1].i, c);
          acc_fma(Sr, bv[b][j - 1].r, sn);
          acc_fma(Si, bv[b][j - 1].i, sn);
        }
        const cplx C{acc_end(Cr), acc_end(Ci)}, S{acc_end(Sr), acc_end(Si)};
        if (!INV) {
          buf[slot(o + q * ds)] = cplx{C.r + S.i, C.i - S.r};
          buf[slot(o + (R - q) * ds)] = cplx{C.r - S.i, C.i + S.r};
        } else {
          buf[slot(o + q * ds)] = cplx{C.r - S.i, C.i + S.r};
          buf[slot(o + (R - q) * ds)] = cplx{C.r + S.i, C.i - S.r};
        }
      }
    }
    __syncthreads();
  }
}

// all passes of a length-N transform over (at most) NL lines
template <int N, int NL, bool INV, bool LM = false, int K = 0, class Post = NoPost>
__device__ __forceinline__ void ip_transform(cplx *buf, int nl, int ls, int es, const cplx *tw,
                                             const AxisPlan &p, const Post &post = Post()) {
  if constexpr (K < fac_count(N)) {
    if constexpr (K + 1 == fac_count(N))
      ip_pass<N, NL, fac_radix(N, K), fac_ns(N, K), INV, LM>(buf, nl, ls, es, tw + p.twoff[K],
                                                             post);
    else
      ip_pass<N, NL, fac_radix(N, K), fac_ns(N, K), INV, LM>(buf, nl, ls, es, tw + p.twoff[K]);
    ip_transform<N, NL, INV, LM, K + 1>(buf, nl, ls, es, tw, p, post);
  }
}

// line-major thread order, unswizzled slots: the x lines are NX apart (odd
// on every instantiated plane), the y lines adjacent
template <int NX, int NY>
__device__ __forceinline__ void xy_transform(cplx *buf, const FftArgs &a, bool inv) {
  static_assert(NX % 2 == 1, "conflict-free line-major passes need an odd row length");
  if (!inv) {
    ip_transform<NX, NY, false, true>(buf, NY, NX, 1, a.tw_f, a.ax);
    ip_transform<NY, NX, false, true>(buf, NX, 1, NX, a.tw_f, a.ay);
  } else {
    ip_transform<NY, NX, true, true>(buf, NX, 1, NX, a.tw_b, a.ay);
    ip_transform<NX, NY, true, true>(buf, NY, NX, 1, a.tw_b, a.ax);
  }
}

// One block per z2 plane: x and y transforms (and the mid operation and the
// opposite transforms) with a single read and write of the plane.
template <int NX, int NY>
__global__ void __launch_bounds__(PT, 1) k_fft_plane(const FftArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx *buf = reinterpret_cast<cplx *>(smem_raw);
  constexpr int plane = NX * NY;
  const int z = a.z0 + blockIdx.x;
  const int64_t off = (int64_t)z * plane;
  for (int t = threadIdx.x; t < plane; t += PT) load_async(buf + t, a, off + t);
  cp_async_wait_all();
  if constexpr (REAL_IS_DD)
    for (int t = threadIdx.x; t < plane; t += PT) fix_loaded(buf + t, a);
  __syncthreads();
  xy_transform<NX, NY>(buf, a, a.dir != 0);
  if (a.mid != MID_NONE) {
    for (int t = threadIdx.x; t < plane; t += PT)
      buf[t] = mid_op(a, off + t, t % NX, t / NX, z, buf[t]);
    __syncthreads();
    if (a.second) xy_transform<NX, NY>(buf, a, a.dir == 0);
  }
  for (int t = threadIdx.x; t < plane; t += PT) store(a, off + t, buf[t]);
}

// The z2 axis as a four-step transform, N = N1 * N2: z = N2 a + b
// (a < N1, b < N2), kz = k1 + N1 k2, and
//   X[k1 + N1 k2] = sum_b w_N2^(b k2) w_N^(b k1) sum_a x[N2 a + b] w_N1^(a k1).
// The fused pass "forward, mid operation at kz, inverse" of a diffraction
// step becomes three kernels, each reading and writing the mesh once, in
// place:
//   STEP 0, block (b, lines): DFT over a -> k1, times w_N^(b k1); element k1
//           goes to plane N2 k1 + b;
//   STEP 1, block (k1, lines): DFT over b -> k2 (plane N2 k1 + k2 holds
//           kz = k1 + N1 k2), the mid operation, inverse DFT over k2 -> b,
//           times w_N^(-b k1);
//   STEP 2, block (b, lines): inverse DFT over k1 -> a (plane N2 a + b).
// A block holds G adjacent lines (adjacent in HBM: whole 256-byte segments
// per plane) of one short transform, about 33 KB, so several blocks share an
// SM.  The short transforms are the in-place shared-memory passes above, with
// their plans in a.ax (length N1) and a.ay (length N2).
// output operations of the four-step kernels: the twiddle tw[e * s + c] of
// element e, and the propagator / damping of kz = f + n1 * e at the line's
// (x, y) (adjacent lines are adjacent x: coalesced reads of the tables)
struct Z4Twiddle {
  const cplx *tw;
  int s, c;
  __device__ __forceinline__ cplx operator()(int, int e, cplx v) const {
    return cmul(v, tw[e * s + c]);
  }
};
struct Z4Mid {
  const FftArgs *a;
  int L0, f, n1;
  __device__ __forceinline__ cplx operator()(int l, int e, cplx v) const {
    const int L = L0 + l;
    const int x = L % a->T.nx, y = L / a->T.nx;
    return mid_op(*a, 0, x, y, f + n1 * e, v);
  }
};

template <int N1, int N2, int G, int STEP>
__global__ void __launch_bounds__(PT, (sizeof(real) == 4) ? 4 : 3) k_z4(const FftArgs a) {
  static_assert(PT % G == 0, "a thread keeps one line of its group");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx *buf = reinterpret_cast<cplx *>(smem_raw);
  constexpr int M = (STEP == 1) ? N2 : N1;  // length of this step's transforms
  constexpr int JS = PT / G;                 // element stride of a thread's loops
  const int64_t plane = (int64_t)a.T.nx * a.T.ny;  // = number of lines
  const int64_t ngroups = (plane + G - 1) / G;
  const int64_t grp = (int64_t)blockIdx.x % ngroups;
  const int f = (int)((int64_t)blockIdx.x / ngroups);  // b (steps 0, 2) or k1 (step 1)
  const int64_t L0 = grp * G;
  const int nl = (int)min((int64_t)G, plane - L0);
  // the G lines interleaved in shared memory (element j of line l at
  // j * G + l): every element loop and every butterfly pass has consecutive
  // threads on adjacent lines (adjacent in HBM, consecutive shared slots: no
  // bank conflicts), and a thread's line never changes in the element loops
  const int l = threadIdx.x % G, j0 = threadIdx.x / G;
  const bool on = l < nl;
  auto pos_of = [&](int j) -> int64_t {
    const int64_t pz = (STEP == 1) ? (int64_t)N2 * f + j : (int64_t)N2 * j + f;
    return pz * plane + L0 + l;
  };
  if (on)
    for (int j = j0; j < M; j += JS) load_async(buf + j * G + l, a, pos_of(j));
  cp_async_wait_all();
  if constexpr (REAL_IS_DD)
    if (on)
      for (int j = j0; j < M; j += JS) fix_loaded(buf + j * G + l, a);
  __syncthreads();
  // FP32 (LSU-bound): the twiddles and the propagator / damping are applied
  // as the last radix pass writes its outputs (Z4Twiddle, Z4Mid); FP64
  // (FP64-bound, and short of registers for the fused form): separate
  // element passes
  constexpr bool FUSED = sizeof(real) == 4;
  if constexpr (STEP == 0 && FUSED) {
    ip_transform<N1, G, false, true>(buf, nl, 1, G, a.tw_f, a.ax, Z4Twiddle{a.tw4f, N2, f});
  } else if constexpr (STEP == 1 && FUSED) {
    ip_transform<N2, G, false, true>(buf, nl, 1, G, a.tw_f, a.ay,
                                     Z4Mid{&a, (int)L0, f, N1});
    ip_transform<N2, G, true, true>(buf, nl, 1, G, a.tw_b, a.ay, Z4Twiddle{a.tw4b, 1, f * N2});
  } else if constexpr (STEP == 0) {
    ip_transform<N1, G, false, true>(buf, nl, 1, G, a.tw_f, a.ax);
    if (on)
      for (int k1 = j0; k1 < M; k1 += JS)
        buf[k1 * G + l] = cmul(buf[k1 * G + l], a.tw4f[k1 * N2 + f]);
    __syncthreads();
  } else if constexpr (STEP == 1) {
    ip_transform<N2, G, false, true>(buf, nl, 1, G, a.tw_f, a.ay);
    if (on) {
      const int L = (int)(L0 + l);
      const int x = L % a.T.nx, y = L / a.T.nx;
      for (int k2 = j0; k2 < M; k2 += JS)
        buf[k2 * G + l] = mid_op(a, 0, x, y, f + N1 * k2, buf[k2 * G + l]);
    }
    __syncthreads();
    ip_transform<N2, G, true, true>(buf, nl, 1, G, a.tw_b, a.ay);
    if (on)
      for (int b = j0; b < M; b += JS)
        buf[b * G + l] = cmul(buf[b * G + l], a.tw4b[f * N2 + b]);
    __syncthreads();
  } else {
    ip_transform<N1, G, true, true>(buf, nl, 1, G, a.tw_b, a.ax);
  }
  if (on)
    for (int j = j0; j < M; j += JS) store(a, pos_of(j), buf[j * G + l]);
}

// Instantiated transverse planes (square meshes of the workloads) and long
// z2 lines; a plane must fit the 227 KB of shared memory of one block.
typedef void (*FftKernel)(const FftArgs);
struct PlaneKernel {
  int nx, ny;
  FftKernel fn;
};

static const PlaneKernel kPlaneKernels[] = {
    {17, 17, k_fft_plane<17, 17>}, {21, 21, k_fft_plane<21, 21>}, {33, 33, k_fft_plane<33, 33>},
    {65, 65, k_fft_plane<65, 65>},
#if FFT_REAL_IS_FLOAT
    {129, 129, k_fft_plane<129, 129>},
#endif
};
// four-step z2 transforms (N = n1 * n2) with g lines per block
constexpr int ZG = (sizeof(real) == 4) ? 64 : 32;
struct Z4Kernel {
  int n1, n2, g;
  FftKernel k[3];
};
static const Z4Kernel kZ4Kernels[] = {
    {64, 64, ZG, {k_z4<64, 64, ZG, 0>, k_z4<64, 64, ZG, 1>, k_z4<64, 64, ZG, 2>}},
    {64, 32, ZG, {k_z4<64, 32, ZG, 0>, k_z4<64, 32, ZG, 1>, k_z4<64, 32, ZG, 2>}},
};


// per-call tables: propagator and damping factors for step h
__global__ void k_tables(cplx *px, cplx *py, real *dxt, real *dyt, const double *kx,
                         const double *ky, const double *kz, int nx, int ny, int nz, double h,
                         double hd, double sbeta) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nxz = (int64_t)nx * nz, nyz = (int64_t)ny * nz;
  if (t < nxz) {
    const int z = (int)(t / nx), x = (int)(t % nx);
    const double kzz = kz[z];
    const double th = h * (kx[x] * kx[x]) / (2.0 * kzz);
    double s, c;
    sincos(th, &s, &c);
    px[t] = (kzz != 0.0) ? cplx{(real)c, (real)s} : cplx{(real)1, (real)0};
    dxt[t] = (real)((kzz != 0.0) ? exp(-hd * sbeta * fabs(kx[x]) / sqrt(fabs(2.0 * kzz))) : 1.0);
  } else if (t < nxz + nyz) {
    t -= nxz;
    const int z = (int)(t / ny), y = (int)(t % ny);
    const double kzz = kz[z];
    const double th = h * (ky[y] * ky[y]) / (2.0 * kzz);
    double s, c;
    sincos(th, &s, &c);
    py[t] = (kzz != 0.0) ? cplx{(real)c, (real)s} : cplx{(real)1, (real)0};
    dyt[t] = (real)((kzz != 0.0) ? exp(-hd * sbeta * fabs(ky[y]) / sqrt(fabs(2.0 * kzz))) : 1.0);
  }
}



struct Plan {
  int nx = 0, ny = 0, nz = 0;
  int64_t n = 0;
  AxisPlan ax[3];
  size_t smem[3] = {0, 0, 0};
  FftKernel plane = nullptr;  // x and y in one k_fft_plane pass
  size_t plane_smem = 0;
  const Z4Kernel *z4 = nullptr;  // four-step z2 transform, when N factors
  AxisPlan z4p1, z4p2;            // plans of the N1 and N2 transforms
  cplx *tw4 = nullptr;            // w_N^(b k1), forward then backward
  size_t z4_smem = 0;
  cplx *A = nullptr, *anb = nullptr;
  cplx *tw = nullptr;  // forward block then backward block
  size_t ntw = 0;
  cplx *px = nullptr, *py = nullptr;
  real *dxt = nullptr, *dyt = nullptr;
  double *kx = nullptr, *ky = nullptr, *kz = nullptr;
  real *mask = nullptr, *mz = nullptr;
  unsigned char *zflag = nullptr;
  double ffact = 1.0;
};

static void destroy(Plan *d) {
  if (!d) return;
  void *ptrs[] = {d->A, d->anb, d->tw, d->px, d->py, d->dxt, d->dyt,
                  d->kx, d->ky, d->kz, d->mask, d->mz, d->zflag, d->tw4};
  for (void *q : ptrs) cudaFree(q);
  delete d;
}

static bool radix_supported(int r) {
  if (r == 2 || r == 4 || r == 8) return true;
  for (int q = 0; q < N_ODD; ++q)
    if (ODD_R[q] == r) return true;
  return false;
}

static std::vector<int> factorize(int n) {
  std::vector<int> f;
  while (n % 8 == 0) { f.push_back(8); n /= 8; }
  while (n % 4 == 0) { f.push_back(4); n /= 4; }
  while (n % 2 == 0) { f.push_back(2); n /= 2; }
  for (int p = 3; n > 1; p += 2)
    while (n % p == 0) { f.push_back(p); n /= p; }
  return f;
}

// linspace (base_functions.f90:67-98)
static std::vector<double> linspace(double a, double b, int n) {
  std::vector<double> v(n);
  if (n == 1) { v[0] = a; return v; }
  const double d = (b - a) / (double)(n - 1);
  for (int i = 0; i < n; ++i) v[i] = a + i * d;
  return v;
}

static double sq(double v) { return v * v; }

// Mask1D2 (masks.f90:266-302): the lower-end assignment is made second and
// wins where the two ends overlap.
static std::vector<double> mask1d2(const std::vector<double> &x, double dx, int nx, int nb) {
  const double pi = PF_PUFFIN_PI;
  std::vector<double> m(nx, 0.0);
  const double lb = (nb - 1) * dx, x01 = x[nx - 1], x02 = x[0];
  for (int j = std::max(0, nx - nb); j < nx; ++j) m[j] = sq(cos(pi * (x[j] - x01) / (2.0 * lb)));
  for (int j = 0; j < std::min(nb, nx); ++j) m[j] = sq(cos(pi * (x[j] - x02) / (2.0 * lb)));
  for (int j = nb; j < nx - nb; ++j) m[j] = 0.0;
  return m;
}

// Maskf4 (masks.f90:329-361)
static std::vector<double> maskf4(const std::vector<double> &x, double dx, int nx, int nb) {
  const double pi = PF_PUFFIN_PI;
  std::vector<double> m(nx, 0.0);
  const double lb = (nb - 1) * dx, x01 = x[std::max(0, nx - nb)], x02 = x[std::min(nb, nx) - 1];
  for (int j = std::max(0, nx - nb); j < nx; ++j) m[j] = sq(cos(pi * (x[j] - x01) / (2.0 * lb)));
  for (int j = 0; j < std::min(nb, nx); ++j) m[j] = sq(cos(pi * (x[j] - x02) / (2.0 * lb)));
  for (int j = nb; j < nx - nb; ++j) m[j] = 1.0;
  return m;
}

static int build_plan(pf_handle *h, Plan *&out) {
  const pf_params &p = h->p;
  Plan *d = new Plan();
  out = d;
  d->nx = p.nx;
  d->ny = p.ny;
  d->nz = (int)h->npl;
  d->n = (int64_t)d->nx * d->ny * d->nz;
  d->ffact = (double)p.nx * (double)p.ny * (double)d->nz;
  const int dims[3] = {d->nx, d->ny, d->nz};
  const int64_t strides[3] = {1, d->nx, (int64_t)d->nx * d->ny};
  if (d->nz < 2) {
    h->err = "diffraction needs at least 2 z2 planes in the transform";
    return PF_BAD_ARG;
  }

  // roots of unity of the unrolled odd radices
  {
    std::vector<cplx> roots;
    for (int q = 0; q < N_ODD; ++q)
      for (int m = 0; m < ODD_R[q]; ++m) {
        const double ang = 2.0 * PF_FULL_PI * (double)m / (double)ODD_R[q];
        roots.push_back(cplx{(real)cos(ang), (real)sin(ang)});
      }
    PF_CUDA(cudaMemcpyToSymbol(c_roots, roots.data(), roots.size() * sizeof(cplx)));
  }

  std::vector<cplx> tab, tabb;
  int max_smem = 0;
  PF_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->dev));
  for (int a = 0; a < 3; ++a) {
    AxisPlan &ap = d->ax[a];
    memset(&ap, 0, sizeof(ap));
    ap.axis = a;
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
    if (ap.n == 1) continue;
    const std::vector<int> f = factorize(ap.n);
    for (int r : f)
      if (!radix_supported(r)) {
        h->err = "FFT length " + std::to_string(ap.n) + " has a prime factor " +
                 std::to_string(r) + " without a butterfly (supported: 2, 3, 5, 7, 11, 13, 17, 43)";
        return PF_BAD_ARG;
      }
    if ((int)f.size() > MAX_PASSES) {
      h->err = "FFT length has too many factors";
      return PF_BAD_ARG;
    }
    ap.npass = (int)f.size();
    ap.pfa = (ap.n == 129) ? 1 : 0;
    int scratch = 0;
    for (int r : f) scratch = std::max(scratch, odd_scratch(r));
    int ns = 1;
    int64_t lpb = (int64_t)1 << 20;
    for (int ps = 0; ps < ap.npass; ++ps) {
      const int R = f[ps];
      ap.radix[ps] = R;
      ap.ns[ps] = ns;
      ap.twoff[ps] = (int)tab.size();
      for (int k = 0; k < ns; ++k)
        for (int r = 0; r < R; ++r) {
          const double ang = -2.0 * PF_FULL_PI * (double)(k * r) / (double)(ns * R);
          tab.push_back(cplx{(real)cos(ang), (real)sin(ang)});
          tabb.push_back(cplx{(real)cos(ang), (real)-sin(ang)});
        }
      ns *= R;
    }
    // lines per block: about 2048 points per block, adjacent lines for the
    // strided axes, two buffers within the shared-memory limit
    // (FP64: about 1400 points, so that three blocks share an SM: measured
    // 5 % faster than two blocks of 2048 points, and faster than four)
    lpb = std::max<int64_t>(1, (sizeof(real) == 8 ? 1400 : 2048) / ap.n);
    lpb = std::min<int64_t>(lpb, ap.nlines);
    auto bytes = [&](int64_t lp) { return (size_t)(2 * lp * ap.n + scratch) * sizeof(cplx); };
    while (lpb > 1 && bytes(lpb) > (size_t)max_smem) --lpb;
    if (bytes(lpb) > (size_t)max_smem) {
      h->err = "FFT line too long for shared memory";
      return PF_BAD_ARG;
    }
    ap.lpb = (int)lpb;
    d->smem[a] = bytes(lpb);
  }
  // transverse-plane kernel: the whole nx*ny plane in one shared buffer
  for (const PlaneKernel &k : kPlaneKernels)
    if (k.nx == d->nx && k.ny == d->ny) {
      d->plane = k.fn;
      // whole swizzle groups of 16 elements (sw() permutes within a group)
      d->plane_smem = (((size_t)d->nx * d->ny + 15) / 16) * 16 * sizeof(cplx);
      PF_CUDA(cudaFuncSetAttribute((const void *)k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   max_smem));
    }
  if (d->plane_smem > (size_t)max_smem) d->plane = nullptr;
  // four-step z2 transform: sub-plans of lengths N1 and N2 (their twiddles
  // appended to the pass tables) and the w_N^(b k1) table
  std::vector<cplx> tw4;
  for (const Z4Kernel &k : kZ4Kernels)
    if (k.n1 * k.n2 == d->nz && !d->z4) {
      AxisPlan *sp[2] = {&d->z4p1, &d->z4p2};
      const int sn[2] = {k.n1, k.n2};
      for (int q = 0; q < 2; ++q) {
        AxisPlan &ap = *sp[q];
        memset(&ap, 0, sizeof(ap));
        ap.axis = 2;
        ap.n = sn[q];
        const std::vector<int> f = factorize(sn[q]);
        ap.npass = (int)f.size();
        int ns = 1;
        for (int ps = 0; ps < ap.npass; ++ps) {
          const int R = f[ps];
          ap.radix[ps] = R;
          ap.ns[ps] = ns;
          ap.twoff[ps] = (int)tab.size();
          for (int kk = 0; kk < ns; ++kk)
            for (int r = 0; r < R; ++r) {
              const double ang = -2.0 * PF_FULL_PI * (double)(kk * r) / (double)(ns * R);
              tab.push_back(cplx{(real)cos(ang), (real)sin(ang)});
              tabb.push_back(cplx{(real)cos(ang), (real)-sin(ang)});
            }
          ns *= R;
        }
      }
      tw4.resize((size_t)2 * d->nz);
      for (int k1 = 0; k1 < k.n1; ++k1)
        for (int b = 0; b < k.n2; ++b) {
          const double ang = -2.0 * PF_FULL_PI * (double)(b * k1) / (double)d->nz;
          tw4[(size_t)k1 * k.n2 + b] = cplx{(real)cos(ang), (real)sin(ang)};
          tw4[(size_t)d->nz + (size_t)k1 * k.n2 + b] = cplx{(real)cos(ang), (real)-sin(ang)};
        }
      const int m = std::max(k.n1, k.n2);
      d->z4_smem = (((size_t)k.g * m + 15) / 16) * 16 * sizeof(cplx);
      if (d->z4_smem > (size_t)max_smem) continue;
      for (int q = 0; q < 3; ++q)
        PF_CUDA(cudaFuncSetAttribute((const void *)k.k[q],
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
      d->z4 = &k;
    }
  if (d->z4) {
    PF_CUDA(cudaMalloc(&d->tw4, tw4.size() * sizeof(cplx)));
    PF_CUDA(cudaMemcpy(d->tw4, tw4.data(), tw4.size() * sizeof(cplx), cudaMemcpyHostToDevice));
  }
  d->ntw = tab.size();
  if (d->ntw) {
    PF_CUDA(cudaMalloc(&d->tw, 2 * d->ntw * sizeof(cplx)));
    PF_CUDA(cudaMemcpy(d->tw, tab.data(), d->ntw * sizeof(cplx), cudaMemcpyHostToDevice));
    PF_CUDA(cudaMemcpy(d->tw + d->ntw, tabb.data(), d->ntw * sizeof(cplx),
                       cudaMemcpyHostToDevice));
  }
  PF_CUDA(cudaFuncSetAttribute(k_fft, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));

  PF_CUDA(cudaMalloc(&d->A, d->n * sizeof(cplx)));
  PF_CUDA(cudaMalloc(&d->anb, d->n * sizeof(cplx)));
  PF_CUDA(cudaMalloc(&d->px, (size_t)d->nx * d->nz * sizeof(cplx)));
  PF_CUDA(cudaMalloc(&d->py, (size_t)d->ny * d->nz * sizeof(cplx)));
  PF_CUDA(cudaMalloc(&d->dxt, (size_t)d->nx * d->nz * sizeof(real)));
  PF_CUDA(cudaMalloc(&d->dyt, (size_t)d->ny * d->nz * sizeof(real)));

  // k-values (transforms.f90:472-590), full-precision pi
  auto kvals = [](int m, double len) {
    std::vector<double> k(m);
    const int mx = (int)ceil((double)m / 2.0);
    for (int i = 0; i < m; ++i) k[i] = 2.0 * PF_FULL_PI * (double)(i >= mx ? i - m : i) / len;
    return k;
  };
  const std::vector<double> kx = kvals(d->nx, (double)d->nx * p.dx);
  const std::vector<double> ky = kvals(d->ny, (double)d->ny * p.dy);
  const std::vector<double> kz = kvals(d->nz, (double)d->nz * p.dz2);
  PF_CUDA(cudaMalloc(&d->kx, kx.size() * sizeof(double)));
  PF_CUDA(cudaMalloc(&d->ky, ky.size() * sizeof(double)));
  PF_CUDA(cudaMalloc(&d->kz, kz.size() * sizeof(double)));
  PF_CUDA(cudaMemcpy(d->kx, kx.data(), kx.size() * sizeof(double), cudaMemcpyHostToDevice));
  PF_CUDA(cudaMemcpy(d->ky, ky.data(), ky.size() * sizeof(double), cudaMemcpyHostToDevice));
  PF_CUDA(cudaMemcpy(d->kz, kz.data(), kz.size() * sizeof(double), cudaMemcpyHostToDevice));

  // filter cutoff (diffraction.f90:138-139; sFilt from setup_calcs.f90:208-210)
  const double ppi = PF_PUFFIN_PI;
  const double lenz2 = p.dz2 * p.nz2;
  const double sfilt = lenz2 / (4 * ppi * p.rho) * p.sfilt_frac;
  double cutoff = 2.0 * ppi * sfilt / ((double)p.nz2 * p.dz2);
  if (p.mesh_type == PF_MESH_PERIODIC && p.sperwaves <= 1.1) cutoff = 0.0;
  std::vector<unsigned char> zf(d->nz);
  for (int z = 0; z < d->nz; ++z)
    zf[z] = (unsigned char)(((kz[z] > cutoff) || (kz[z] < -cutoff)) ? 1 : 0) |
            (unsigned char)((kz[z] != 0.0) ? 2 : 0);
  PF_CUDA(cudaMalloc(&d->zflag, zf.size()));
  PF_CUDA(cudaMemcpy(d->zflag, zf.data(), zf.size(), cudaMemcpyHostToDevice));

  // masks (masks.f90:50-189, 366-430)
  const double lenx = (d->nx - 1) * p.dx, leny = (d->ny - 1) * p.dy;
  const std::vector<double> xs = linspace(-lenx / 2, lenx / 2, d->nx);
  const std::vector<double> ys = linspace(-leny / 2, leny / 2, d->ny);
  const std::vector<double> maskx = mask1d2(xs, p.dx, d->nx, p.nbx);
  const std::vector<double> masky = mask1d2(ys, p.dy, d->ny, p.nby);
  const std::vector<double> maskx2 = maskf4(xs, p.dx, d->nx, p.nbx);
  std::vector<double> m2((size_t)d->nx * d->ny);
  for (int y = 0; y < d->ny; ++y)
    for (int x = 0; x < d->nx; ++x)
      m2[(size_t)y * d->nx + x] = 1.0 * maskx[x] + maskx2[x] * masky[y];
  std::vector<double> mzv(d->nz, 0.0);
  if (p.mesh_type != PF_MESH_PERIODIC) {
    const double dx = p.dz2;
    const std::vector<double> xz = linspace(0.0 * dx, (double)(d->nz - 1) * dx, d->nz);
    const double lb = (p.nbz2 - 1) * dx;
    const double lf = (p.nz2 - 1 * dx);  // getZ2Mask's own form (masks.f90:366-430)
    const double x0 = lf - lb / 2.0;
    const int fbn = p.nz2 - p.nbz2 + 1;
    for (int i = 0; i < d->nz; ++i)
      if (i + 1 >= fbn) mzv[i] = sq(cos(ppi * (xz[i] - x0) / lb));
  }
  {
    const std::vector<real> m2r(m2.begin(), m2.end()), mzr(mzv.begin(), mzv.end());
    PF_CUDA(cudaMalloc(&d->mask, m2r.size() * sizeof(real)));
    PF_CUDA(cudaMalloc(&d->mz, mzr.size() * sizeof(real)));
    PF_CUDA(cudaMemcpy(d->mask, m2r.data(), m2r.size() * sizeof(real), cudaMemcpyHostToDevice));
    PF_CUDA(cudaMemcpy(d->mz, mzr.data(), mzr.size() * sizeof(real), cudaMemcpyHostToDevice));
  }
  return PF_OK;
}

// One fused pass along `axis`; an axis of length 1 degrades to the
// element-wise form (load/store conversion, split, recombine).
static int fft_pass(pf_handle *h, Plan *d, FftArgs a, int axis) {
  a.ax = d->ax[axis];
  if (a.ax.n == 1) {
    if (a.mid == MID_SPLIT || a.mid == MID_RECOMB || a.load_split || a.store_split) {
      const unsigned g = (unsigned)((d->n + 255) / 256);
      pf_prof_begin(h, PROF_DIFF);
      k_elementwise<<<g, 256, 0, h->stream>>>(a);
      pf_prof_end(h);
      PF_LAUNCHED(h);
    }
    return PF_OK;
  }
  if (axis == 2 && d->z4 && a.dir == 0 && a.second && !a.load_split && !a.store_split &&
      (a.mid == MID_PROP || a.mid == MID_DAMP)) {
    const Z4Kernel &k = *d->z4;
    a.ax = d->z4p1;
    a.ay = d->z4p2;
    a.tw4f = d->tw4;
    a.tw4b = d->tw4 + d->nz;
    const int64_t ngroups = ((int64_t)d->nx * d->ny + k.g - 1) / k.g;
    for (int q = 0; q < 3; ++q) {
      const int64_t blocks = ngroups * (q == 1 ? k.n1 : k.n2);
      pf_prof_begin(h, PROF_FFT);
      k.k[q]<<<(unsigned)blocks, PT, d->z4_smem, h->stream>>>(a);
      pf_prof_end(h);
      PF_LAUNCHED(h);
    }
    return PF_OK;
  }
  const int64_t blocks = (a.ax.nlines + a.ax.lpb - 1) / a.ax.lpb;
  pf_prof_begin(h, PROF_FFT);
  k_fft<<<(unsigned)blocks, NTHREADS, d->smem[axis], h->stream>>>(a);
  pf_prof_end(h);
  PF_LAUNCHED(h);
  return PF_OK;
}

// One transverse-plane pass (x and y together).
static int plane_pass(pf_handle *h, Plan *d, FftArgs a) {
  a.ax = d->ax[0];
  a.ay = d->ax[1];
  pf_prof_begin(h, PROF_FFT);
  d->plane<<<(unsigned)d->nz, PT, d->plane_smem, h->stream>>>(a);
  pf_prof_end(h);
  PF_LAUNCHED(h);
  return PF_OK;
}

static void base_args(pf_handle *h, Plan *d, io_real *re, io_real *im, cplx *oc, FftArgs &a);
static int run_schedule(pf_handle *h, Plan *d, const FftArgs &a, bool split, bool adjoint);

// Diffract the outer mesh: split real/imaginary arrays (re, im) or, when
// those are null, the interleaved complex mesh oc (nz2 planes either way).
static int diffract(pf_handle *h, Plan *&plan, io_real *re, io_real *im, cplx *oc, double dz) {
  const pf_params &p = h->p;
  if (!plan) {
    int rc = build_plan(h, plan);
    if (rc) return rc;
  }
  Plan *d = plan;
  FftArgs a;
  base_args(h, d, re, im, oc, a);
  const bool split = (re != nullptr);
  const int64_t ntab = (int64_t)(d->nx + d->ny) * d->nz;
  pf_prof_begin(h, PROF_DIFF);
  k_tables<<<(unsigned)((ntab + 255) / 256), 256, 0, h->stream>>>(
      d->px, d->py, d->dxt, d->dyt, d->kx, d->ky, d->kz, d->nx, d->ny, d->nz, dz, dz, p.sbeta);
  pf_prof_end(h);
  PF_LAUNCHED(h);
  return run_schedule(h, d, a, split, false);
}

static void base_args(pf_handle *h, Plan *d, io_real *re, io_real *im, cplx *oc, FftArgs &a) {
  const pf_params &p = h->p;
  memset(&a, 0, sizeof(a));
  a.A = d->A;
  a.anb = d->anb;
  a.tw_f = d->tw;
  a.tw_b = d->tw + d->ntw;
  a.T.px = d->px;
  a.T.py = d->py;
  a.T.dxt = d->dxt;
  a.T.dyt = d->dyt;
  a.T.zflag = d->zflag;
  a.T.mask = d->mask;
  a.T.mz = d->mz;
  a.T.nx = d->nx;
  a.T.ny = d->ny;
  a.T.nz = d->nz;
  a.T.qfilter = p.qfilter;
  a.T.ffact = (real)d->ffact;
  if (re == nullptr) a.A = oc;  // transform the complex outer mesh in place
  a.re_in = re;
  a.im_in = im;
  a.re_out = re;
  a.im_out = im;
  a.mirror = (p.mesh_type == PF_MESH_PERIODIC);
}

// The pass sequence of one diffraction call: the forward step, or (adjoint)
// the same passes with the adjoint operations in reversed order.
static int run_schedule(pf_handle *h, Plan *d, const FftArgs &a, bool split, bool adjoint) {
  // forward: xy fwd | z fwd * prop * z inv | xy inv, split, xy fwd |
  //          z fwd * damp * z inv | xy inv, + A_nb
  // adjoint: (A_nb = (1 - m) v) xy fwd | z fwd * damp * z inv |
  //          xy inv, m v / ffact + A_nb, xy fwd | z fwd * conj(prop) * z inv |
  //          xy inv, / ffact
  const int mid2 = adjoint ? MID_DAMP : MID_PROP;
  const int mid3 = adjoint ? MID_ADJ_RECOMB : MID_SPLIT;
  const int mid4 = adjoint ? MID_PROP : MID_DAMP;
  const int mid5 = adjoint ? MID_SCALE : MID_RECOMB;
  if (d->plane) {
    struct PStep {
      int plane, dir, mid, second, load_split, store_split;
    };
    const PStep ps[5] = {
        {1, 0, MID_NONE, 0, 1, 0},
        {0, 0, mid2, 1, 0, 0},
        {1, 1, mid3, 1, 0, 0},
        {0, 0, mid4, 1, 0, 0},
        {1, 1, mid5, 0, 0, 1},
    };
    for (const PStep &s : ps) {
      FftArgs b = a;
      b.dir = s.dir;
      b.mid = s.mid;
      b.second = s.second;
      b.load_split = split && s.load_split && !adjoint;  // the adjoint loads A
      b.store_split = split && s.store_split;
      b.mirror = a.mirror && s.store_split;
      const int rc = s.plane ? plane_pass(h, d, b) : fft_pass(h, d, b, 2);
      if (rc) return rc;
    }
    return PF_OK;
  }
  struct Step {
    int axis, dir, mid, second, load_split, store_split;
  };
  const Step steps[9] = {
      {0, 0, MID_NONE, 0, 1, 0},  // x fwd (from re/im)
      {1, 0, MID_NONE, 0, 0, 0},  // y fwd
      {2, 0, mid2, 1, 0, 0},      // z fwd, propagate + filter (adjoint: damp), z inv
      {1, 1, MID_NONE, 0, 0, 0},  // y inv
      {0, 1, mid3, 1, 0, 0},      // x inv, split (adjoint: recombine), x fwd
      {1, 0, MID_NONE, 0, 0, 0},  // y fwd
      {2, 0, mid4, 1, 0, 0},      // z fwd, damp (adjoint: conjugate propagator), z inv
      {1, 1, MID_NONE, 0, 0, 0},  // y inv
      {0, 1, mid5, 0, 0, 1},      // x inv, recombine (adjoint: scale) (to re/im)
  };
  for (const Step &s : steps) {
    FftArgs b = a;
    b.dir = s.dir;
    b.mid = s.mid;
    b.second = s.second;
    b.load_split = split && s.load_split && !adjoint;
    b.store_split = split && s.store_split;
    // the mirror plane is written by the last pass only
    b.mirror = a.mirror && s.store_split;
    const int rc = fft_pass(h, d, b, s.axis);
    if (rc) return rc;
  }
  return PF_OK;
}

// The diffraction step of diffract() (split re/im arrays, or the
// interleaved complex mesh oc when re is null), with the first and the last
// transverse pass cut into ranges of z2 planes [zcut[c], zcut[c + 1]): the
// x passes of the line kernels (an x line lies in one plane: line y + ny z)
// or the plane kernel's passes.  before(c) runs before the first pass reads
// range c, after(c) once the last pass has written it (range 0 also carries
// the periodic mirror plane).  The other passes run whole.
static int diffract_ranges(pf_handle *h, Plan *&plan, io_real *re, io_real *im, cplx *oc,
                           double dz, const std::vector<int64_t> &zcut,
                           const std::function<int(int)> &before,
                           const std::function<int(int)> &after) {
  const pf_params &p = h->p;
  if (!plan) {
    int rc = build_plan(h, plan);
    if (rc) return rc;
  }
  Plan *d = plan;
  const int nch = (int)zcut.size() - 1;
  const bool split = (re != nullptr);
  if (!d->plane && d->ax[0].n == 1) {  // no transverse pass to cut: run whole
    for (int c = 0; c < nch; ++c) {
      const int rc = before(c);
      if (rc) return rc;
    }
    int rc = diffract(h, plan, re, im, oc, dz);
    for (int c = 0; c < nch && rc == PF_OK; ++c) rc = after(c);
    return rc;
  }
  FftArgs a;
  base_args(h, d, re, im, oc, a);
  const int64_t ntab = (int64_t)(d->nx + d->ny) * d->nz;
  pf_prof_begin(h, PROF_DIFF);
  k_tables<<<(unsigned)((ntab + 255) / 256), 256, 0, h->stream>>>(
      d->px, d->py, d->dxt, d->dyt, d->kx, d->ky, d->kz, d->nx, d->ny, d->nz, dz, dz, p.sbeta);
  pf_prof_end(h);
  PF_LAUNCHED(h);
  // a transverse pass (the plane kernel, or the line kernel along x or y:
  // x lines and y lines each lie in one plane) over the planes of range c
  auto range_pass = [&](FftArgs b, int axis, int c) {
    const int64_t z0 = zcut[c], z1 = zcut[c + 1];
    if (z1 <= z0) return PF_OK;
    pf_prof_begin(h, PROF_FFT);
    if (d->plane) {
      b.ax = d->ax[0];
      b.ay = d->ax[1];
      b.z0 = (int)z0;
      d->plane<<<(unsigned)(z1 - z0), PT, d->plane_smem, h->stream>>>(b);
    } else {
      const int64_t per = axis == 0 ? d->ny : d->nx;  // lines per plane
      b.ax = d->ax[axis];
      b.ax.line0 = per * z0;
      b.ax.nlines = per * z1;
      const int64_t blocks = (b.ax.nlines - b.ax.line0 + b.ax.lpb - 1) / b.ax.lpb;
      k_fft<<<(unsigned)blocks, NTHREADS, d->smem[axis], h->stream>>>(b);
    }
    pf_prof_end(h);
    PF_LAUNCHED(h);
    return PF_OK;
  };
  struct Step {
    int transverse, axis, dir, mid, second, load_split, store_split;
  };
  // the schedules of run_schedule: five passes with the plane kernel, nine
  // with the line kernels
  const Step plane_steps[5] = {
      {1, 0, 0, MID_NONE, 0, 1, 0}, {0, 2, 0, MID_PROP, 1, 0, 0}, {1, 0, 1, MID_SPLIT, 1, 0, 0},
      {0, 2, 0, MID_DAMP, 1, 0, 0}, {1, 0, 1, MID_RECOMB, 0, 0, 1},
  };
  const Step line_steps[9] = {
      {1, 0, 0, MID_NONE, 0, 1, 0},   {0, 1, 0, MID_NONE, 0, 0, 0}, {0, 2, 0, MID_PROP, 1, 0, 0},
      {0, 1, 1, MID_NONE, 0, 0, 0},   {0, 0, 1, MID_SPLIT, 1, 0, 0}, {0, 1, 0, MID_NONE, 0, 0, 0},
      {0, 2, 0, MID_DAMP, 1, 0, 0},   {0, 1, 1, MID_NONE, 0, 0, 0}, {1, 0, 1, MID_RECOMB, 0, 0, 1},
  };
  const Step *steps = d->plane ? plane_steps : line_steps;
  const int nsteps = d->plane ? 5 : 9;
  auto args_of = [&](const Step &st) {
    FftArgs b = a;
    b.dir = st.dir;
    b.mid = st.mid;
    b.second = st.second;
    b.load_split = split && st.load_split;
    b.store_split = split && st.store_split;
    b.mirror = a.mirror && st.store_split;
    return b;
  };
  // range by range: the first pass (x, or the plane kernel) as each range
  // arrives and, on the line schedule, the y pass after it; the last y pass
  // and the last pass before each range goes out.  The passes between run
  // whole.
  const int nedge = (!d->plane && d->ax[1].n > 1) ? 2 : 1;
  int rc = PF_OK;
  for (int c = 0; c < nch && rc == PF_OK; ++c) {
    rc = before(c);
    for (int k = 0; k < nedge && rc == PF_OK; ++k) rc = range_pass(args_of(steps[k]), steps[k].axis, c);
  }
  for (int k = nedge; k < nsteps - nedge && rc == PF_OK; ++k) {
    const Step &st = steps[k];
    rc = st.transverse ? plane_pass(h, d, args_of(st)) : fft_pass(h, d, args_of(st), st.axis);
  }
  for (int c = 0; c < nch && rc == PF_OK; ++c) {
    for (int k = nsteps - nedge; k < nsteps && rc == PF_OK; ++k)
      rc = range_pass(args_of(steps[k]), steps[k].axis, c);
    if (rc == PF_OK) rc = after(c);
  }
  return rc;
}

// Adjoint (with respect to the real inner product sum re*re' + im*im') of
// one diffraction step over dz on split re/im arrays of the outer mesh or,
// when those are null, on the interleaved complex mesh oc in place.  The
// step is A -> Abs(Prop(A)) with Prop = B P F / N (P the propagator and
// high-pass filter) and Abs(A) = B D F (m A) / N + (1 - m) A (D the damping,
// m the mask); FFTW's B is the adjoint of F, P's adjoint is the propagator
// over -dz (the filter and D are real), so the adjoint is
// Prop^H(Abs^H(v)) with Abs^H(v) = m (B D F v / N) + (1 - m) v.  The periodic
// mirror plane is not written.
static int diffract_adjoint(pf_handle *h, Plan *&plan, io_real *re, io_real *im, cplx *oc,
                            double dz) {
  const pf_params &p = h->p;
  if (!plan) {
    int rc = build_plan(h, plan);
    if (rc) return rc;
  }
  Plan *d = plan;
  FftArgs a;
  const bool split = (re != nullptr);
  base_args(h, d, re, im, oc, a);
  a.mirror = 0;
  const int64_t ntab = (int64_t)(d->nx + d->ny) * d->nz;
  k_tables<<<(unsigned)((ntab + 255) / 256), 256, 0, h->stream>>>(
      d->px, d->py, d->dxt, d->dyt, d->kx, d->ky, d->kz, d->nx, d->ny, d->nz, -dz, dz, p.sbeta);
  PF_LAUNCHED(h);
  // A = v, A_nb = (1 - m) v
  {
    FftArgs b = a;
    b.load_split = split ? 1 : 0;
    b.store_split = 0;
    b.mid = MID_ADJ_SPLIT;
    const unsigned g = (unsigned)((d->n + 255) / 256);
    k_elementwise<<<g, 256, 0, h->stream>>>(b);
    PF_LAUNCHED(h);
  }
  return run_schedule(h, d, a, split, true);
}

}  // namespace FFT_NS
