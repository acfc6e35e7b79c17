// Device-side helpers shared by the tprf_gb300 kernels (complex128 arithmetic,
// small DFT butterflies and the shared-memory Stockham FFT, generic over the
// element type: double2 or the double-float cdf of dfloat.cuh).
#pragma once

#include <cuda_runtime.h>

#include "dfloat.cuh"
#include "internal.hpp"

namespace tprf {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
// FP64 forms of the double-float butterfly adds (dfloat.cuh): plain adds, no renormalisation
__device__ __forceinline__ double2 cadd_lz(double2 a, double2 b) { return cadd(a, b); }
__device__ __forceinline__ double2 csub_lz(double2 a, double2 b) { return csub(a, b); }
__device__ __forceinline__ double2 cnorm(double2 a) { return a; }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// acc + a * b
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 acc) {
  return make_double2(fma(a.x, b.x, fma(-a.y, b.y, acc.x)), fma(a.x, b.y, fma(a.y, b.x, acc.y)));
}
// acc - a * b
__device__ __forceinline__ double2 cfms(double2 a, double2 b, double2 acc) {
  return make_double2(fma(-a.x, b.x, fma(a.y, b.y, acc.x)), fma(-a.x, b.y, fma(-a.y, b.x, acc.y)));
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double cabs2(double2 a) { return fma(a.x, a.x, a.y * a.y); }
__device__ __forceinline__ double2 crecip(double2 a) {
  const double d = 1.0 / cabs2(a);
  return make_double2(a.x * d, -a.y * d);
}
// multiply by -i (FWD) or +i
template <bool FWD>
__device__ __forceinline__ double2 mul_mi(double2 a) {
  return FWD ? make_double2(a.y, -a.x) : make_double2(-a.y, a.x);
}

// ---------------------------------------------------------------------------
// Generic complex element types for the FFT: double2 (native FP64) and cdf
// (double-float on the FP32 pipe). RealT<C> is the matching real type, kc<C>
// turns a literal into it at compile time.
template <class C> struct RealT;
template <> struct RealT<double2> { using type = double; };
template <> struct RealT<cdf> { using type = dfl; };

template <class C> __host__ __device__ constexpr typename RealT<C>::type kc(double v);
template <> __host__ __device__ constexpr double kc<double2>(double v) { return v; }
template <> __host__ __device__ constexpr dfl kc<cdf>(double v) { return kdf(v); }

__device__ __forceinline__ double2 caxpy(double k, double2 x, double2 y) {
  return make_double2(fma(k, x.x, y.x), fma(k, x.y, y.y));
}

template <class C> __device__ __forceinline__ C czero();
template <> __device__ __forceinline__ double2 czero<double2>() { return make_double2(0.0, 0.0); }
template <> __device__ __forceinline__ cdf czero<cdf>() { return cdf{dfl{0.f, 0.f}, dfl{0.f, 0.f}}; }

// Twiddle table of a plan in element type C: exp(-2 pi i t / n), t < n.
template <class C> __device__ __forceinline__ const C *twiddles(const FftDesc &d);
template <> __device__ __forceinline__ const double2 *twiddles<double2>(const FftDesc &d) { return d.tw; }
template <> __device__ __forceinline__ const cdf *twiddles<cdf>(const FftDesc &d) {
  return reinterpret_cast<const cdf *>(d.twf);
}

template <bool FWD, class C>
__device__ __forceinline__ C root(const C *tw, int idx) {
  const C t = tw[idx];
  return FWD ? t : cconj(t);
}

// ---------------------------------------------------------------------------
// Small DFTs, y_q = sum_r v_r exp(-+ 2 pi i r q / R) (FWD: minus sign).
template <class C, class K>
__device__ __forceinline__ C caxpy_lz(K k, C x, C y) {  // y + k x inside a butterfly
  return cadd_lz(y, cscale(x, k));
}
__device__ __forceinline__ double2 caxpy_lz(double k, double2 x, double2 y) { return caxpy(k, x, y); }

template <int R, bool FWD, class C> struct Dft;

template <bool FWD, class C> struct Dft<2, FWD, C> {
  static __device__ __forceinline__ void run(C *v) {
    const C a = v[0], b = v[1];
    v[0] = cadd_lz(a, b);
    v[1] = csub_lz(a, b);
  }
};

template <bool FWD, class C> struct Dft<3, FWD, C> {
  static __device__ __forceinline__ void run(C *v) {
    constexpr auto s3 = kc<C>(0.86602540378443864676);  // sin(2 pi / 3)
    constexpr auto mh = kc<C>(-0.5);
    const C t1 = cadd_lz(v[1], v[2]);
    const C t2 = caxpy_lz(mh, t1, v[0]);
    const C t4 = mul_mi<FWD>(cscale(csub_lz(v[1], v[2]), s3));
    v[0] = cadd_lz(v[0], t1);
    v[1] = cadd_lz(t2, t4);
    v[2] = csub_lz(t2, t4);
  }
};

template <bool FWD, class C> struct Dft<4, FWD, C> {
  static __device__ __forceinline__ void run(C *v) {
    const C a = cadd_lz(v[0], v[2]), b = csub_lz(v[0], v[2]);
    const C c = cadd_lz(v[1], v[3]), d = mul_mi<FWD>(csub_lz(v[1], v[3]));
    v[0] = cadd_lz(a, c);
    v[2] = csub_lz(a, c);
    v[1] = cadd_lz(b, d);
    v[3] = csub_lz(b, d);
  }
};

template <bool FWD, class C> struct Dft<5, FWD, C> {
  static __device__ __forceinline__ void run(C *v) {
    constexpr auto c1 = kc<C>(0.30901699437494742410);   // cos(2 pi / 5)
    constexpr auto c2 = kc<C>(-0.80901699437494742410);  // cos(4 pi / 5)
    constexpr auto s1 = kc<C>(0.95105651629515357212);   // sin(2 pi / 5)
    constexpr auto s2 = kc<C>(0.58778525229247312917);   // sin(4 pi / 5)
    constexpr auto ms1 = kc<C>(-0.95105651629515357212);
    const C a1 = cadd_lz(v[1], v[4]), b1 = csub_lz(v[1], v[4]);
    const C a2 = cadd_lz(v[2], v[3]), b2 = csub_lz(v[2], v[3]);
    const C x0 = v[0];
    const C r1 = caxpy_lz(c2, a2, caxpy_lz(c1, a1, x0));
    const C r2 = caxpy_lz(c1, a2, caxpy_lz(c2, a1, x0));
    // q = 1: -i (s1 b1 + s2 b2), q = 2: -i (s2 b1 - s1 b2)  (FWD)
    const C i1 = mul_mi<FWD>(caxpy_lz(s2, b2, cscale(b1, s1)));
    const C i2 = mul_mi<FWD>(caxpy_lz(ms1, b2, cscale(b1, s2)));
    v[0] = cadd_lz(x0, cadd_lz(a1, a2));
    v[1] = cadd_lz(r1, i1);
    v[4] = csub_lz(r1, i1);
    v[2] = cadd_lz(r2, i2);
    v[3] = csub_lz(r2, i2);
  }
};

template <bool FWD, class C> struct Dft<7, FWD, C> {
  static __device__ __forceinline__ void run(C *v) {
    // cos and sin of 2 pi m / 7, m = 1..6
    constexpr double cs[6] = {0.62348980185873353053, -0.22252093395631440429, -0.90096886790241912624,
                              -0.90096886790241912624, -0.22252093395631440429, 0.62348980185873353053};
    constexpr double sn[6] = {0.78183148246802980871, 0.97492791218182360702, 0.43388373911755812048,
                              -0.43388373911755812048, -0.97492791218182360702, -0.78183148246802980871};
    C a[3], b[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      a[q] = cadd_lz(v[q + 1], v[6 - q]);
      b[q] = csub_lz(v[q + 1], v[6 - q]);
    }
    const C x0 = v[0];
    v[0] = cadd_lz(x0, cadd_lz(a[0], cadd_lz(a[1], a[2])));
#pragma unroll
    for (int q = 1; q <= 3; ++q) {
      C re = x0, im = czero<C>();
#pragma unroll
      for (int r = 1; r <= 3; ++r) {
        const int m = (q * r) % 7;
        re = caxpy_lz(kc<C>(cs[m - 1]), a[r - 1], re);
        im = caxpy_lz(kc<C>(sn[m - 1]), b[r - 1], im);
      }
      im = mul_mi<FWD>(im);
      v[q] = cadd_lz(re, im);
      v[7 - q] = csub_lz(re, im);
    }
  }
};

template <bool FWD, class C> struct Dft<8, FWD, C> {
  static __device__ __forceinline__ void run(C *v) {
    constexpr auto h = kc<C>(0.70710678118654752440);
    C e[4] = {v[0], v[2], v[4], v[6]};
    C o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, FWD, C>::run(e);
    Dft<4, FWD, C>::run(o);
    // W8^1 o1 = h (o1 + mul_mi(o1)),  W8^2 o2 = mul_mi(o2),  W8^3 o3 = h (mul_mi(o3) - o3)
    const C t1 = cscale(cadd_lz(o[1], mul_mi<FWD>(o[1])), h);
    const C t2 = mul_mi<FWD>(o[2]);
    const C t3 = cscale(csub_lz(mul_mi<FWD>(o[3]), o[3]), h);
    v[0] = cadd_lz(e[0], o[0]);
    v[4] = csub_lz(e[0], o[0]);
    v[1] = cadd_lz(e[1], t1);
    v[5] = csub_lz(e[1], t1);
    v[2] = cadd_lz(e[2], t2);
    v[6] = csub_lz(e[2], t2);
    v[3] = cadd_lz(e[3], t3);
    v[7] = csub_lz(e[3], t3);
  }
};

// ---------------------------------------------------------------------------
// In-place decimation-in-time FFT on `ncol` interleaved columns held in
// shared memory: element i of column c is at [i * ncol + c]. The input must
// be loaded in mixed-radix digit-reversed order (element t of a column goes to
// position FftDesc::rev[t]); the output comes out in natural order. Stage s
// with radix R and Ns = R_0 ... R_{s-1} combines, for every butterfly j, the R
// elements base + r Ns (base = (j - j mod Ns) R + j mod Ns) after twiddling
// element r by W_{Ns R}^{(j mod Ns) r}. Butterflies of a stage touch disjoint
// elements, so one buffer suffices.
//
// Threads: ncol divides blockDim.x; a thread keeps one column and walks the
// butterflies j = j0, j0 + step, ..., so no integer division happens inside
// the loops.
// Column layout of an FFT buffer: element i of column c sits at
// cbase(c) + i * stride, cbase(c) = (c >> lgt) * blk + (c & (2^lgt - 1)).
// The plain interleaved layout is stride = ncol, lgt >= log2(ncol).
struct ColLayout {
  int stride, blk, lgt;
  __device__ __forceinline__ int cbase(int c) const { return ((c >> lgt) * blk) + (c & ((1 << lgt) - 1)); }
};
__device__ __forceinline__ ColLayout interleaved(int ncol) { return ColLayout{ncol, 0, 30}; }

template <int R, bool FWD, class C>
__device__ __forceinline__ void fft_stage(C *__restrict__ a, int n, int Ns, int ncol, const C *__restrict__ tw,
                                          ColLayout lay) {
  const int nbf = n / R;
  const int tws = n / (Ns * R);
  const int cb = lay.cbase(threadIdx.x % ncol);
  const int j0 = threadIdx.x / ncol;
  const int step = blockDim.x / ncol;
  const int kstep = step % Ns;
  int k = j0 % Ns;
  for (int j = j0; j < nbf; j += step) {
    const int base = (j - k) * R + k;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = a[(base + r * Ns) * lay.stride + cb];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], root<FWD>(tw, k * r * tws));
    }
    Dft<R, FWD, C>::run(v);
#pragma unroll
    for (int r = 0; r < R; ++r) a[(base + r * Ns) * lay.stride + cb] = cnorm(v[r]);
    k += kstep;
    if (k >= Ns) k -= Ns;
  }
}

// Stage with an arbitrary radix R (a prime factor the fixed butterflies do
// not cover): each work item computes one output q of one butterfly as a
// direct R-point sum, reading buffer `in` and writing the same positions of
// `out`. Cost R complex multiply-adds per output.
template <bool FWD, class C>
__device__ __noinline__ void fft_stage_generic(const C *__restrict__ in, C *__restrict__ out, int n, int R, int Ns,
                                               int ncol, const C *__restrict__ tw, ColLayout lay) {
  const int tws = n / (Ns * R);
  const int nbf = n / R;
  const int cb = lay.cbase(threadIdx.x % ncol);
  const int step = blockDim.x / ncol;
  for (int w = threadIdx.x / ncol; w < n; w += step) {
    const int j = w / R, q = w - (w / R) * R;
    const int k = j % Ns;
    const int base = (j - k) * R + k;
    C acc = czero<C>();
    for (int r = 0; r < R; ++r) {
      const int e = (int)(((long)k * r * tws + (long)((r * q) % R) * nbf) % n);
      acc = cadd(acc, cmul(in[(base + r * Ns) * lay.stride + cb], root<FWD>(tw, e)));
    }
    out[(base + q * Ns) * lay.stride + cb] = acc;
  }
}

// Full transform of the `ncol` columns in buffer a (digit-reversed order in,
// natural order out). b is a second buffer of the same size, used only when
// the plan has a generic-radix stage (d.has_generic), else may be null.
// Returns the buffer holding the result. Starts and ends with a barrier.
// With n_stages >= 0 only the first n_stages stages run (see last_stage_output).
template <bool FWD, class C>
__device__ C *fft_smem(C *a, C *b, const FftDesc &d, int ncol, int n_stages = -1, ColLayout lay = ColLayout{0, 0, 30}) {
  __syncthreads();
  const C *tw = twiddles<C>(d);
  int Ns = 1;
  const int nst = n_stages < 0 ? d.nst : n_stages;
  if (lay.stride == 0) lay = interleaved(ncol);
  for (int s = 0; s < nst; ++s) {
    const int R = d.radix[s];
    switch (R) {
      case 2: fft_stage<2, FWD>(a, d.n, Ns, ncol, tw, lay); break;
      case 3: fft_stage<3, FWD>(a, d.n, Ns, ncol, tw, lay); break;
      case 4: fft_stage<4, FWD>(a, d.n, Ns, ncol, tw, lay); break;
      case 5: fft_stage<5, FWD>(a, d.n, Ns, ncol, tw, lay); break;
      case 7: fft_stage<7, FWD>(a, d.n, Ns, ncol, tw, lay); break;
      case 8: fft_stage<8, FWD>(a, d.n, Ns, ncol, tw, lay); break;
      default: {
        fft_stage_generic<FWD>(a, b, d.n, R, Ns, ncol, tw, lay);
        C *t = a;
        a = b;
        b = t;
      }
    }
    Ns *= R;
    __syncthreads();
  }
  return a;
}

// Decimation in frequency: natural order in, digit-reversed order out (output
// t at position FftDesc::rev[t]). The DFT matrix is symmetric, so transposing
// the DIT factorisation F = S_last ... S_0 P (S_s = butterflies after
// twiddles) gives F = P^T (T_0 B_0) ... (T_last B_last): the same stages in
// reverse order, each butterfly first and its twiddles after. Lets a tile be
// loaded in natural order (bulk copies) and permuted on the way out instead.
template <int R, bool FWD, class C>
__device__ __forceinline__ void fft_stage_dif(C *__restrict__ a, int n, int Ns, int ncol, const C *__restrict__ tw,
                                              ColLayout lay) {
  const int nbf = n / R;
  const int tws = n / (Ns * R);
  const int cb = lay.cbase(threadIdx.x % ncol);
  const int j0 = threadIdx.x / ncol;
  const int step = blockDim.x / ncol;
  const int kstep = step % Ns;
  int k = j0 % Ns;
  for (int j = j0; j < nbf; j += step) {
    const int base = (j - k) * R + k;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = a[(base + r * Ns) * lay.stride + cb];
    Dft<R, FWD, C>::run(v);
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], root<FWD>(tw, k * r * tws));
    }
#pragma unroll
    for (int r = 0; r < R; ++r) a[(base + r * Ns) * lay.stride + cb] = cnorm(v[r]);
    k += kstep;
    if (k >= Ns) k -= Ns;
  }
}

// The full DIF transform of the `ncol` columns of buffer a, in place; plans
// with a generic-radix stage are not supported here (use fft_smem). Starts and
// ends with a barrier.
template <bool FWD, class C>
__device__ void fft_smem_dif(C *a, const FftDesc &d, int ncol, ColLayout lay = ColLayout{0, 0, 30}) {
  __syncthreads();
  const C *tw = twiddles<C>(d);
  if (lay.stride == 0) lay = interleaved(ncol);
  int Ns = d.n;
  for (int s = d.nst - 1; s >= 0; --s) {
    const int R = d.radix[s];
    Ns /= R;
    switch (R) {
      case 2: fft_stage_dif<2, FWD>(a, d.n, Ns, ncol, tw, lay); break;
      case 3: fft_stage_dif<3, FWD>(a, d.n, Ns, ncol, tw, lay); break;
      case 4: fft_stage_dif<4, FWD>(a, d.n, Ns, ncol, tw, lay); break;
      case 5: fft_stage_dif<5, FWD>(a, d.n, Ns, ncol, tw, lay); break;
      case 7: fft_stage_dif<7, FWD>(a, d.n, Ns, ncol, tw, lay); break;
      default: fft_stage_dif<8, FWD>(a, d.n, Ns, ncol, tw, lay); break;
    }
    __syncthreads();
  }
}

// One output i of the last DIT stage (radix R, Ns = n / R) computed directly
// from the buffer left by the other stages: X[i] = sum_r W_n^{r i} v[i mod Ns + r Ns]
// (the butterfly k = i mod Ns, its output q = i / Ns, with the twiddle and the
// R-point DFT root combined into one power of W_n). Used where only some
// outputs are needed.
template <bool FWD, class C>
__device__ __forceinline__ C last_stage_output(const C *__restrict__ a, const FftDesc &d, int ncol, int col, int i) {
  const C *tw = twiddles<C>(d);
  const int n = d.n, R = d.radix[d.nst - 1], Ns = n / R;
  // k = i mod Ns; the outputs kept (|m| < nw <= Ns) lie in the first and the last
  // block of Ns, which need no division
  const int k = i < Ns ? i : i >= n - Ns ? i - (n - Ns) : i % Ns;
  C v = a[k * ncol + col];
  int e = 0;
  for (int r = 1; r < R; ++r) {
    e += i;
    if (e >= n) e -= n;
    v = cadd(v, cmul(a[(k + r * Ns) * ncol + col], root<FWD>(tw, e)));
  }
  return v;
}

}  // namespace tprf
