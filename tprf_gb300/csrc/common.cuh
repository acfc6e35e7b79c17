// Device-side helpers shared by the tprf_gb300 kernels (complex128 arithmetic,
// small DFT butterflies, the shared-memory Stockham FFT).
#pragma once

#include <cuda_runtime.h>

#include "internal.hpp"

namespace tprf {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
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
// Small DFTs, y_q = sum_r v_r exp(-+ 2 pi i r q / R) (FWD: minus sign).
template <int R, bool FWD> struct Dft;

template <bool FWD> struct Dft<2, FWD> {
  static __device__ __forceinline__ void run(double2 *v) {
    double2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <bool FWD> struct Dft<3, FWD> {
  static __device__ __forceinline__ void run(double2 *v) {
    const double s3 = 0.86602540378443864676;  // sin(2 pi / 3)
    double2 t1 = cadd(v[1], v[2]);
    double2 t2 = make_double2(fma(-0.5, t1.x, v[0].x), fma(-0.5, t1.y, v[0].y));
    double2 t3 = csub(v[1], v[2]);
    // -i s3 t3 (FWD) or +i s3 t3
    double2 t4 = FWD ? make_double2(s3 * t3.y, -s3 * t3.x) : make_double2(-s3 * t3.y, s3 * t3.x);
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, t4);
    v[2] = csub(t2, t4);
  }
};

template <bool FWD> struct Dft<4, FWD> {
  static __device__ __forceinline__ void run(double2 *v) {
    double2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    double2 c = cadd(v[1], v[3]), d = mul_mi<FWD>(csub(v[1], v[3]));
    v[0] = cadd(a, c);
    v[2] = csub(a, c);
    v[1] = cadd(b, d);
    v[3] = csub(b, d);
  }
};

template <bool FWD> struct Dft<5, FWD> {
  static __device__ __forceinline__ void run(double2 *v) {
    const double c1 = 0.30901699437494742410;   // cos(2 pi / 5)
    const double c2 = -0.80901699437494742410;  // cos(4 pi / 5)
    const double s1 = 0.95105651629515357212;   // sin(2 pi / 5)
    const double s2 = 0.58778525229247312917;   // sin(4 pi / 5)
    double2 a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
    double2 a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
    double2 x0 = v[0];
    double2 r1 = make_double2(x0.x + c1 * a1.x + c2 * a2.x, x0.y + c1 * a1.y + c2 * a2.y);
    double2 r2 = make_double2(x0.x + c2 * a1.x + c1 * a2.x, x0.y + c2 * a1.y + c1 * a2.y);
    // i-parts: q=1: -i(s1 b1 + s2 b2), q=2: -i(s2 b1 - s1 b2)  (FWD)
    double2 i1 = make_double2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y);
    double2 i2 = make_double2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y);
    i1 = mul_mi<FWD>(i1);
    i2 = mul_mi<FWD>(i2);
    v[0] = cadd(x0, cadd(a1, a2));
    v[1] = cadd(r1, i1);
    v[4] = csub(r1, i1);
    v[2] = cadd(r2, i2);
    v[3] = csub(r2, i2);
  }
};

template <bool FWD> struct Dft<7, FWD> {
  static __device__ __forceinline__ void run(double2 *v) {
    const double c[3] = {0.62348980185873353053, -0.22252093395631440429, -0.90096886790241912624};
    const double s[3] = {0.78183148246802980871, 0.97492791218182360702, 0.43388373911755812048};
    double2 a[3], b[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      a[q] = cadd(v[q + 1], v[6 - q]);
      b[q] = csub(v[q + 1], v[6 - q]);
    }
    double2 x0 = v[0];
    v[0] = cadd(x0, cadd(a[0], cadd(a[1], a[2])));
#pragma unroll
    for (int q = 1; q <= 3; ++q) {
      double2 re = x0, im = make_double2(0.0, 0.0);
#pragma unroll
      for (int r = 1; r <= 3; ++r) {
        const int m = (q * r) % 7;
        const double cc = (m <= 3) ? c[m - 1] : c[7 - m - 1];
        const double ss = (m <= 3) ? s[m - 1] : -s[7 - m - 1];
        re = make_double2(fma(cc, a[r - 1].x, re.x), fma(cc, a[r - 1].y, re.y));
        im = make_double2(fma(ss, b[r - 1].x, im.x), fma(ss, b[r - 1].y, im.y));
      }
      im = mul_mi<FWD>(im);
      v[q] = cadd(re, im);
      v[7 - q] = csub(re, im);
    }
  }
};

template <bool FWD> struct Dft<8, FWD> {
  static __device__ __forceinline__ void run(double2 *v) {
    const double h = 0.70710678118654752440;
    // radix-2 split into even / odd halves, each a 4-point DFT
    double2 e[4] = {v[0], v[2], v[4], v[6]};
    double2 o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, FWD>::run(e);
    Dft<4, FWD>::run(o);
    // twiddles W8^q for q = 0..3
    double2 o1 = o[1], o3 = o[3];
    // W8 = (1 - i)/sqrt2 (FWD) ; W8^3 = (-1 - i)/sqrt2 (FWD)
    double2 t1 = FWD ? make_double2(h * (o1.x + o1.y), h * (o1.y - o1.x))
                     : make_double2(h * (o1.x - o1.y), h * (o1.y + o1.x));
    double2 t2 = mul_mi<FWD>(o[2]);
    double2 t3 = FWD ? make_double2(h * (o3.y - o3.x), -h * (o3.x + o3.y))
                     : make_double2(-h * (o3.x + o3.y), h * (o3.x - o3.y));
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], t1);
    v[5] = csub(e[1], t1);
    v[2] = cadd(e[2], t2);
    v[6] = csub(e[2], t2);
    v[3] = cadd(e[3], t3);
    v[7] = csub(e[3], t3);
  }
};

// ---------------------------------------------------------------------------
// One Stockham stage on `ncol` interleaved columns: element i of column c is
// at [i * ncol + c]. Ns = product of the radices of the earlier stages.
template <int R, bool FWD>
__device__ __forceinline__ void fft_stage(const double2 *__restrict__ in, double2 *__restrict__ out, int n,
                                          int Ns, int ncol, const double2 *__restrict__ tw, int tid, int nthr) {
  const int nbf = n / R;
  const int tws = n / (Ns * R);
  const int total = nbf * ncol;
  for (int w = tid; w < total; w += nthr) {
    const int col = w % ncol;
    const int j = w / ncol;
    const int k = j % Ns;
    double2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = in[(j + r * nbf) * ncol + col];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        double2 t = __ldg(&tw[k * r * tws]);
        if (!FWD) t.y = -t.y;
        v[r] = cmul(v[r], t);
      }
    }
    Dft<R, FWD>::run(v);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) out[(base + r * Ns) * ncol + col] = v[r];
  }
}

// Stage with an arbitrary radix R (any prime factor the fixed butterflies do
// not cover): each work item computes one output of one butterfly as a direct
// R-point sum, y_q = sum_r v_r W_n^(k r n/(Ns R)) W_R^(r q), with both roots
// read from the length-n table. Cost R complex multiply-adds per output.
template <bool FWD>
__device__ __noinline__ void fft_stage_generic(const double2 *__restrict__ in, double2 *__restrict__ out, int n,
                                               int R, int Ns, int ncol, const double2 *__restrict__ tw, int tid,
                                               int nthr) {
  const int nbf = n / R;
  const int tws = n / (Ns * R);
  const long total = (long)n * ncol;
  for (long w = tid; w < total; w += nthr) {
    const int col = (int)(w % ncol);
    const long t = w / ncol;
    const int q = (int)(t % R);
    const int j = (int)(t / R);
    const int k = j % Ns;
    double2 acc = make_double2(0.0, 0.0);
    for (int r = 0; r < R; ++r) {
      const long e = ((long)k * r * tws + (long)((r * q) % R) * nbf) % n;
      double2 root = __ldg(&tw[e]);
      if (!FWD) root.y = -root.y;
      acc = cfma(in[(j + r * nbf) * ncol + col], root, acc);
    }
    out[((j - k) * R + k + q * Ns) * ncol + col] = acc;
  }
}

// Full transform of `ncol` columns held in buffer a (b is scratch of the same
// size). Returns the buffer that holds the result. Starts and ends with a
// block-wide barrier.
template <bool FWD>
__device__ double2 *fft_smem(double2 *a, double2 *b, const FftDesc &d, int ncol) {
  __syncthreads();
  const int tid = threadIdx.x, nthr = blockDim.x;
  int Ns = 1;
  for (int s = 0; s < d.nst; ++s) {
    const int R = d.radix[s];
    switch (R) {
      case 2: fft_stage<2, FWD>(a, b, d.n, Ns, ncol, d.tw, tid, nthr); break;
      case 3: fft_stage<3, FWD>(a, b, d.n, Ns, ncol, d.tw, tid, nthr); break;
      case 4: fft_stage<4, FWD>(a, b, d.n, Ns, ncol, d.tw, tid, nthr); break;
      case 5: fft_stage<5, FWD>(a, b, d.n, Ns, ncol, d.tw, tid, nthr); break;
      case 7: fft_stage<7, FWD>(a, b, d.n, Ns, ncol, d.tw, tid, nthr); break;
      case 8: fft_stage<8, FWD>(a, b, d.n, Ns, ncol, d.tw, tid, nthr); break;
      default: fft_stage_generic<FWD>(a, b, d.n, R, Ns, ncol, d.tw, tid, nthr); break;
    }
    Ns *= R;
    double2 *t = a;
    a = b;
    b = t;
    __syncthreads();
  }
  return a;
}

}  // namespace tprf
