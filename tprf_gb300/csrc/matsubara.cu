// Kernel (b), Matsubara part, and kernel (c), the particle-hole bubble.
//
//  * Matsubara -> tau with the three-pole tail model and the tail fit:
//    restates c++/triqs_tprf/fourier/fourier_matsubara.cpp:218-308 as driven
//    per r by lattice/fourier.hpp:99-130; fermionic (fourier_wr_to_tr) and
//    bosonic (chi_tr_from_chi_wr).
//  * tau -> Matsubara with the fit_derivatives moments: restates
//    fourier_matsubara.cpp:42-97 and :123-184, driven by lattice/fourier.hpp:133-163;
//    bosonic (chi_wr_from_chi_tr, the bubble) and fermionic (fourier_tr_to_wr).
//  * bubble chi0_abcd(tau_i, r) = G_da(tau_i, r) G_bc(tau_{N-1-i}, -r):
//    restates lattice/chi_imtime.cpp:88-136 (product at :127); the fused
//    bubble + tau -> w of chi_imtime.cpp:139-182; the trapezoid branch of
//    chi_imtime.cpp:185-276.
//
// Design: every transform works on "columns" (one (r, target element) pair
// each; columns are contiguous in HBM), a tile of `ic` columns per CTA. The
// whole tau or nu series of the tile sits in shared memory, the tail moments
// are fitted in the same CTA and the Stockham FFT runs there, so each
// transform reads its input once and writes its output once. The reference
// subtracts the tail model before the FFT and adds it back after; because
// that is linear in the moments, the per-pole parts are folded into tables
// precomputed once per mesh and applied after the FFT (same result up to
// rounding, and no per-element work before the FFT). The fused bubble builds
// chi0(tau) for its columns directly in shared memory from G(tau, r) and
// G(beta - tau, -r): chi0(tau, r) never reaches HBM. The FFT and the tail
// arithmetic run in double-float pairs on the FP32 pipe by default
// (tprf_set_arithmetic), with inputs and outputs in complex128.
#include <algorithm>
#include <vector>

#include <type_traits>

#include "common.cuh"

namespace tprf {
namespace {

constexpr int kMatsubaraThreads = 256;  // columns per CTA (<= 32) divide it
constexpr int kMidBatch = 12;            // row loads per thread in flight (load phases)
constexpr int kEpiBatch = 2;             // iv -> tau output rows whose tables are read together

struct VinvRows {
  double r0[8];  // row 0 of the inverse Vandermonde: first derivative
  double r1[8];  // row 1: second-order coefficient
};

VinvRows make_vinv_rows() {
  VinvRows r;
  fit_derivative_rows(r.r0, r.r1);
  return r;
}

// fit_derivatives with the divisions folded into constants: the moments need
// sum_m r[m] (g[m] - g[0]) / tau_m, computed as sum_m (r[m] / tau_m) (g[m] - g[0])
// (the same algebra; FP64 divisions are slow on this GPU), and m3 carries -2 / dtau.
struct FitRows {
  double c0[8], c1[8];
  double k3;
};

FitRows make_fit_rows(double beta, int n_tau) {
  double r0[8], r1[8];
  fit_derivative_rows(r0, r1);
  const double dtau = beta / (double)(n_tau - 1);
  FitRows f;
  for (int m = 0; m < 8; ++m) {
    const double tau = (double)(m + 1) * dtau;
    f.c0[m] = r0[m] / tau;
    f.c1[m] = r1[m] / tau;
  }
  f.k3 = -2.0 / dtau;
  return f;
}

// element-type plumbing: double2 (FP64) or cdf (double-float)
template <class C> struct IsDfElem { static constexpr bool value = false; };
template <> struct IsDfElem<cdf> { static constexpr bool value = true; };
template <class C> __device__ __forceinline__ C from_d2(double2 z);
template <> __device__ __forceinline__ double2 from_d2<double2>(double2 z) { return z; }
__device__ __forceinline__ double2 hi_parts(double2 z) { return z; }
__device__ __forceinline__ double2 hi_parts(cdf z) { return make_double2(z.x.hi, z.y.hi); }
__device__ __forceinline__ double2 conj_el(double2 z) { return cconj(z); }
__device__ __forceinline__ cdf conj_el(cdf z) { return cconj(z); }
__device__ __forceinline__ double2 half_el(double2 z) { return make_double2(0.5 * z.x, 0.5 * z.y); }
__device__ __forceinline__ cdf half_el(cdf z) {  // exact: scales both words by 1/2
  return cdf{dfl{0.5f * z.x.hi, 0.5f * z.x.lo}, dfl{0.5f * z.y.hi, 0.5f * z.y.lo}};
}
template <> __device__ __forceinline__ cdf from_d2<cdf>(double2 z) { return to_cdf(z); }
__device__ __forceinline__ double2 as_d2(double2 z) { return z; }
__device__ __forceinline__ double2 as_d2(cdf z) { return to_double2(z); }
template <class C> __device__ __forceinline__ C table(const double2 *d, const float4 *f, long i);
template <> __device__ __forceinline__ double2 table<double2>(const double2 *d, const float4 *, long i) { return d[i]; }
template <> __device__ __forceinline__ cdf table<cdf>(const double2 *, const float4 *f, long i) {
  const float4 v = f[i];
  return cdf{dfl{v.x, v.y}, dfl{v.z, v.w}};
}
template <class C> __device__ __forceinline__ typename RealT<C>::type real_of(double v);
template <> __device__ __forceinline__ double real_of<double2>(double v) { return v; }
template <> __device__ __forceinline__ dfl real_of<cdf>(double v) { return split_double(v); }

// The three-pole tail amplitudes a_j from the moments m1..m3
// (fourier_matsubara.cpp:156-171 and 268-284): fermion b = (0, 1, -1),
// a = (m1-m3, (m2+m3)/2, (m3-m2)/2); boson b = (-1/2, -1, 1),
// a = (4(m1-m3)/3, m3-(m1+m2)/2, m1/6+m2/2+m3/3). am[3] keeps m1.
template <class C>
__device__ __forceinline__ void tail_amplitudes(int fermion, double2 m1, double2 m2, double2 m3, C *am, int ic,
                                                int c) {
  if (fermion) {
    am[0 * ic + c] = from_d2<C>(csub(m1, m3));
    am[1 * ic + c] = from_d2<C>(cscale(cadd(m2, m3), 0.5));
    am[2 * ic + c] = from_d2<C>(cscale(csub(m3, m2), 0.5));
  } else {
    am[0 * ic + c] = from_d2<C>(cscale(csub(m1, m3), 4.0 / 3.0));
    am[1 * ic + c] = from_d2<C>(csub(m3, cscale(cadd(m1, m2), 0.5)));
    am[2 * ic + c] = from_d2<C>(cadd(cadd(cscale(m1, 1.0 / 6.0), cscale(m2, 0.5)), cscale(m3, 1.0 / 3.0)));
  }
  am[3 * ic + c] = from_d2<C>(m1);
}

// ---------------------------------------------------------------------------
// Matsubara -> tau. The tail model enters after the FFT through the folded
// tables (exactly the reference's model subtracted before and added after the
// FFT, by linearity): G(tau_t) = P[t] FFT(g)[t] + sum_j a_j Q[j][t].

template <class C>
__global__ void __launch_bounds__(kMatsubaraThreads, 2) nu_to_tau_kernel(NuTauPlan p, const double2 *__restrict__ gw,
                                                        const double2 *__restrict__ mom, double2 *__restrict__ gt,
                                                        long Ccols, int ic, int lg, unsigned *status,
                                                        cdf *__restrict__ gt_df, unsigned *gmax,
                                                        const unsigned *hwords, int fit_rows_only,
                                                        const int2 *__restrict__ tpairs, long n_can) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned s_res;
  C *a = reinterpret_cast<C *>(smem_raw);
  const int L = p.L, nnu = p.n_in;
  const int *rev = p.fft.rev;
  C *b = p.fft.has_generic ? a + (size_t)L * ic : nullptr;
  C *am = a + (size_t)(p.fft.has_generic ? 2 : 1) * L * ic;  // [4][ic]: a1, a2, a3, m1; then the fit coefficients
  const int tid = threadIdx.x, nthr = blockDim.x;
  // Real pairs (double-float path, hwords saying G(iv, r) is Hermitian in iv,
  // so G(tau, r) is real): two columns g1, g2 go through one transform as
  // z = g1 + i g2 and G1(tau) = Re T(z), G2(tau) = Im T(z) (T is complex-linear;
  // the fit coefficients and tail moments of such data are real). Column c of
  // the CTA is then the pair of real columns 2 (col0 + c) and 2 (col0 + c) + 1.
  // Transposition partners (real pairs with hwords saying G(iv, -r) =
  // G(iv, r)^T, and the rank-2 pairs given): the units run over the canonical
  // columns only, the f-th real column being tpairs[f].x, and each result is
  // stored at that column and at its partner tpairs[f].y.
  bool pairs = false, canon = false;
  if constexpr (IsDfElem<C>::value) {
    if (hwords != nullptr && status != nullptr && blockIdx.x == 0 && tid == 0) {
      const float gm = __uint_as_float(hwords[0]);  // max |G(iv, r)|; inf when beyond FP32
      if (!(gm <= kDfGMax) || (gm > 0.f && gm < kDfGMin)) atomicOr(status, kDevErrRange);
    }
    pairs = hermitian_says_yes(hwords);
    canon = pairs && tpairs != nullptr && transpose_says_yes(hwords);
  }
  const long n_real = canon ? n_can : Ccols;  // real columns to transform
  const long n_units = pairs ? (n_real + 1) / 2 : n_real;
  const long col0 = blockIdx.x * (long)ic;
  if (col0 >= n_units) return;  // the rest of the grid in pair mode
  const int ncol = (int)min((long)ic, n_units - col0);
  __shared__ int s_col[64], s_par[64];  // canonical mode: the CTA's real columns and partners (ic <= 32)
  if (canon)
    for (int k = tid; k < 2 * ic; k += nthr) {
      const long f = 2 * col0 + k;
      const int2 cp = f < n_real ? tpairs[f] : make_int2(0, 0);
      s_col[k] = cp.x;
      s_par[k] = cp.y;
    }
  __syncthreads();
  // memory column of real column f of this CTA (f in [2 col0, 2 col0 + 2 ic))
  auto rcol = [&](long f) -> long { return canon ? (long)s_col[f - 2 * col0] : f; };
  // input of unit c at frequency row n: the column, or z of the pair
  auto in_at = [&](long n, int c) -> double2 {
    if (!pairs) return gw[n * Ccols + col0 + c];
    const long f = 2 * (col0 + c);
    const double2 g1 = gw[n * Ccols + rcol(f)];
    const double2 g2 = f + 1 < n_real ? gw[n * Ccols + rcol(f + 1)] : make_double2(0.0, 0.0);
    return make_double2(g1.x - g2.y, g1.y + g2.x);
  };

  for (int w = tid; w < L * ic; w += nthr) a[w] = czero<C>();
  if (tid == 0) s_res = 0u;
  __syncthreads();
  // frequency n sits at FFT row (n + L) % L, stored at its digit-reversed
  // position; kMidBatch loads per thread are in flight before the first is stored
  for (int w0 = tid; w0 < nnu * ic; w0 += kMidBatch * nthr) {
    double2 v[kMidBatch];
#pragma unroll
    for (int u = 0; u < kMidBatch; ++u) {
      const int w = w0 + u * nthr;
      const int c = w & (ic - 1), n = w >> lg;
      if (w < nnu * ic && c < ncol) v[u] = in_at(n, c);
    }
#pragma unroll
    for (int u = 0; u < kMidBatch; ++u) {
      const int w = w0 + u * nthr;
      const int c = w & (ic - 1), n = w >> lg;
      if (w < nnu * ic && c < ncol) a[rev[(n + p.in0 + L) % L] * ic + c] = from_d2<C>(v[u]);
    }
  }
  __syncthreads();
  if (mom == nullptr) {
    // The least-squares fit is ill-conditioned for short meshes, so it runs in
    // FP64 on the original complex128 data (not on the double-float copy).
    const int nf = p.n_fit, nm = p.n_mom;
    double2 *coef = reinterpret_cast<double2 *>(am + 4 * ic);  // [n_mom <= 10][ic]
    for (int w = tid; w < nm * ic; w += nthr) {
      const int c = w & (ic - 1), q = w >> lg;
      double2 acc = make_double2(0.0, 0.0);
      if (c < ncol)
        for (int i = 0; i < nf; ++i) acc = cfma(p.fitF[q * nf + i], in_at(p.fit_row[i], c), acc);
      coef[q * ic + c] = acc;
    }
    __syncthreads();
    for (int w = tid; w < nf * ic; w += nthr) {
      const int c = w & (ic - 1), i = w >> lg;
      if (c >= ncol) continue;
      if (!pairs) {
        double2 model = make_double2(0.0, 0.0);
        for (int q = 0; q < nm; ++q) model = cfma(p.fitG[i * nm + q], coef[q * ic + c], model);
        const double2 d = csub(model, gw[(long)p.fit_row[i] * Ccols + col0 + c]);
        atomicMax(&s_res, __float_as_uint(sqrtf((float)cabs2(d))));  // compared with 1e-3
      } else {
        // each real column of the pair against its own model (real and imaginary
        // parts of the pair's coefficients)
        const long f = 2 * (col0 + c);
        for (int h = 0; h < 2 && f + h < n_real; ++h) {
          double2 model = make_double2(0.0, 0.0);
          for (int q = 0; q < nm; ++q) {
            const double2 cq = coef[q * ic + c];
            model = cfma(p.fitG[i * nm + q], make_double2(h ? cq.y : cq.x, 0.0), model);
          }
          const double2 d = csub(model, gw[(long)p.fit_row[i] * Ccols + rcol(f + h)]);
          atomicMax(&s_res, __float_as_uint(sqrtf((float)cabs2(d))));
        }
      }
    }
    for (int c = tid; c < ic; c += nthr)
      tail_amplitudes(p.fermion, coef[1 * ic + c], coef[2 * ic + c], coef[3 * ic + c], am, ic, c);
  } else {
    for (int c = tid; c < ic; c += nthr) {
      double2 m1 = make_double2(0.0, 0.0), m2 = m1, m3 = m1;
      if (c < ncol && !pairs) {
        m1 = mom[0 * Ccols + col0 + c];
        m2 = mom[1 * Ccols + col0 + c];
        m3 = mom[2 * Ccols + col0 + c];
      } else if (c < ncol) {  // z = g1 + i g2: moments likewise
        const long f = 2 * (col0 + c);
        const bool two = f + 1 < n_real;
        auto zm = [&](int q) {
          const double2 a1 = mom[q * Ccols + rcol(f)], a2 = two ? mom[q * Ccols + rcol(f + 1)] : make_double2(0.0, 0.0);
          return make_double2(a1.x - a2.y, a1.y + a2.x);
        };
        m1 = zm(0);
        m2 = zm(1);
        m3 = zm(2);
      }
      tail_amplitudes(p.fermion, m1, m2, m3, am, ic, c);
    }
  }
  __syncthreads();
  if (tid == 0 && __uint_as_float(s_res) > 1e-3f) atomicOr(status, kDevErrTailFit);
  C *r = fft_smem<true>(a, b, p.fft, ic);
  float g_abs = 0.f, g_im = 0.f;
  // the phase and tail tables (larger than what L1 keeps beside the FFT
  // buffers) of kEpiBatch iterations are read before any is used
  const int n_out = (L + 1) * ic;
  for (int w0 = tid; w0 < n_out; w0 += kEpiBatch * nthr) {
    C tp[kEpiBatch], tq[kEpiBatch][3];
#pragma unroll
    for (int u = 0; u < kEpiBatch; ++u) {
      const int w = w0 + u * nthr, t = w >> lg;
      const int tt = (t < L) ? t : 0;
      if (w < n_out) {
        tp[u] = table<C>(p.P, p.Pf, tt);
#pragma unroll
        for (int j = 0; j < 3; ++j) tq[u][j] = table<C>(p.Q, p.Qf, (long)j * L + tt);
      }
    }
#pragma unroll
    for (int u = 0; u < kEpiBatch; ++u) {
      const int w = w0 + u * nthr;
      if (w >= n_out) break;
      const int c = w & (ic - 1), t = w >> lg;
      if (c >= ncol) continue;
      const int tt = (t < L) ? t : 0;
      C v = cmul(tp[u], r[tt * ic + c]);
#pragma unroll
      for (int j = 0; j < 3; ++j) v = cadd(v, cmul(am[j * ic + c], tq[u][j]));
      // G[L] = -(G[0] + m1) for fermions, +(G[0] + m1) for bosons
      if (t == L) v = p.fermion ? csub(czero<C>(), cadd(v, am[3 * ic + c])) : cadd(v, am[3 * ic + c]);
      if (pairs) {
        if constexpr (IsDfElem<C>::value) {
          // real results: the double-float copy keeps the real parts only (dfl,
          // 8 bytes), the complex128 copy all rows or the fit rows only
          const long f = 2 * (col0 + c);
          const bool keep = !fit_rows_only || t <= 8 || t >= L - 8;
          dfl *gre = reinterpret_cast<dfl *>(gt_df);
          // real column f + h gets x, and in the canonical mode its partner too
          auto put = [&](long fh, dfl x) {
            const long col = rcol(fh);
            if (keep) gt[(long)t * Ccols + col] = as_d2(cdf{x, dfl{0.f, 0.f}});
            if (gt_df) gre[(long)t * Ccols + col] = x;
            if (canon) {
              const long pc = s_par[fh - 2 * col0];
              if (pc != col) {
                if (keep) gt[(long)t * Ccols + pc] = as_d2(cdf{x, dfl{0.f, 0.f}});
                if (gt_df) gre[(long)t * Ccols + pc] = x;
              }
            }
          };
          put(f, v.x);
          if (f + 1 < n_real) put(f + 1, v.y);
          if (gmax) g_abs = fmaxf(g_abs, fmaxf(fabsf(v.x.hi), fabsf(v.y.hi)));  // both parts are real columns
        }
        continue;
      }
      gt[(long)t * Ccols + col0 + c] = as_d2(v);
      if constexpr (IsDfElem<C>::value) {
        if (gt_df) gt_df[(long)t * Ccols + col0 + c] = v;  // the value before rounding to complex128
      }
      if (gmax) {
        const double2 h = hi_parts(v);
        g_abs = fmaxf(g_abs, fmaxf(fabsf((float)h.x), fabsf((float)h.y)));
        g_im = fmaxf(g_im, fabsf((float)h.y));
      }
    }
  }
  // max |G| and max |Im G| of the whole transform, for the real-pair bubble
  if (gmax) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      g_abs = fmaxf(g_abs, __shfl_xor_sync(0xffffffffu, g_abs, o));
      g_im = fmaxf(g_im, __shfl_xor_sync(0xffffffffu, g_im, o));
    }
    if ((tid & 31) == 0) {
      atomicMax(gmax, __float_as_uint(g_abs));
      atomicMax(gmax + 1, __float_as_uint(g_im));
    }
  }
}

// ---------------------------------------------------------------------------
// Column loaders for the tau -> w transform and the trapezoid integral.

struct ArrayLoader {  // chi(tau, col) stored as [n_tau][C]
  const double2 *x;
  long C;
  __device__ __forceinline__ double2 operator()(int t, long col) const { return x[(long)t * C + col]; }
  __device__ __forceinline__ void setup(long, int, int, long *) const {}
  template <class E>
  __device__ __forceinline__ E get(int t, int c, long col0, int, const long *) const {
    return from_d2<E>(x[(long)t * C + col0 + c]);
  }
  __device__ __forceinline__ double2 get64(int t, int c, long col0, int, const long *) const {
    return x[(long)t * C + col0 + c];
  }
};

struct BubbleLoader {  // chi0 columns computed from G(tau, r): col = r * nb^4 + abcd
  const double2 *g;    // [n_tau][N_r][nb][nb]
  long Nr;
  int nb, n_tau;
  int d0, d1, d2;
  // offsets of G_da(., r) and G_bc(., -r) within one tau slice of G
  // 32-bit index arithmetic: N_r nb^4 < 2^31 is checked at launch (bubble_columns)
  __device__ __forceinline__ void offsets(long col, long &ox, long &oy) const {
    const int nb2 = nb * nb, nb4 = nb2 * nb2;
    const int ci = (int)col;
    const int r = ci / nb4;
    int e = ci - r * nb4;
    const int d = e % nb;
    e /= nb;
    const int c = e % nb;
    e /= nb;
    const int b = e % nb;
    const int a = e / nb;
    const int i2 = r % d2;
    const int i1 = (r / d2) % d1;
    const int i0 = r / (d2 * d1);
    const long mr = ((long)((d0 - i0) % d0) * d1 + (d1 - i1) % d1) * d2 + (d2 - i2) % d2;
    ox = (long)r * nb2 + d * nb + a;
    oy = mr * nb2 + b * nb + c;
  }
  __device__ __forceinline__ double2 operator()(int t, long col) const {
    long ox, oy;
    offsets(col, ox, oy);
    const long slice = Nr * nb * nb;
    return cmul(g[(long)t * slice + ox], g[(long)(n_tau - 1 - t) * slice + oy]);
  }
  // per CTA: the two offsets of each of its ic columns, once
  __device__ __forceinline__ void setup(long col0, int ic, int ncol, long *s) const {
    for (int c = threadIdx.x; c < ic; c += blockDim.x) {
      long ox = 0, oy = 0;
      if (c < ncol) offsets(col0 + c, ox, oy);
      s[c] = ox;
      s[ic + c] = oy;
    }
  }
  // the product in FP64, then one conversion (two would cost more than the product)
  template <class E>
  __device__ __forceinline__ E get(int t, int c, long col0, int ic, const long *s) const {
    return from_d2<E>(get64(t, c, col0, ic, s));
  }
  __device__ __forceinline__ double2 get64(int t, int c, long, int ic, const long *s) const {
    const long slice = Nr * nb * nb;
    return cmul(g[(long)t * slice + s[c]], g[(long)(n_tau - 1 - t) * slice + s[ic + c]]);
  }
};

// Gathered reads of the double-float copy of G(tau, r) as single 8- and
// 16-byte loads (dfl itself is only 4-byte aligned).
__device__ __forceinline__ cdf ld_cdf(const cdf *p, long i) { return p[i]; }
__device__ __forceinline__ dfl ld_dfl(const void *p, long i) {  // 8 bytes at element i of dfl[] p
  const float2 v = reinterpret_cast<const float2 *>(p)[i];
  return dfl{v.x, v.y};
}
__device__ __forceinline__ dfl ld_re(const cdf *p, long i) {  // the real part of element i of cdf[] p
  const float2 v = reinterpret_cast<const float2 *>(p)[2 * i];
  return dfl{v.x, v.y};
}

// The fused bubble with a double-float copy of G(tau, r) beside the complex128
// one: the FFT input is the double-float product of the copies (FP32 pipe, no
// conversion), and only the rows fit_derivatives samples take the FP64
// product of the complex128 values (get64).
struct BubbleLoaderDF : BubbleLoader {
  const cdf *gdf;
  template <class E>
  __device__ __forceinline__ E get(int t, int c, long col0, int ic, const long *s) const {
    if constexpr (IsDfElem<E>::value) {
      const long slice = Nr * nb * nb;
      return cmul(ld_cdf(gdf, (long)t * slice + s[c]), ld_cdf(gdf, (long)(n_tau - 1 - t) * slice + s[ic + c]));
    } else {
      return get64(t, c, col0, ic, s);
    }
  }
};

// Real pairs. When G(tau, r) is real (Hermitian hoppings that are real in
// real space: the iv -> tau pass records max |G| and max |Im G| in gmax and
// the data count as real when the second is at most 1e-11 of the first: the
// transforms leave an imaginary residue of about 1e-12 on a real G, and 1e-11
// is a tenth of the 1e-10 accuracy bar of the path), every
// bubble column chi0(tau) is real, and two of them, f and h, go through one
// complex transform as z = f + i h. The tau -> i omega map T is complex-linear
// and T(f)(-m) = conj(T(f)(m)) for real f, so T(f)(m) = (T(z)(m) + conj(T(z)(-m)))/2
// and T(h)(m) = (T(z)(m) - conj(T(z)(-m)))/(2i): half the transforms. The
// moments of z are the moments of f plus i times those of h (the fit is
// linear with real coefficients), so the tail works unchanged on z. The
// imaginary parts of G (rounding residue, below the bound) are dropped.

// Transposition partners: when iv -> tau also ran on canonical columns (its
// words say G(iv, -r) = G(iv, r)^T, and G(tau, -r) = G(tau, r)^T then holds bit
// for bit), chi0(tau, -r)_dcba = G_ad(tau, -r) G_cb(beta - tau, r) is the same
// product, in the same order, as chi0(tau, r)_abcd = G_da(tau, r) G_bc(beta - tau,
// -r): the columns (r, abcd) and (-r, dcba) are equal, and only the canonical one
// of each pair (tpairs, rank 4) is transformed, its result stored at both.
struct BubblePairLoaderDF : BubbleLoaderDF {
  // the five words of the chain: [max |G|, max |Im G|] of G(tau, r), then the
  // Hermitian and transposition words of G(iv, r), as float bits; null: no pairs
  const unsigned *gmax;
  const int2 *tpairs = nullptr;  // rank-4 transposition pairs (nullable)
  long n_can = 0;
  bool pairs = false;
  bool compact = false;  // gdf holds real parts only (dfl per element): iv -> tau ran on real pairs
  bool canon = false;    // transform the canonical columns of tpairs only
  // canonical orbital output (CompactChi): in the canonical mode each result
  // goes to cout[w][r][ocomp[o]] for whichever of its column (r, o) and partner
  // is a canonical orbital column (both when o is a palindrome), rows w >= 0
  cdf *cout = nullptr;
  const int *ocomp = nullptr;
  int nc = 0;
  __device__ __forceinline__ void init() {
    pairs = gmax_says_real(gmax);
    compact = pairs && hermitian_says_yes(gmax + 2);
    canon = compact && tpairs != nullptr && transpose_says_yes(gmax + 2);
  }
  __device__ __forceinline__ long real_cols() const { return canon ? n_can : Nr * nb * nb * nb * nb; }
  __device__ __forceinline__ long real_col(long f) const { return canon ? (long)tpairs[f].x : f; }
  // offsets of the two real columns 2 (col0 + c) and 2 (col0 + c) + 1 (the
  // second past the last column reads the first: its results are not stored)
  __device__ __forceinline__ void setup(long col0, int ic, int ncol, long *s) const {
    if (!pairs) return BubbleLoader::setup(col0, ic, ncol, s);
    const long nreal = real_cols();
    for (int c = threadIdx.x; c < ic; c += blockDim.x) {
      long o[4] = {0, 0, 0, 0};
      if (c < ncol) {
        const long f = 2 * (col0 + c);
        offsets(real_col(f), o[0], o[1]);
        offsets(real_col(f + 1 < nreal ? f + 1 : f), o[2], o[3]);
      }
      for (int q = 0; q < 4; ++q) s[q * ic + c] = o[q];
    }
  }
  template <class E>
  __device__ __forceinline__ E get(int t, int c, long col0, int ic, const long *s) const {
    if (!pairs) return BubbleLoaderDF::template get<E>(t, c, col0, ic, s);
    if constexpr (IsDfElem<E>::value) {
      const long slice = Nr * nb * nb, t1 = (long)t * slice, t2 = (long)(n_tau - 1 - t) * slice;
      if (compact)
        return cdf{dmul(ld_dfl(gdf, t1 + s[c]), ld_dfl(gdf, t2 + s[ic + c])),
                   dmul(ld_dfl(gdf, t1 + s[2 * ic + c]), ld_dfl(gdf, t2 + s[3 * ic + c]))};
      return cdf{dmul(ld_re(gdf, t1 + s[c]), ld_re(gdf, t2 + s[ic + c])),
                 dmul(ld_re(gdf, t1 + s[2 * ic + c]), ld_re(gdf, t2 + s[3 * ic + c]))};
    } else {
      return get64(t, c, col0, ic, s);
    }
  }
  __device__ __forceinline__ double2 get64(int t, int c, long col0, int ic, const long *s) const {
    if (!pairs) return BubbleLoader::get64(t, c, col0, ic, s);
    const long slice = Nr * nb * nb, t1 = (long)t * slice, t2 = (long)(n_tau - 1 - t) * slice;
    return make_double2(g[t1 + s[c]].x * g[t2 + s[ic + c]].x, g[t1 + s[2 * ic + c]].x * g[t2 + s[3 * ic + c]].x);
  }
};
template <class L> struct HasPairs { static constexpr bool value = false; };
template <> struct HasPairs<BubblePairLoaderDF> { static constexpr bool value = true; };

// tau -> i omega. fit_derivatives moments in FP64 from the end rows; the tail
// model enters after the FFT: chi(i w_m) = (beta/L) FFT(chi)[k_m] + sum_j a_j K[j][m].
// FERM: the fermionic transform (input phase, fermion moments); a template
// parameter so that the bosonic bubble path carries no branch for it.
template <class Loader, class C, bool FERM>
__global__ void __launch_bounds__(kMatsubaraThreads, 2) tau_to_w_kernel(TauWPlan p, Loader ld_in, FitRows fr, double2 *__restrict__ out,
                                                       long Ccols, int ic, int lg, int out_df, int skip_neg) {
  Loader ld = ld_in;
  bool pairs = false;  // real pairs (BubblePairLoaderDF on real input): Ccols real columns, half as many FFT columns
  bool canon = false;  // and only the canonical columns of the transposition pairs
  long n_real = Ccols;
  if constexpr (HasPairs<Loader>::value) {
    ld.init();
    pairs = ld.pairs;
    canon = ld.canon;
    n_real = ld.real_cols();
  }
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *a = reinterpret_cast<C *>(smem_raw);
  const int L = p.L, nwt = p.n_out;
  const int *rev = p.fft.rev;
  C *b = p.fft.has_generic ? a + (size_t)L * ic : nullptr;
  C *last = a + (size_t)(p.fft.has_generic ? 2 : 1) * L * ic;  // [ic] row L
  C *am = last + ic;                                            // [4][ic] a1, a2, a3, m1
  long *soff = reinterpret_cast<long *>(am + 4 * ic);           // [4][ic] loader offsets
  double2 *smp = reinterpret_cast<double2 *>(soff + 4 * ic);    // [18][ic] FP64 rows 0..8, L-8..L
  const int tid = threadIdx.x, nthr = blockDim.x;
  const long n_fft_cols = pairs ? (n_real + 1) / 2 : Ccols;
  const long col0 = blockIdx.x * (long)ic;
  if (col0 >= n_fft_cols) return;  // the rest of the grid in pair mode
  const int ncol = (int)min((long)ic, n_fft_cols - col0);
  ld.setup(col0, ic, ncol, soff);
  __shared__ int s_tcol[64], s_tpar[64];  // canonical mode: the CTA's real columns and partners (ic <= 32)
  bool corb = false;  // canonical orbital output: s_tcol / s_tpar hold compact offsets r nc + j (or -1)
  if constexpr (HasPairs<Loader>::value) {
    corb = canon && ld.cout != nullptr;
    if (canon)
      for (int k = tid; k < 2 * ic; k += nthr) {
        const long f = 2 * col0 + k;
        const int2 cp = f < n_real ? ld.tpairs[f] : make_int2(0, 0);
        if (corb) {
          const int nb4 = ld.nb * ld.nb * ld.nb * ld.nb;
          auto dst = [&](int col) {
            const int r = col / nb4, j = ld.ocomp[col - r * nb4];
            return j >= 0 ? r * ld.nc + j : -1;
          };
          s_tcol[k] = dst(cp.x);
          s_tpar[k] = cp.y != cp.x ? dst(cp.y) : -1;
        } else {
          s_tcol[k] = cp.x;
          s_tpar[k] = cp.y;
        }
      }
  }
  __syncthreads();
  // Rows t < L go to their digit-reversed FFT positions, row L aside. The loads
  // of several iterations are issued before any is used (their latency
  // overlaps), and the FP64 values of the 18 rows that fit_derivatives samples
  // are kept. The bosonic transform loads its rows 9 .. L-9 through the
  // element type (eight iterations in flight), then the 18 sampled rows in FP64.
  if constexpr (!FERM) {
    const int mid0 = 9 * ic, mid = (L - 17) * ic;
    for (int w0 = tid; w0 < mid; w0 += kMidBatch * nthr) {
      C e[kMidBatch];
#pragma unroll
      for (int u = 0; u < kMidBatch; ++u) {
        const int w = mid0 + w0 + u * nthr;
        const int c = w & (ic - 1), t = w >> lg;
        e[u] = (w0 + u * nthr < mid && c < ncol) ? ld.template get<C>(t, c, col0, ic, soff) : czero<C>();
      }
#pragma unroll
      for (int u = 0; u < kMidBatch; ++u) {
        const int w = mid0 + w0 + u * nthr;
        if (w0 + u * nthr < mid) a[rev[w >> lg] * ic + (w & (ic - 1))] = e[u];
      }
    }
    // sampled row q: t = q for q <= 8, t = L - 17 + q (L - 8 .. L) for q >= 9
    for (int w = tid; w < 18 * ic; w += nthr) {
      const int c = w & (ic - 1), q = w >> lg;
      const int t = q <= 8 ? q : L - 17 + q;
      const double2 v = c < ncol ? ld.get64(t, c, col0, ic, soff) : make_double2(0.0, 0.0);
      smp[q * ic + c] = v;
      if (t < L)
        a[rev[t] * ic + c] = from_d2<C>(v);
      else
        last[c] = from_d2<C>(v);
    }
  }
  const int total = FERM ? (L + 1) * ic : 0;
  for (int w0 = tid; w0 < total; w0 += 4 * nthr) {
    double2 v[4];
    C e[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int w = w0 + u * nthr;
      const int c = w & (ic - 1), t = w >> lg;
      const bool live = w < total && c < ncol;
      // the sampled rows (and every row of the fermionic transform) in FP64
      const bool in64 = FERM || t <= 8 || t >= L - 8;
      v[u] = (live && in64) ? ld.get64(t, c, col0, ic, soff) : make_double2(0.0, 0.0);
      e[u] = (live && !in64) ? ld.template get<C>(t, c, col0, ic, soff) : czero<C>();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int w = w0 + u * nthr;
      if (w < total) {
        const int c = w & (ic - 1), t = w >> lg;
        const bool in64 = FERM || t <= 8 || t >= L - 8;
        if (t <= 8) smp[t * ic + c] = v[u];
        if (t >= L - 8) smp[(t - L + 17) * ic + c] = v[u];
        // the fermionic transform takes exp(i pi tau / beta) g(tau) (fourier_matsubara.cpp:164)
        const C x = in64 ? from_d2<C>(FERM && t < L ? cmul(v[u], p.ph[t]) : v[u]) : e[u];
        if (t < L)
          a[rev[t] * ic + c] = x;
        else
          last[c] = x;
      }
    }
  }
  __syncthreads();
  // fit_derivatives differentiates and then applies the inverse Vandermonde
  // matrix, which amplifies rounding: its 18 samples are the FP64 values, not
  // the double-float copy in the FFT buffer.
  // The four 8-term sums of a column (gl0, gl1, gr0, gr1) run on four adjacent
  // lanes and meet by shuffles: 4 ic lanes work instead of ic, and no barrier
  // is added (the FFT's own barrier orders am before the epilogue).
  if (tid < ((4 * ic + 31) & ~31)) {
    const int c = tid >> 2, q = tid & 3;
    const int cc = c < ic ? c : 0;  // lanes past the tile read column 0 and store nothing
    const double2 g0 = smp[cc], gL = smp[17 * ic + cc];
    double2 sum = make_double2(0.0, 0.0);
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const double w = (q & 1) ? fr.c1[m] : fr.c0[m];
      const double2 x = smp[(q < 2 ? m + 1 : 16 - m) * ic + cc];
      const double2 d = q < 2 ? make_double2(x.x - g0.x, x.y - g0.y) : make_double2(gL.x - x.x, gL.y - x.y);
      sum = make_double2(fma(w, d.x, sum.x), fma(w, d.y, sum.y));
    }
    const int l0 = (tid & 31) & ~3;
    const double2 gl0 = make_double2(__shfl_sync(0xffffffffu, sum.x, l0), __shfl_sync(0xffffffffu, sum.y, l0));
    const double2 gl1 = make_double2(__shfl_sync(0xffffffffu, sum.x, l0 + 1), __shfl_sync(0xffffffffu, sum.y, l0 + 1));
    const double2 gr0 = make_double2(__shfl_sync(0xffffffffu, sum.x, l0 + 2), __shfl_sync(0xffffffffu, sum.y, l0 + 2));
    const double2 gr1 = make_double2(__shfl_sync(0xffffffffu, sum.x, l0 + 3), __shfl_sync(0xffffffffu, sum.y, l0 + 3));
    if (q == 0 && c < ic && c >= ncol) am[c] = am[ic + c] = am[2 * ic + c] = czero<C>();
    if (q == 0 && c < ncol) {
      // m1 = -(g[0] -+ g[L]); m2 = gl0 - s gr0; m3 = -(gl1 + s gr1) 2 / dtau with
      // s = +1 (boson), -1 (fermion) (fourier_matsubara.cpp:87-90, 153, 166)
      double2 m1, m2, m3;
      if (FERM) {
        m1 = make_double2(-(g0.x + gL.x), -(g0.y + gL.y));
        m2 = cadd(gl0, gr0);
        m3 = cscale(csub(gl1, gr1), fr.k3);
      } else {
        m1 = make_double2(-(g0.x - gL.x), -(g0.y - gL.y));
        m2 = csub(gl0, gr0);
        m3 = cscale(cadd(gl1, gr1), fr.k3);
      }
      tail_amplitudes(FERM, m1, m2, m3, am, ic, c);
    }
  }
  // all stages but the last; the last is evaluated only at the kept frequencies
  C *r = fft_smem<false>(a, b, p.fft, ic, p.fft.nst - 1);
  const auto fact = real_of<C>(p.beta / (double)L);
  auto value = [&](int c, int mi) {  // T(column c) at output mi: FFT term and tail
    const int m = mi + p.out0;
    C v = cscale(last_stage_output<false>(r, p.fft, ic, c, m < 0 ? m + L : m), fact);
#pragma unroll
    for (int j = 0; j < 3; ++j) v = cadd(v, cmul(am[j * ic + c], table<C>(p.K, p.Kf, (long)j * nwt + mi)));
    return v;
  };
  auto store = [&](long idx, C v) {  // complex128, or the element type itself for a following double-float pass
    if (out_df)
      reinterpret_cast<C *>(out)[idx] = v;
    else
      out[idx] = as_d2(v);
  };
  if constexpr (HasPairs<Loader>::value && !FERM) {
    if (pairs) {
      // bosonic outputs m = -(nw-1) .. nw-1 at mi = m + nw - 1: the pair (m, -m)
      // from T(z)(m) and T(z)(-m); column 2q gets F, column 2q + 1 gets H
      const int nw = (nwt + 1) / 2;
      for (int w = tid; w < nw * ic; w += nthr) {
        const int c = w & (ic - 1), mh = w >> lg;
        if (c >= ncol) continue;
        const int mp = nw - 1 + mh, mn = nw - 1 - mh;
        // F = (T(z)(m) + conj(T(z)(-m))) / 2 and H = (T(z)(m) - conj(T(z)(-m))) / (2 i),
        // the FFT terms as such; in the tail, a_j = a_j(f) + i a_j(h) with real
        // a_j(f), a_j(h) (the fit is linear with real coefficients) and
        // K_j(-m) = conj(K_j(m)) (the transform of a real one-pole function), so
        // F takes a_j(f) K_j(m) and H takes a_j(h) K_j(m)
        auto fft_term = [&](int mi) {
          const int m = mi + p.out0;
          return cscale(last_stage_output<false>(r, p.fft, ic, c, m < 0 ? m + L : m), fact);
        };
        const C vp = fft_term(mp), vn = conj_el(fft_term(mn));
        C F = half_el(cadd(vp, vn));
        C H = mul_mi<true>(half_el(csub(vp, vn)));
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const C k = table<C>(p.K, p.Kf, (long)j * nwt + mp), a = am[j * ic + c];
          F = cadd(F, cscale(k, a.x));
          H = cadd(H, cscale(k, a.y));
        }
        const long f = 2 * (col0 + c);
        // the negative frequencies only when the caller does not fill them by symmetry
        const bool neg = mh > 0 && !skip_neg;
        // real column fh gets val (its memory column, and in the canonical mode its partner)
        auto put = [&](long fh, C val) {
          if (corb) {  // the canonical orbital column(s) of the pair, row w = mh of cout
            const long row = (long)mh * ld.Nr * ld.nc;
            const int d1 = s_tcol[fh - 2 * col0], d2 = s_tpar[fh - 2 * col0];
            if (d1 >= 0) reinterpret_cast<C *>(ld.cout)[row + d1] = val;
            if (d2 >= 0) reinterpret_cast<C *>(ld.cout)[row + d2] = val;
            return;
          }
          long col = fh, pc = -1;
          if (canon) {
            col = s_tcol[fh - 2 * col0];
            pc = s_tpar[fh - 2 * col0];
            if (pc == col) pc = -1;
          }
          store((long)mp * Ccols + col, val);
          if (neg) store((long)mn * Ccols + col, conj_el(val));
          if (pc >= 0) {
            store((long)mp * Ccols + pc, val);
            if (neg) store((long)mn * Ccols + pc, conj_el(val));
          }
        };
        put(f, F);
        if (f + 1 < n_real) put(f + 1, H);
      }
      return;
    }
  }
  for (int w = tid; w < nwt * ic; w += nthr) {
    const int c = w & (ic - 1), mi = w >> lg;
    if (c >= ncol) continue;
    store((long)mi * Ccols + col0 + c, value(c, mi));
  }
}

template <class Loader>
__global__ void __launch_bounds__(256) trapz_kernel(Loader ld, double2 *__restrict__ out, long C, int n_tau,
                                                    double beta) {
  for (long col = blockIdx.x * (long)blockDim.x + threadIdx.x; col < C; col += (long)gridDim.x * blockDim.x) {
    double2 s = make_double2(0.0, 0.0);
    for (int t = 0; t < n_tau; ++t) s = cadd(s, ld(t, col));
    s = csub(s, cscale(ld(0, col), 0.5));
    s = csub(s, cscale(ld(n_tau - 1, col), 0.5));
    out[col] = cscale(s, beta / (double)(n_tau - 1));
  }
}

__global__ void __launch_bounds__(256) bubble_kernel(BubbleLoader ld, double2 *__restrict__ out, long C) {
  const long total = C * ld.n_tau;
  for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
    const int t = (int)(idx / C);
    out[idx] = ld(t, idx - (long)t * C);
  }
}

// Columns per CTA: a power of two (dividing the 512 threads) such that one
// length-L buffer (two when the FFT has a generic-radix stage) plus the
// per-column extras fit in shared memory.
int pick_ic(const FftDesc &fft, size_t extra_per_col, int *ic_out, int *lg_out, size_t *smem_out) {
  // Two CTAs per SM where the mesh allows: while one waits at a stage barrier
  // or on its loads, the other computes.
  const size_t full = (size_t)std::min(max_smem_optin(), 220 * 1024);
  size_t budget = full / 2 - 1024;
  if ((fft.has_generic ? 2 : 1) * (size_t)fft.n * sizeof(double2) + extra_per_col > budget) budget = full;
  const size_t bufs = fft.has_generic ? 2 : 1;
  const size_t L = fft.n;
  int ic = 32;
  while (ic > 1 && (bufs * L * ic * sizeof(double2) + extra_per_col * ic) > budget) ic /= 2;
  const size_t smem = bufs * L * ic * sizeof(double2) + extra_per_col * ic;
  if (smem > budget)
    return set_error(TPRF_ERR_UNSUPPORTED_SIZE, "Matsubara FFT: time mesh too long for one CTA");
  int lg = 0;
  while ((1 << lg) < ic) ++lg;
  *ic_out = ic;
  *lg_out = lg;
  *smem_out = smem;
  return TPRF_OK;
}

// Every power-of-two column count up to 32 whose tile fits one CTA (the
// autotuner's candidates; pick_ic gives the heuristic one), and the shared
// memory of a tile.
size_t ic_smem(const FftDesc &fft, size_t extra_per_col, int ic) {
  return (fft.has_generic ? 2 : 1) * (size_t)fft.n * ic * sizeof(double2) + extra_per_col * ic;
}
std::vector<int> ic_candidates(const FftDesc &fft, size_t extra_per_col) {
  const size_t full = (size_t)std::min(max_smem_optin(), 220 * 1024);
  std::vector<int> out;
  for (int ic = 1; ic <= 32; ic *= 2)
    if (ic_smem(fft, extra_per_col, ic) <= full) out.push_back(ic);
  return out;
}
int log2_ic(int ic) {
  int lg = 0;
  while ((1 << lg) < ic) ++lg;
  return lg;
}
// Columns timed per candidate: enough CTAs to fill the GPU several times.
long tune_columns(long C) { return std::min(C, (long)num_sms() * 8 * 32); }

long grid_for(long work, int threads) {
  long blocks = (work + threads - 1) / threads;
  const long cap = (long)num_sms() * 32;
  return std::max(1L, std::min(blocks, cap));
}

// Tuning reruns a prefix of the columns, so it needs the input apart from the output.
bool aliases(const ArrayLoader &l, const double2 *out) { return (const void *)l.x == (const void *)out; }
bool aliases(const BubbleLoader &l, const double2 *out) { return (const void *)l.g == (const void *)out; }
int tune_tag(const ArrayLoader &) { return 0; }
int tune_tag(const BubbleLoader &l) { return 10 + l.nb; }
int tune_tag(const BubbleLoaderDF &l) { return 20 + l.nb; }
int tune_tag(const BubblePairLoaderDF &l) { return 30 + l.nb; }

template <class Loader, class E>
int launch_tau_to_w_as(const TauWPlan *p, Loader ld, double2 *out, long C, cudaStream_t stream,
                       bool out_df = false, bool skip_neg = false) {
  const size_t extra = 5 * sizeof(double2) + 4 * sizeof(long) + 18 * sizeof(double2);
  int ic, lg;
  size_t smem;
  int st = pick_ic(p->fft, extra, &ic, &lg, &smem);
  if (st) return st;
  if (p->fermion && !std::is_same<Loader, ArrayLoader>::value)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "tau -> w: fermionic transform of a bubble");
  const FitRows fr = make_fit_rows(p->beta, p->n_tau);
  int radix = 0;  // radix order of the FFT (fft_variants), chosen after the columns per CTA
  // columns [0, n_cols) of the C columns with icv columns per CTA and radix order rv
  auto launch_rv = [&](int icv, long n_cols, int rv) -> int {
    TauWPlan pv = *p;
    if (rv != 0 && (st = get_fft_variant(p->L, rv, &pv.fft))) return st;
    const size_t sm = ic_smem(pv.fft, extra, icv);
    const long blocks = (n_cols + icv - 1) / icv;
    if constexpr (std::is_same<Loader, ArrayLoader>::value) {
      if (p->fermion) {
        TPRF_CUDA(cudaFuncSetAttribute(tau_to_w_kernel<Loader, E, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sm));
        tau_to_w_kernel<Loader, E, true><<<(unsigned)blocks, kMatsubaraThreads, sm, stream>>>(pv, ld, fr, out, C, icv,
                                                                                              log2_ic(icv), out_df, skip_neg);
        TPRF_KERNEL_LAUNCHED("tau_to_w_kernel");
        return TPRF_OK;
      }
    }
    TPRF_CUDA(cudaFuncSetAttribute(tau_to_w_kernel<Loader, E, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)sm));
    tau_to_w_kernel<Loader, E, false><<<(unsigned)blocks, kMatsubaraThreads, sm, stream>>>(pv, ld, fr, out, C, icv,
                                                                                           log2_ic(icv), out_df, skip_neg);
    TPRF_KERNEL_LAUNCHED("tau_to_w_kernel");
    return TPRF_OK;
  };
  auto launch = [&](int icv, long n_cols) -> int { return launch_rv(icv, n_cols, radix); };
  const long Ct = tune_columns(C);
  const std::vector<int> radix_cands = fft_variants(p->L);
  const std::string rkey = tune_key("tau_to_w_radix", {p->L, p->nw, p->fermion, tune_tag(ld), out_df});
  if (!aliases(ld, out)) {
    if ((st = tune_pick(tune_key("tau_to_w", {p->L, p->nw, p->fermion, tune_tag(ld), out_df}),
                        ic_candidates(p->fft, extra), ic, stream, [&](int v) { return launch(v, Ct); }, &ic)))
      return st;
    if (radix_cands.size() > 1 &&
        (st = tune_pick(rkey, radix_cands, 0, stream, [&](int v) { return launch_rv(ic, Ct, v); }, &radix)))
      return st;
  } else if ((st = tune_lookup(rkey, radix_cands, 0, &radix))) {
    return st;
  }
  return launch(ic, C);
}

template <class Loader>
int launch_tau_to_w_with(const TauWPlan *p, Loader ld, double2 *out, long C, cudaStream_t stream) {
  if (arith_mode() == kArithFP64) return launch_tau_to_w_as<Loader, double2>(p, ld, out, C, stream);
  return launch_tau_to_w_as<Loader, cdf>(p, ld, out, C, stream);
}

int check_tau_w(double beta, int n_tau, int nw) {
  if (!(beta > 0.0) || n_tau < 10 || nw < 1)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "tau -> w: need beta > 0, n_tau >= 10, nw >= 1");
  if (n_tau - 1 < 2 * nw)
    return set_error(TPRF_ERR_MESH_TOO_SHORT,
                     "Fourier: the time mesh must be at least twice as long as the number of positive frequencies");
  return TPRF_OK;
}

BubbleLoader make_bubble(const double2 *g, int n_tau, const int dims[3], int nb) {
  BubbleLoader ld;
  ld.g = g;
  ld.Nr = (long)dims[0] * dims[1] * dims[2];
  ld.nb = nb;
  ld.n_tau = n_tau;
  ld.d0 = dims[0];
  ld.d1 = dims[1];
  ld.d2 = dims[2];
  return ld;
}

// the bubble's column index (r, abcd) must fit the loaders' 32-bit arithmetic
int bubble_columns(const int dims[3], int nb) {
  const long long cols = (long long)dims[0] * dims[1] * dims[2] * nb * nb * nb * nb;
  if (cols >= (1LL << 31)) return set_error(TPRF_ERR_UNSUPPORTED_SIZE, "bubble: N_r nb^4 must be below 2^31");
  return TPRF_OK;
}

int check_bubble(int n_tau, const int dims[3], int nb, const void *g, const void *out) {
  if (!dims || !g || !out || n_tau < 2 || nb < 1 || nb > 8)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "bubble: bad shape (nb 1..8, n_tau >= 2) or null pointer");
  for (int a = 0; a < 3; ++a)
    if (dims[a] < 1) return set_error(TPRF_ERR_INVALID_ARGUMENT, "bubble: mesh dims must be >= 1");
  return bubble_columns(dims, nb);
}

// ---------------------------------------------------------------------------
// Adjoints (transposed linear maps) for the differentiable path: tail terms
// and sums in FP64, the FFT butterflies in double-float (FP64 in the FP64
// arithmetic mode), as in the forward transforms.

// Sum over the threads of a CTA that share a column (c = tid & (ic - 1),
// ic a power of two <= 32) of three complex partials: shuffles inside a warp
// over the lanes that differ in the bits above c, then the warps' results
// through red ([n_warps][3][ic]). The sums end in the threads tid < ic; every
// thread of the CTA must call it.
__device__ __forceinline__ void column_sum3(double2 v[3], double2 *red, int ic) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, n_warps = blockDim.x >> 5;
#pragma unroll
  for (int j = 0; j < 3; ++j)
    for (int off = 16; off >= ic; off >>= 1) {
      v[j].x += __shfl_xor_sync(0xffffffffu, v[j].x, off);
      v[j].y += __shfl_xor_sync(0xffffffffu, v[j].y, off);
    }
  if (lane < ic)
#pragma unroll
    for (int j = 0; j < 3; ++j) red[(warp * 3 + j) * ic + lane] = v[j];
  __syncthreads();
  if (tid < ic)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double2 s = make_double2(0.0, 0.0);
      for (int w = 0; w < n_warps; ++w) s = cadd(s, red[(w * 3 + j) * ic + tid]);
      v[j] = s;
    }
}

// tau -> i omega is linear in chi(tau): chi(i w_m) = (beta/L) sum_{t<L} g_t e^{+2 pi i t k_m / L}
// + sum_j a_j K[j][m], with a = C m and the moments m linear in the 18 end samples
// (m1 = -(g_0 - g_L), m2/m3 from fit_derivatives). Its transpose maps the output
// gradient y to: (beta/L) FFT_FORWARD(y placed at rows k_m)[t] for t < L, plus
// the moment terms D^T C^T (K^H y) on the end samples. K^H y is summed by all
// threads of the CTA while y is placed.
//
// FUSED: the columns are the bubble's (r, abcd) and, instead of storing
// chi0_grad(tau, r), each column adds its two bubble-adjoint terms to
// G_grad(tau, r) (zeroed by the caller) with FP64 atomics:
//   G_grad_da(tau_t, r)           += conj(G_bc(tau_{N-1-t}, -r)) chi0_grad_abcd(tau_t, r),
//   G_grad_bc(tau_{N-1-t}, -r)    += conj(G_da(tau_t, r))        chi0_grad_abcd(tau_t, r),
// the transpose of chi0_abcd(tau_t, r) = G_da(tau_t, r) G_bc(tau_{N-1-t}, -r), so
// chi0_grad(tau, r) never exists in device memory.
template <class C, bool FUSED = false>
__global__ void __launch_bounds__(256) tau_to_w_adjoint_kernel(TauWPlan p, VinvRows vr, const double2 *__restrict__ yg,
                                                               double2 *__restrict__ xg, long Ccols, int ic, int lg,
                                                               BubbleLoader ld) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *a = reinterpret_cast<C *>(smem_raw);
  const int L = p.L, nw = p.nw, nwt = 2 * p.nw - 1;
  const int *rev = p.fft.rev;
  C *b = p.fft.has_generic ? a + (size_t)L * ic : nullptr;
  double2 *ends = reinterpret_cast<double2 *>(a + (size_t)(p.fft.has_generic ? 2 : 1) * L * ic);  // [18][ic]
  double2 *red = ends + 18 * ic;                                      // [8][3][ic]
  long *soff = reinterpret_cast<long *>(red + 24 * ic);               // FUSED: [2][ic] G offsets of the columns
  const int tid = threadIdx.x, nthr = blockDim.x;
  const long col0 = blockIdx.x * (long)ic;
  const int ncol = (int)min((long)ic, Ccols - col0);
  if constexpr (FUSED) ld.setup(col0, ic, ncol, soff);  // ordered before use by the barriers below
  for (int w = tid; w < L * ic; w += nthr) a[w] = from_d2<C>(make_double2(0.0, 0.0));
  __syncthreads();
  double2 v[3] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
  for (int w = tid; w < nwt * ic; w += nthr) {
    const int c = w & (ic - 1), mi = w >> lg;
    if (c < ncol) {
      const double2 y = yg[(long)mi * Ccols + col0 + c];
      a[rev[(mi - (nw - 1) + L) % L] * ic + c] = from_d2<C>(y);
#pragma unroll
      for (int j = 0; j < 3; ++j) v[j] = cfma(cconj(p.K[j * nwt + mi]), y, v[j]);
    }
  }
  column_sum3(v, red, ic);
  const double dtau = p.beta / (double)(p.n_tau - 1);
  if (tid < ic) {
    const int c = tid;
    double2 e[18];
#pragma unroll
    for (int q = 0; q < 18; ++q) e[q] = make_double2(0.0, 0.0);
    if (c < ncol) {
      // a1 = 4(m1 - m3)/3, a2 = m3 - (m1 + m2)/2, a3 = m1/6 + m2/2 + m3/3: transpose
      const double2 m1g = cadd(cadd(cscale(v[0], 4.0 / 3.0), cscale(v[1], -0.5)), cscale(v[2], 1.0 / 6.0));
      const double2 m2g = cadd(cscale(v[1], -0.5), cscale(v[2], 0.5));
      const double2 m3g = cadd(cadd(cscale(v[0], -4.0 / 3.0), v[1]), cscale(v[2], 1.0 / 3.0));
      // m1 = -(g0 - gL); m2 = gl0 - gr0; m3 = -(gl1 + gr1) 2/dtau
      e[0] = csub(e[0], m1g);
      e[17] = cadd(e[17], m1g);
      const double2 gl0g = m2g, gr0g = cscale(m2g, -1.0);
      const double2 gl1g = cscale(m3g, -2.0 / dtau), gr1g = gl1g;
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const double tau_m = (double)(m + 1) * dtau;
        const double2 dlg = cscale(cadd(cscale(gl0g, vr.r0[m]), cscale(gl1g, vr.r1[m])), 1.0 / tau_m);
        const double2 drg = cscale(cadd(cscale(gr0g, vr.r0[m]), cscale(gr1g, vr.r1[m])), 1.0 / tau_m);
        e[m + 1] = cadd(e[m + 1], dlg);  // dl[m] = (g[m+1] - g[0]) / tau
        e[0] = csub(e[0], dlg);
        e[17] = cadd(e[17], drg);        // dr[m] = (g[L] - g[L-1-m]) / tau
        e[16 - m] = csub(e[16 - m], drg);  // slot 9 + s holds row L - 8 + s; row L-1-m -> s = 7 - m
      }
    }
#pragma unroll
    for (int q = 0; q < 18; ++q) ends[q * ic + c] = e[q];
  }
  C *r = fft_smem<true>(a, b, p.fft, ic);  // its first barrier orders the ends writes
  const double fact = p.beta / (double)L;
  for (int w = tid; w < (L + 1) * ic; w += nthr) {
    const int c = w & (ic - 1), t = w >> lg;
    if (c >= ncol) continue;
    double2 v = (t < L) ? cscale(as_d2(r[t * ic + c]), fact) : make_double2(0.0, 0.0);
    if (t <= 8) v = cadd(v, ends[t * ic + c]);
    if (t >= L - 8) v = cadd(v, ends[(9 + t - (L - 8)) * ic + c]);
    if constexpr (FUSED) {
      const long slice = ld.Nr * ld.nb * ld.nb, ox = soff[c], oy = soff[ic + c];
      const long tm = (long)ld.n_tau - 1 - t;
      const double2 t1 = cmul(cconj(ld.g[tm * slice + oy]), v);       // into G_grad_da(tau_t, r)
      const double2 t2 = cmul(cconj(ld.g[(long)t * slice + ox]), v);  // into G_grad_bc(tau_{N-1-t}, -r)
      double *g1 = reinterpret_cast<double *>(xg + (long)t * slice + ox);
      double *g2 = reinterpret_cast<double *>(xg + tm * slice + oy);
      atomicAdd(g1, t1.x);
      atomicAdd(g1 + 1, t1.y);
      atomicAdd(g2, t2.x);
      atomicAdd(g2 + 1, t2.y);
    } else {
      xg[(long)t * Ccols + col0 + c] = v;
    }
  }
}

// iv -> tau is linear in G(iv): G(tau_t) = P[t] F[t] + sum_j a_j Q[j][t] (t < L),
// G[L] = -(G[0] + m1), F = FFT_FORWARD of g placed at rows (n+L)%L, a = Cf m,
// m = Fit g[fit rows] (when fitted). Transpose: y_0 -= y_L; BACKWARD FFT of
// conj(P) y at rows (n+L)%L; plus Fit^H Cf^T (Q^H y) on the fit rows. Q^H y is
// summed by all threads of the CTA while y is placed; the fit terms are added
// to the transformed rows in shared memory (each fit row once per column).
template <class C>
__global__ void __launch_bounds__(256) nu_to_tau_adjoint_kernel(NuTauPlan p, const double2 *__restrict__ yg,
                                                                double2 *__restrict__ gg, long Ccols, int ic, int lg,
                                                                int fitted) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *a = reinterpret_cast<C *>(smem_raw);
  const int L = p.L, n_iw = p.n_iw, nnu = 2 * p.n_iw;
  const int *rev = p.fft.rev;
  C *b = p.fft.has_generic ? a + (size_t)L * ic : nullptr;
  double2 *mg = reinterpret_cast<double2 *>(a + (size_t)(p.fft.has_generic ? 2 : 1) * L * ic);  // [3][ic]
  double2 *red = mg + 3 * ic;                                       // [8][3][ic]
  const int tid = threadIdx.x, nthr = blockDim.x;
  const long col0 = blockIdx.x * (long)ic;
  const int ncol = (int)min((long)ic, Ccols - col0);
  double2 v[3] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
  for (int w = tid; w < L * ic; w += nthr) {
    const int c = w & (ic - 1), t = w >> lg;
    double2 y = make_double2(0.0, 0.0);
    if (c < ncol) {
      y = yg[(long)t * Ccols + col0 + c];
      if (t == 0) y = csub(y, yg[(long)L * Ccols + col0 + c]);
      if (fitted)
#pragma unroll
        for (int j = 0; j < 3; ++j) v[j] = cfma(cconj(p.Q[j * L + t]), y, v[j]);
    }
    a[rev[t] * ic + c] = from_d2<C>(cmul(cconj(p.P[t]), y));
  }
  column_sum3(v, red, ic);
  if (tid < ic) {
    const int c = tid;
    const double2 yL = (c < ncol && fitted) ? yg[(long)L * Ccols + col0 + c] : make_double2(0.0, 0.0);
    // a1 = m1 - m3, a2 = (m2 + m3)/2, a3 = (m3 - m2)/2; G[L] adds -m1
    mg[0 * ic + c] = csub(v[0], yL);
    mg[1 * ic + c] = cscale(csub(v[1], v[2]), 0.5);
    mg[2 * ic + c] = cadd(cscale(v[0], -1.0), cscale(cadd(v[1], v[2]), 0.5));
  }
  C *r = fft_smem<false>(a, b, p.fft, ic);  // its first barrier orders the mg writes
  if (fitted) {
    for (int w = tid; w < p.n_fit * ic; w += nthr) {
      const int c = w & (ic - 1), i = w >> lg;
      const int row = (p.fit_row[i] - n_iw + L) % L;
      double2 s = as_d2(r[row * ic + c]);
      for (int q = 1; q <= 3; ++q) s = cfma(cconj(p.fitF[q * p.n_fit + i]), mg[(q - 1) * ic + c], s);
      r[row * ic + c] = from_d2<C>(s);
    }
    __syncthreads();
  }
  for (int w = tid; w < nnu * ic; w += nthr) {
    const int c = w & (ic - 1), n = w >> lg;
    if (c >= ncol) continue;
    gg[(long)n * Ccols + col0 + c] = as_d2(r[((n - n_iw + L) % L) * ic + c]);
  }
}

// Bubble adjoint as a gather: G_grad(tau_i, r)_xy =
//   sum_bc conj(G_bc(tau_{N-1-i}, -r)) chig_{y b c x}(tau_i, r)
// + sum_ad conj(G_da(tau_{N-1-i}, -r)) chig_{a x y d}(tau_{N-1-i}, -r).
__global__ void __launch_bounds__(256) bubble_adjoint_kernel(BubbleLoader ld, const double2 *__restrict__ chig,
                                                             double2 *__restrict__ gg) {
  const int nb = ld.nb, nb2 = nb * nb, nb4 = nb2 * nb2;
  const long Nr = ld.Nr, total = (long)ld.n_tau * Nr * nb2;
  for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
    const int xy = (int)(idx % nb2);
    const long r = (idx / nb2) % Nr;
    const int i = (int)(idx / ((long)nb2 * Nr));
    const int x = xy / nb, y = xy % nb;
    const int i2 = (int)(r % ld.d2), i1 = (int)((r / ld.d2) % ld.d1), i0 = (int)(r / ((long)ld.d2 * ld.d1));
    const long mr = ((long)((ld.d0 - i0) % ld.d0) * ld.d1 + (ld.d1 - i1) % ld.d1) * ld.d2 + (ld.d2 - i2) % ld.d2;
    const int im = ld.n_tau - 1 - i;
    const double2 *gm = ld.g + ((long)im * Nr + mr) * nb2;  // G(tau_{N-1-i}, -r)
    const double2 *c1 = chig + ((long)i * Nr + r) * nb4;
    const double2 *c2 = chig + ((long)im * Nr + mr) * nb4;
    double2 acc = make_double2(0.0, 0.0);
    for (int bb = 0; bb < nb; ++bb)
      for (int cc = 0; cc < nb; ++cc)
        acc = cfma(cconj(gm[bb * nb + cc]), c1[((y * nb + bb) * nb + cc) * nb + x], acc);
    for (int aa = 0; aa < nb; ++aa)
      for (int dd = 0; dd < nb; ++dd)
        acc = cfma(cconj(gm[dd * nb + aa]), c2[((aa * nb + x) * nb + y) * nb + dd], acc);
    gg[idx] = acc;
  }
}

}  // namespace

// ---- internal launchers (no synchronisation) --------------------------------

int launch_nu_to_tau_stat(double beta, int n_iw, int n_tau, bool fermion, long C, const double2 *gw,
                          const double2 *mom, double2 *gt, cudaStream_t stream, cdf *gt_df = nullptr,
                          unsigned *gmax = nullptr, const unsigned *hwords = nullptr, bool fit_rows_only = false,
                          const TransposePairs *tp = nullptr);

// The fermionic transform that also writes G(tau) as double-float pairs into
// gt_df (left untouched in the FP64 arithmetic mode), for the fused bubble's
// double-float product.
// gmax (nullable, two words the caller zeroed): max |G| and max |Im G| of the
// result as float bits, which decide whether the bubble can pair real columns.
int launch_nu_to_tau_df(double beta, int n_iw, int n_tau, long C, const double2 *gw, const double2 *mom, double2 *gt,
                        void *gt_df, cudaStream_t stream, unsigned *gmax, const unsigned *hwords, bool fit_rows_only,
                        const TransposePairs *tp) {
  return launch_nu_to_tau_stat(beta, n_iw, n_tau, true, C, gw, mom, gt, stream, reinterpret_cast<cdf *>(gt_df), gmax,
                               hwords, fit_rows_only, tp);
}

// Words of G(iv, r): hw[0] = max |G|, hw[1] = max |G(iv) - conj(G(-iv))|
// (Hermitian in iv: G(tau, r) is real) and, with the column layout (nb > 0,
// C = N_r nb^2), hw[2] = max |G_ab(iv, -r) - G_ba(iv, r)| over all rows (the
// transposition symmetry of real hoppings); nb = 0 marks hw[2] infinite (no).
__global__ void __launch_bounds__(256) hermitian_check_kernel(const double2 *__restrict__ gw, int n_iw, long C,
                                                              unsigned *hw, int nb, int d0, int d1, int d2) {
  // magnitudes as the larger of |Re| and |Im| (within sqrt 2 of the modulus, and
  // no squares that could overflow or underflow FP32): the difference in FP64 (it
  // cancels), everything else in FP32 (the FP64 pipe is the scarce one)
  float g_abs = 0.f, g_dev = 0.f, g_tdev = 0.f;
  const int nb2 = nb * nb;
  // rows i < n_iw against rows 2 n_iw - 1 - i; the (row, column) of the
  // grid-stride index advance without a division per element
  const long stride = (long)gridDim.x * blockDim.x;
  const long start = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long dstep = stride / C, cstep = stride - dstep * C;
  long i = start / C, c = start - i * C;
  for (; i < n_iw; i += dstep, c += cstep) {
    if (c >= C) {
      c -= C;
      ++i;
      if (i >= n_iw) break;
    }
    const double2 a = gw[i * C + c], b = gw[(2L * n_iw - 1 - i) * C + c];
    // FP32 values by truncating bit operations (a conversion instruction would
    // run on the FP64 pipe): the tolerance test needs magnitudes to a few digits
    const float ax = split_double(a.x).hi, ay = split_double(a.y).hi, bx = split_double(b.x).hi,
                by = split_double(b.y).hi;
    const float dx = split_double(a.x - b.x).hi, dy = split_double(a.y + b.y).hi;
    g_abs = fmaxf(g_abs, fmaxf(fmaxf(fabsf(ax), fabsf(ay)), fmaxf(fabsf(bx), fabsf(by))));
    g_dev = fmaxf(g_dev, fmaxf(fabsf(dx), fabsf(dy)));
    if (nb > 0) {
      // the partner column (-r, ba) of c = (r, ab), at both rows
      const int ci = (int)c, r = ci / nb2, e = ci - r * nb2, ea = e / nb, eb = e - ea * nb;
      const int i2 = r % d2, i1 = (r / d2) % d1, i0 = r / (d2 * d1);
      const long mr = ((long)((d0 - i0) % d0) * d1 + (d1 - i1) % d1) * d2 + (d2 - i2) % d2;
      const long tc = mr * nb2 + eb * nb + ea;
      const double2 at = gw[i * C + tc], bt = gw[(2L * n_iw - 1 - i) * C + tc];
      g_tdev = fmaxf(g_tdev, fmaxf(fmaxf(fabsf(split_double(a.x - at.x).hi), fabsf(split_double(a.y - at.y).hi)),
                                   fmaxf(fabsf(split_double(b.x - bt.x).hi), fabsf(split_double(b.y - bt.y).hi))));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    g_abs = fmaxf(g_abs, __shfl_xor_sync(0xffffffffu, g_abs, o));
    g_dev = fmaxf(g_dev, __shfl_xor_sync(0xffffffffu, g_dev, o));
    g_tdev = fmaxf(g_tdev, __shfl_xor_sync(0xffffffffu, g_tdev, o));
  }
  if ((threadIdx.x & 31) == 0) {  // non-negative floats order as their bit patterns
    atomicMax(hw, __float_as_uint(g_abs));
    atomicMax(hw + 1, __float_as_uint(g_dev));
    atomicMax(hw + 2, nb > 0 ? __float_as_uint(g_tdev) : 0x7f800000u);
  }
}

int launch_hermitian_check(int n_iw, long C, const double2 *gw, unsigned *hwords, cudaStream_t stream,
                           const int *dims, int nb) {
  const long total = (long)n_iw * C;
  const unsigned blocks = (unsigned)std::max(1L, std::min((total + 255) / 256, (long)num_sms() * 8));
  const bool layout = dims && nb > 0 && (long)dims[0] * dims[1] * dims[2] * nb * nb == C && C < 0x7fffffffL;
  hermitian_check_kernel<<<blocks, 256, 0, stream>>>(gw, n_iw, C, hwords, layout ? nb : 0, layout ? dims[0] : 1,
                                                     layout ? dims[1] : 1, layout ? dims[2] : 1);
  TPRF_KERNEL_LAUNCHED("hermitian_check_kernel");
  return TPRF_OK;
}

int launch_nu_to_tau(double beta, int n_iw, int n_tau, long C, const double2 *gw, const double2 *mom, double2 *gt,
                     cudaStream_t stream) {
  return launch_nu_to_tau_stat(beta, n_iw, n_tau, true, C, gw, mom, gt, stream);
}

// n: fermionic n_max or bosonic nw; the time mesh must hold L >= 2 n points
// (fourier_matsubara.cpp:250-254).
int launch_nu_to_tau_stat(double beta, int n_iw, int n_tau, bool fermion, long C, const double2 *gw,
                          const double2 *mom, double2 *gt, cudaStream_t stream, cdf *gt_df, unsigned *gmax,
                          const unsigned *hwords, bool fit_rows_only, const TransposePairs *tp) {
  if (n_tau < 0) n_tau = default_n_tau(n_iw);
  if (!(beta > 0.0) || n_iw < 1 || n_tau < 2 || C < 1 || (!fermion && n_iw < 2))
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "fourier_wr_to_tr: bad mesh");
  if (n_tau - 1 < 2 * n_iw)
    return set_error(TPRF_ERR_MESH_TOO_SHORT,
                     "Inverse Fourier: the time mesh must be at least twice as long as the freq mesh");
  const NuTauPlan *p = nullptr;
  int st = get_nu_tau_plan_stat(beta, n_iw, n_tau, fermion, &p);
  if (st) return st;
  if (!mom && p->n_mom < 4)
    return set_error(TPRF_ERR_TAIL_FIT, "Inverse Fourier requires at least a proper 3rd high-frequency moment");
  unsigned *status = device_status_word();
  if (!status) return TPRF_ERR_CUDA;
  const size_t extra = 14 * sizeof(double2);
  int ic, lg;
  size_t smem;
  st = pick_ic(p->fft, extra, &ic, &lg, &smem);
  if (st) return st;
  const bool fp64 = arith_mode() == kArithFP64;
  int radix = 0;  // radix order of the FFT (fft_variants), chosen after the columns per CTA
  auto launch_rv = [&](int icv, long n_cols, int rv) -> int {  // columns [0, n_cols), icv per CTA, radix order rv
    NuTauPlan pv = *p;
    if (rv != 0 && (st = get_fft_variant(p->L, rv, &pv.fft))) return st;
    const size_t sm = ic_smem(pv.fft, extra, icv);
    const long blocks = (n_cols + icv - 1) / icv;
    if (fp64) {
      TPRF_CUDA(cudaFuncSetAttribute(nu_to_tau_kernel<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      nu_to_tau_kernel<double2><<<(unsigned)blocks, kMatsubaraThreads, sm, stream>>>(pv, gw, mom, gt, C, icv,
                                                                                      log2_ic(icv), status, nullptr,
                                                                                      gmax, nullptr, 0, nullptr, 0L);
    } else {
      TPRF_CUDA(cudaFuncSetAttribute(nu_to_tau_kernel<cdf>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      nu_to_tau_kernel<cdf><<<(unsigned)blocks, kMatsubaraThreads, sm, stream>>>(pv, gw, mom, gt, C, icv, log2_ic(icv),
                                                                                  status, gt_df, gmax, hwords,
                                                                                  fit_rows_only ? 1 : 0,
                                                                                  tp ? tp->pairs : nullptr,
                                                                                  tp ? tp->n_can : 0L);
    }
    TPRF_KERNEL_LAUNCHED("nu_to_tau_kernel");
    return TPRF_OK;
  };
  auto launch = [&](int icv, long n_cols) -> int { return launch_rv(icv, n_cols, radix); };
  const long Ct = tune_columns(C);
  const std::vector<int> radix_cands = fft_variants(p->L);
  const std::string rkey = tune_key("nu_to_tau_radix", {p->L, p->n_iw, p->fermion, mom != nullptr, gt_df != nullptr});
  if ((const void *)gw != (const void *)gt) {
    if ((st = tune_pick(tune_key("nu_to_tau", {p->L, p->n_iw, p->fermion, mom != nullptr, gt_df != nullptr}),
                        ic_candidates(p->fft, extra), ic, stream, [&](int v) { return launch(v, Ct); }, &ic)))
      return st;
    if (radix_cands.size() > 1 &&
        (st = tune_pick(rkey, radix_cands, 0, stream, [&](int v) { return launch_rv(ic, Ct, v); }, &radix)))
      return st;
  } else if ((st = tune_lookup(rkey, radix_cands, 0, &radix))) {
    return st;
  }
  return launch(ic, C);
}

int launch_chi_wr_from_chi_tr(double beta, int n_tau, int nw, long C, const double2 *chi_tr, double2 *chi_wr,
                              cudaStream_t stream) {
  int st = check_tau_w(beta, n_tau, nw);
  if (st) return st;
  const TauWPlan *p = nullptr;
  if ((st = get_tau_w_plan(beta, n_tau, nw, &p))) return st;
  return launch_tau_to_w_with(p, ArrayLoader{chi_tr, C}, chi_wr, C, stream);
}

// fermionic tau -> i nu (fourier_matsubara.cpp:123-184, fermion branch): n_iw
// positive frequencies, outputs n = -n_iw .. n_iw-1
int launch_fourier_tr_to_wr(double beta, int n_tau, int n_iw, long C, const double2 *g_tr, double2 *g_wr,
                            cudaStream_t stream) {
  int st = check_tau_w(beta, n_tau, n_iw);
  if (st) return st;
  const TauWPlan *p = nullptr;
  if ((st = get_tau_w_plan_stat(beta, n_tau, n_iw, true, &p))) return st;
  return launch_tau_to_w_with(p, ArrayLoader{g_tr, C}, g_wr, C, stream);
}

int launch_chi0_wr_from_grt(double beta, int n_tau, int nw, const int dims[3], int nb, const double2 *g,
                            double2 *chi0_wr, cudaStream_t stream) {
  int st = check_tau_w(beta, n_tau, nw);
  if (st) return st;
  if ((st = bubble_columns(dims, nb))) return st;
  const TauWPlan *p = nullptr;
  if ((st = get_tau_w_plan(beta, n_tau, nw, &p))) return st;
  const BubbleLoader ld = make_bubble(g, n_tau, dims, nb);
  const long C = ld.Nr * nb * nb * nb * nb;
  return launch_tau_to_w_with(p, ld, chi0_wr, C, stream);
}

// The fused bubble + tau -> w reading a double-float copy of G(tau, r) as well
// (written by launch_nu_to_tau_df); g_df == NULL or the FP64 arithmetic mode
// takes the complex128 path.
int launch_chi0_wr_from_grt_df(double beta, int n_tau, int nw, const int dims[3], int nb, const double2 *g,
                               const void *g_df, double2 *chi0_wr, cudaStream_t stream, bool want_df, bool *wrote_df,
                               const unsigned *gmax, bool skip_neg, const CompactChi *cc) {
  if (wrote_df) *wrote_df = false;
  if (!g_df || arith_mode() == kArithFP64) return launch_chi0_wr_from_grt(beta, n_tau, nw, dims, nb, g, chi0_wr, stream);
  int st = check_tau_w(beta, n_tau, nw);
  if (st) return st;
  if ((st = bubble_columns(dims, nb))) return st;
  const TauWPlan *p = nullptr;
  if ((st = get_tau_w_plan(beta, n_tau, nw, &p))) return st;
  BubblePairLoaderDF ld;
  static_cast<BubbleLoader &>(ld) = make_bubble(g, n_tau, dims, nb);
  ld.gdf = reinterpret_cast<const cdf *>(g_df);
  ld.gmax = gmax;
  if (gmax) {
    const TransposePairs *tp = nullptr;
    if ((st = get_transpose_pairs(dims, nb, 4, &tp))) return st;
    ld.tpairs = tp->pairs;
    ld.n_can = tp->n_can;
    if (cc && cc->gmax == gmax && cc->buf && cc->oc && skip_neg && want_df) {
      ld.cout = reinterpret_cast<cdf *>(cc->buf);
      ld.ocomp = cc->oc->ocomp;
      ld.nc = cc->oc->nc;
    }
  }
  const long C = ld.Nr * nb * nb * nb * nb;
  st = gmax ? launch_tau_to_w_as<BubblePairLoaderDF, cdf>(p, ld, chi0_wr, C, stream, want_df, skip_neg)
            : launch_tau_to_w_as<BubbleLoaderDF, cdf>(p, static_cast<const BubbleLoaderDF &>(ld), chi0_wr, C, stream,
                                                       want_df);
  if (!st && wrote_df) *wrote_df = want_df;
  return st;
}

int launch_chi0_w0r_from_grt(double beta, int n_tau, const int dims[3], int nb, const double2 *g, double2 *chi0_wr,
                             cudaStream_t stream) {
  if (int st = bubble_columns(dims, nb)) return st;
  const BubbleLoader ld = make_bubble(g, n_tau, dims, nb);
  const long C = ld.Nr * nb * nb * nb * nb;
  trapz_kernel<BubbleLoader><<<(unsigned)grid_for(C, 256), 256, 0, stream>>>(ld, chi0_wr, C, n_tau, beta);
  TPRF_KERNEL_LAUNCHED("trapz_kernel<bubble>");
  return TPRF_OK;
}

}  // namespace tprf

// ---- C ABI ------------------------------------------------------------------

using namespace tprf;

extern "C" int tprf_fourier_wr_to_tr(double beta, int n_iw, int n_tau, long n_r, long n_target, const double *g_wr,
                                     const double *moments, double *g_tr, void *stream) {
  if (!g_wr || !g_tr || n_r < 1 || n_target < 1)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "fourier_wr_to_tr: bad shape or null pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = launch_nu_to_tau(beta, n_iw, n_tau, n_r * n_target, reinterpret_cast<const double2 *>(g_wr),
                            reinterpret_cast<const double2 *>(moments), reinterpret_cast<double2 *>(g_tr), s);
  if (st) return st;
  return finish_with_checks(s, "fourier_wr_to_tr");
}

extern "C" int tprf_fourier_tr_to_wr(double beta, int n_tau, int n_iw, long n_r, long n_target, const double *g_tr,
                                     double *g_wr, void *stream) {
  if (!g_tr || !g_wr || n_r < 1 || n_target < 1)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "fourier_tr_to_wr: bad shape or null pointer");
  if (n_iw < 0) n_iw = (n_tau - 1) / 6;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = launch_fourier_tr_to_wr(beta, n_tau, n_iw, n_r * n_target, reinterpret_cast<const double2 *>(g_tr),
                                   reinterpret_cast<double2 *>(g_wr), s);
  if (st) return st;
  return finish_with_checks(s, "fourier_tr_to_wr");
}

extern "C" int tprf_chi_tr_from_chi_wr(double beta, int nw, int n_tau, long n_r, long n_target, const double *chi_wr,
                                       const double *moments, double *chi_tr, void *stream) {
  if (!chi_wr || !chi_tr || n_r < 1 || n_target < 1)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "chi_tr_from_chi_wr: bad shape or null pointer");
  if (n_tau < 0) n_tau = 6 * nw + 1;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = launch_nu_to_tau_stat(beta, nw, n_tau, false, n_r * n_target, reinterpret_cast<const double2 *>(chi_wr),
                                 reinterpret_cast<const double2 *>(moments), reinterpret_cast<double2 *>(chi_tr), s);
  if (st) return st;
  return finish_with_checks(s, "chi_tr_from_chi_wr");
}

extern "C" int tprf_chi_wr_from_chi_tr(double beta, int n_tau, int nw, long n_r, long n_target, const double *chi_tr,
                                       double *chi_wr, void *stream) {
  if (!chi_tr || !chi_wr || n_r < 1 || n_target < 1)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "chi_wr_from_chi_tr: bad shape or null pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = launch_chi_wr_from_chi_tr(beta, n_tau, nw, n_r * n_target, reinterpret_cast<const double2 *>(chi_tr),
                                     reinterpret_cast<double2 *>(chi_wr), s);
  if (st) return st;
  TPRF_LAUNCH_CHECK("chi_wr_from_chi_tr");
  return TPRF_OK;
}

extern "C" int tprf_chi_w0r_from_chi_tr(double beta, int n_tau, long n_r, long n_target, const double *chi_tr,
                                        double *chi_wr, void *stream) {
  if (!chi_tr || !chi_wr || n_r < 1 || n_target < 1 || n_tau < 2 || !(beta > 0.0))
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "chi_w0r_from_chi_tr: bad shape or null pointer");
  const long C = n_r * n_target;
  trapz_kernel<ArrayLoader><<<(unsigned)grid_for(C, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      ArrayLoader{reinterpret_cast<const double2 *>(chi_tr), C}, reinterpret_cast<double2 *>(chi_wr), C, n_tau, beta);
  TPRF_KERNEL_LAUNCHED("trapz_kernel<array>");
  return TPRF_OK;
}

extern "C" int tprf_chi0_tr_from_grt_PH(int n_tau, const int dims[3], int nb, const double *g_tr, double *chi0_tr,
                                        void *stream) {
  int st = check_bubble(n_tau, dims, nb, g_tr, chi0_tr);
  if (st) return st;
  const BubbleLoader ld = make_bubble(reinterpret_cast<const double2 *>(g_tr), n_tau, dims, nb);
  const long C = ld.Nr * nb * nb * nb * nb;
  bubble_kernel<<<(unsigned)grid_for(C * n_tau, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      ld, reinterpret_cast<double2 *>(chi0_tr), C);
  TPRF_KERNEL_LAUNCHED("bubble_kernel");
  return TPRF_OK;
}

extern "C" int tprf_chi0_wr_from_grt_PH(double beta, int n_tau, int nw, const int dims[3], int nb, const double *g_tr,
                                        double *chi0_wr, void *stream) {
  int st = check_bubble(n_tau, dims, nb, g_tr, chi0_wr);
  if (st) return st;
  st = launch_chi0_wr_from_grt(beta, n_tau, nw, dims, nb, reinterpret_cast<const double2 *>(g_tr),
                               reinterpret_cast<double2 *>(chi0_wr), static_cast<cudaStream_t>(stream));
  if (st) return st;
  TPRF_LAUNCH_CHECK("chi0_wr_from_grt_PH");
  return TPRF_OK;
}

extern "C" int tprf_chi0_w0r_from_grt_PH(double beta, int n_tau, const int dims[3], int nb, const double *g_tr,
                                         double *chi0_wr, void *stream) {
  int st = check_bubble(n_tau, dims, nb, g_tr, chi0_wr);
  if (st) return st;
  if (!(beta > 0.0)) return set_error(TPRF_ERR_INVALID_ARGUMENT, "chi0_w0r_from_grt_PH: beta must be > 0");
  st = launch_chi0_w0r_from_grt(beta, n_tau, dims, nb, reinterpret_cast<const double2 *>(g_tr),
                                reinterpret_cast<double2 *>(chi0_wr), static_cast<cudaStream_t>(stream));
  if (st) return st;
  TPRF_LAUNCH_CHECK("chi0_w0r_from_grt_PH");
  return TPRF_OK;
}

// ---- adjoints (differentiable path) -------------------------------------------

namespace tprf {

// Internal launchers of the adjoints (no synchronisation; also used inside
// the batched gradient's graph capture once their plans exist).
int launch_tau_to_w_adjoint(double beta, int n_tau, int nw, long C, const double2 *yg, double2 *xg,
                            cudaStream_t stream) {
  int st = check_tau_w(beta, n_tau, nw);
  if (st) return st;
  const TauWPlan *p = nullptr;
  if ((st = get_tau_w_plan(beta, n_tau, nw, &p))) return st;
  int ic, lg;
  size_t smem;
  if ((st = pick_ic(p->fft, (18 + 24) * sizeof(double2), &ic, &lg, &smem))) return st;
  // double-float butterflies unless the FP64 arithmetic mode is set
  auto kern = arith_mode() == kArithFP64 ? tau_to_w_adjoint_kernel<double2> : tau_to_w_adjoint_kernel<cdf>;
  TPRF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<(unsigned)((C + ic - 1) / ic), 256, smem, stream>>>(*p, make_vinv_rows(), yg, xg, C, ic, lg, BubbleLoader{});
  TPRF_KERNEL_LAUNCHED("tau_to_w_adjoint_kernel");
  return TPRF_OK;
}

// The fused bubble + tau -> w transposed: G_grad(tau, r) from chi0_grad(w, r)
// (FUSED tau_to_w_adjoint_kernel), chi0_grad(tau, r) never stored.
int launch_chi0_wr_from_grt_adjoint(double beta, int n_tau, int nw, const int dims[3], int nb, const double2 *g_tr,
                                    const double2 *yg, double2 *gg, cudaStream_t stream) {
  int st = check_tau_w(beta, n_tau, nw);
  if (st) return st;
  if ((st = check_bubble(n_tau, dims, nb, g_tr, gg))) return st;
  if ((st = bubble_columns(dims, nb))) return st;
  if (!yg) return set_error(TPRF_ERR_INVALID_ARGUMENT, "bubble adjoint: null gradient");
  const TauWPlan *p = nullptr;
  if ((st = get_tau_w_plan(beta, n_tau, nw, &p))) return st;
  const BubbleLoader ld = make_bubble(g_tr, n_tau, dims, nb);
  const long C = ld.Nr * nb * nb * nb * nb;
  TPRF_CUDA(cudaMemsetAsync(gg, 0, (size_t)n_tau * ld.Nr * nb * nb * sizeof(double2), stream));
  int ic, lg;
  size_t smem;
  if ((st = pick_ic(p->fft, (18 + 24 + 1) * sizeof(double2), &ic, &lg, &smem))) return st;
  auto kern = arith_mode() == kArithFP64 ? tau_to_w_adjoint_kernel<double2, true> : tau_to_w_adjoint_kernel<cdf, true>;
  TPRF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<(unsigned)((C + ic - 1) / ic), 256, smem, stream>>>(*p, make_vinv_rows(), yg, gg, C, ic, lg, ld);
  TPRF_KERNEL_LAUNCHED("tau_to_w_adjoint_kernel<fused bubble>");
  return TPRF_OK;
}

int launch_nu_to_tau_adjoint(double beta, int n_iw, int n_tau, long C, const double2 *yg, double2 *gg, bool fitted,
                             cudaStream_t stream) {
  if (n_tau - 1 < 2 * n_iw)
    return set_error(TPRF_ERR_MESH_TOO_SHORT, "Inverse Fourier: the time mesh must be at least twice as long as the freq mesh");
  const NuTauPlan *p = nullptr;
  int st = get_nu_tau_plan(beta, n_iw, n_tau, &p);
  if (st) return st;
  int ic, lg;
  size_t smem;
  if ((st = pick_ic(p->fft, (3 + 24) * sizeof(double2), &ic, &lg, &smem))) return st;
  auto kern = arith_mode() == kArithFP64 ? nu_to_tau_adjoint_kernel<double2> : nu_to_tau_adjoint_kernel<cdf>;
  TPRF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<(unsigned)((C + ic - 1) / ic), 256, smem, stream>>>(*p, yg, gg, C, ic, lg, fitted ? 1 : 0);
  TPRF_KERNEL_LAUNCHED("nu_to_tau_adjoint_kernel");
  return TPRF_OK;
}

int launch_bubble_adjoint(int n_tau, const int dims[3], int nb, const double2 *g_tr, const double2 *chig,
                          double2 *gg, cudaStream_t stream) {
  int st = check_bubble(n_tau, dims, nb, g_tr, gg);
  if (st) return st;
  if (!chig) return set_error(TPRF_ERR_INVALID_ARGUMENT, "bubble adjoint: null gradient");
  const BubbleLoader ld = make_bubble(g_tr, n_tau, dims, nb);
  const long total = (long)n_tau * ld.Nr * nb * nb;
  bubble_adjoint_kernel<<<(unsigned)grid_for(total, 256), 256, 0, stream>>>(ld, chig, gg);
  TPRF_KERNEL_LAUNCHED("bubble_adjoint_kernel");
  return TPRF_OK;
}

}  // namespace tprf

extern "C" int tprf_chi_wr_from_chi_tr_adjoint(double beta, int n_tau, int nw, long n_r, long n_target,
                                               const double *chi_wr_grad, double *chi_tr_grad, void *stream) {
  if (!chi_wr_grad || !chi_tr_grad || n_r < 1 || n_target < 1)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "chi_wr_from_chi_tr_adjoint: bad shape or null pointer");
  return launch_tau_to_w_adjoint(beta, n_tau, nw, n_r * n_target, reinterpret_cast<const double2 *>(chi_wr_grad),
                                 reinterpret_cast<double2 *>(chi_tr_grad), static_cast<cudaStream_t>(stream));
}

extern "C" int tprf_fourier_wr_to_tr_adjoint(double beta, int n_iw, int n_tau, long n_r, long n_target,
                                             const double *g_tr_grad, int fitted, double *g_wr_grad, void *stream) {
  if (!g_tr_grad || !g_wr_grad || n_r < 1 || n_target < 1 || n_iw < 1 || !(beta > 0.0))
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "fourier_wr_to_tr_adjoint: bad shape or null pointer");
  if (n_tau < 0) n_tau = default_n_tau(n_iw);
  return launch_nu_to_tau_adjoint(beta, n_iw, n_tau, n_r * n_target, reinterpret_cast<const double2 *>(g_tr_grad),
                                  reinterpret_cast<double2 *>(g_wr_grad), fitted != 0,
                                  static_cast<cudaStream_t>(stream));
}

extern "C" int tprf_chi0_wr_from_grt_PH_adjoint(double beta, int n_tau, int nw, const int dims[3], int nb,
                                                const double *g_tr, const double *chi0_wr_grad, double *g_tr_grad,
                                                void *stream) {
  return launch_chi0_wr_from_grt_adjoint(beta, n_tau, nw, dims, nb, reinterpret_cast<const double2 *>(g_tr),
                                         reinterpret_cast<const double2 *>(chi0_wr_grad),
                                         reinterpret_cast<double2 *>(g_tr_grad), static_cast<cudaStream_t>(stream));
}

extern "C" int tprf_chi0_tr_from_grt_PH_adjoint(int n_tau, const int dims[3], int nb, const double *g_tr,
                                                const double *chi0_tr_grad, double *g_tr_grad, void *stream) {
  return launch_bubble_adjoint(n_tau, dims, nb, reinterpret_cast<const double2 *>(g_tr),
                               reinterpret_cast<const double2 *>(chi0_tr_grad), reinterpret_cast<double2 *>(g_tr_grad),
                               static_cast<cudaStream_t>(stream));
}
