// Kernel (d): the RPA solve chi = [I - chi0 U]^-1 chi0 per (omega, q) point.
//
// Restates c++/triqs_tprf/lattice/rpa.cpp:29-64: chi0 and U are grouped into
// nb^2 x nb^2 matrices with rows (a, b) and columns (d, c)
// (idx_group<0,1>, idx_group<3,2>, rpa.cpp:40,54-55) and
// chi = inverse(I - chi0 * U) * chi0 (rpa.cpp:57). Here the same system is
// solved without forming the inverse: A = I - chi0 U, then Gaussian
// elimination with partial pivoting on [A | chi0] and back substitution.
//
// Design: one thread per point. A = I - chi0 U is formed from the non-zeros of
// U only (compacted once per CTA into shared memory), LU-factorised with
// partial pivoting in the thread's slice of shared memory ([element][thread]
// layout: conflict-free although every thread pivots independently), and the
// nb^2 right-hand sides (columns of chi0, re-read from L1/L2 through the row
// permutation) are solved one at a time in registers. Keeping only the LU
// factors in shared memory halves the per-thread footprint of a full
// [A | chi0] elimination, which doubles the warps per SM.
#include <algorithm>

#include "common.cuh"

namespace tprf {
namespace {

template <int NB>
__device__ __forceinline__ int colmap(int c) {  // grouped column (d, c') -> offset c' * nb + d
  return (c % NB) * NB + c / NB;
}

// element-type plumbing: double2 (FP64) or cdf (double-float)
__device__ __forceinline__ double2 el_from(double2 z, double2 *) { return z; }
__device__ __forceinline__ cdf el_from(double2 z, cdf *) { return to_cdf(z); }
__device__ __forceinline__ double2 el_to(double2 z) { return z; }
__device__ __forceinline__ double2 el_to(cdf z) { return to_double2(z); }
__device__ __forceinline__ double2 el_one(double2 *) { return make_double2(1.0, 0.0); }
__device__ __forceinline__ cdf el_one(cdf *) { return cdf{dfl{1.f, 0.f}, dfl{0.f, 0.f}}; }
__device__ __forceinline__ double2 el_zero(double2 *) { return make_double2(0.0, 0.0); }
__device__ __forceinline__ cdf el_zero(cdf *) { return cdf{dfl{0.f, 0.f}, dfl{0.f, 0.f}}; }
__device__ __forceinline__ double el_abs2(double2 z) { return cabs2(z); }
__device__ __forceinline__ double el_abs2(cdf z) { return (double)(z.x.hi * z.x.hi + z.y.hi * z.y.hi); }
__device__ __forceinline__ float el_absf(double2 z) { return (float)sqrt(cabs2(z)); }
__device__ __forceinline__ float el_absf(cdf z) { return sqrtf(z.x.hi * z.x.hi + z.y.hi * z.y.hi); }
template <class E> struct IsDf { static constexpr bool value = false; };
template <> struct IsDf<cdf> { static constexpr bool value = true; };
__device__ __forceinline__ double2 el_fms(double2 a, double2 b, double2 acc) { return cfms(a, b, acc); }
__device__ __forceinline__ cdf el_fms(cdf a, cdf b, cdf acc) { return csub(acc, cmul(a, b)); }
__device__ __forceinline__ double2 el_recip(double2 a) { return crecip(a); }
__device__ __forceinline__ cdf el_recip(cdf a) {
  // 1/(x + iy) = (x - iy) / (x^2 + y^2); the real reciprocal by one Newton step from the float one
  const dfl d = ddot_add(a.x, a.x, a.y, a.y);
  const float r0 = __frcp_rn(d.hi);
  const dfl e = dsub(dfl{1.f, 0.f}, dmul(d, dfl{r0, 0.f}));
  const dfl r = dadd(dfl{r0, 0.f}, dmul(dfl{r0, 0.f}, e));
  return cdf{dmul(a.x, r), dneg(dmul(a.y, r))};
}

// One (w, q) point: A = I - chi0 U from the non-zeros of U, LU with partial
// pivoting in the thread's shared-memory slice, then the nb^2 right-hand
// sides in registers. Returns the conditioning estimate
// (max_ij s_ij / min_j |U_jj|)^2, where s_ij = delta_ij + sum_m |chi0_im| |U_mj|
// is the size of the terms that formed A_ij (so cancellation in forming
// 1 - chi0 U counts as well as small pivots); it sends ill-conditioned points
// from double-float to FP64.
template <int NB, int NT, class E>
__device__ double rpa_point(const double2 *x, double2 *y, E *A, int *perm, const E *s_val, const int *s_off,
                            const int *s_cs, bool &singular) {
  constexpr int N = NB * NB;
#define AE(i, k) A[((i) * N + (k)) * NT]
  double amax = 0.0;
#pragma unroll
  for (int r = 0; r < N; ++r) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      E s = (r == c) ? el_one((E *)nullptr) : el_zero((E *)nullptr);
      float mag = (r == c) ? 1.f : 0.f;
      for (int t = s_cs[c]; t < s_cs[c + 1]; ++t) {
        const E xv = el_from(x[r * N + s_off[t]], (E *)nullptr);
        s = el_fms(xv, s_val[t], s);
        mag = fmaf(el_absf(xv), el_absf(s_val[t]), mag);
      }
      amax = fmax(amax, (double)mag * (double)mag);
      AE(r, c) = s;
    }
    perm[r * NT] = r;
  }
  double pmin = 1e300;
  singular = false;
#pragma unroll 1
  for (int j = 0; j < N; ++j) {
    int p = j;
    double best = el_abs2(AE(j, j));
#pragma unroll
    for (int i = 0; i < N; ++i) {
      if (i > j) {
        const double v = el_abs2(AE(i, j));
        if (v > best) {
          best = v;
          p = i;
        }
      }
    }
    if (best == 0.0) singular = true;
    pmin = fmin(pmin, best);
    if (p != j) {
#pragma unroll
      for (int k = 0; k < N; ++k) {
        const E t = AE(j, k);
        AE(j, k) = AE(p, k);
        AE(p, k) = t;
      }
      const int t = perm[j * NT];
      perm[j * NT] = perm[p * NT];
      perm[p * NT] = t;
    }
    const E inv = el_recip(AE(j, j));
    AE(j, j) = inv;
    E pr[N];
#pragma unroll
    for (int k = 0; k < N; ++k)
      if (k > j) pr[k] = AE(j, k);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      if (i > j) {
        const E f = cmul(AE(i, j), inv);
        AE(i, j) = f;
#pragma unroll
        for (int k = 0; k < N; ++k)
          if (k > j) AE(i, k) = el_fms(f, pr[k], AE(i, k));
      }
    }
  }
#pragma unroll 1
  for (int c = 0; c < N; ++c) {
    // An opaque zero added to the factor offsets keeps the compiler from
    // hoisting all N^2 factor loads out of this loop into registers.
    int z = 0;
    asm volatile("" : "+r"(z));
    const E *F = A + z;
    const int cm = colmap<NB>(c);
    E b[N];
#pragma unroll
    for (int r = 0; r < N; ++r) b[r] = el_from(x[perm[r * NT] * N + cm], (E *)nullptr);
#pragma unroll
    for (int r = 1; r < N; ++r)
#pragma unroll
      for (int l = 0; l < r; ++l) b[r] = el_fms(F[(r * N + l) * NT], b[l], b[r]);
#pragma unroll
    for (int rr = 0; rr < N; ++rr) {
      const int r = N - 1 - rr;
#pragma unroll
      for (int l = r + 1; l < N; ++l) b[r] = el_fms(F[(r * N + l) * NT], b[l], b[r]);
      b[r] = cmul(b[r], F[(r * N + r) * NT]);
    }
#pragma unroll
    for (int r = 0; r < N; ++r) y[r * N + cm] = el_to(b[r]);
  }
#undef AE
  return pmin > 0.0 ? amax / pmin : 1e300;
}

// Squared conditioning estimate above which a double-float solution is
// recomputed in FP64: (max|A| / min pivot)^2 > 1e4, i.e. the estimate > 100.
// Double-float carries ~2^-48 per operation, so below it the solve stays well
// inside 1e-10 relative; near an RPA instability (1 - chi0 U nearly singular)
// the point is solved in FP64.
constexpr double kDf64CondLimit2 = 1e4;

template <int NB, int NT, class E>
__global__ void __launch_bounds__(NT) rpa_lu_kernel(long n_points, const double2 *chi0, const double2 *__restrict__ U,
                                                    double2 *chi, unsigned *status) {
  constexpr int N = NB * NB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // Layout: [N*N] sparse U values (E), [N*N][NT] per-thread LU (16 B elements
  // of either type), [N*N] offsets, [N+1] column starts, [N][NT] permutations.
  E *s_val = reinterpret_cast<E *>(smem_raw);
  unsigned char *lu_base = smem_raw + (size_t)N * N * sizeof(E);
  int *s_off = reinterpret_cast<int *>(lu_base + (size_t)N * N * NT * 16);
  int *s_cs = s_off + N * N;
  int *perm = s_cs + N + 1 + threadIdx.x;
  // Sparse form of the grouped vertex Ug[m][c] = U[m][colmap(c)], column by
  // column: entry t of column c has grouped row m_t, kept as the offset
  // colmap(m_t) into a chi0 row. Exact zeros are dropped (the Kanamori vertex
  // keeps 21 of 81 entries for nb = 3). One thread builds it; it is tiny.
  if (threadIdx.x == 0) {
    int t = 0;
    for (int c = 0; c < N; ++c) {
      s_cs[c] = t;
      for (int m = 0; m < N; ++m) {
        const double2 u = U[m * N + colmap<NB>(c)];
        if (u.x != 0.0 || u.y != 0.0) {
          s_off[t] = colmap<NB>(m);
          s_val[t] = el_from(u, (E *)nullptr);
          ++t;
        }
      }
    }
    s_cs[N] = t;
  }
  __syncthreads();
  for (long base = blockIdx.x * (long)NT; base < n_points; base += (long)gridDim.x * NT) {
    const long pt = base + threadIdx.x;
    if (pt >= n_points) continue;
    const double2 *x = chi0 + pt * N * N;
    double2 *y = chi + pt * N * N;
    bool singular = false;
    const double cond2 = rpa_point<NB, NT, E>(x, y, reinterpret_cast<E *>(lu_base) + threadIdx.x, perm, s_val, s_off,
                                              s_cs, singular);
    if (IsDf<E>::value && !(cond2 <= kDf64CondLimit2)) {
      // FP64 re-solve of an ill-conditioned point, with U in FP64 from global memory
      double2 uval[N * N];
      for (int t = 0; t < s_cs[N]; ++t) {
        int c = 0;
        while (s_cs[c + 1] <= t) ++c;
        const int m = (s_off[t] % NB) * NB + s_off[t] / NB;  // colmap is an involution
        uval[t] = U[m * N + colmap<NB>(c)];
      }
      rpa_point<NB, NT, double2>(x, y, reinterpret_cast<double2 *>(lu_base) + threadIdx.x, perm, uval, s_off, s_cs,
                                 singular);
    }
    if (singular) atomicOr(status, kDevErrSingular);
  }
}

template <int NB, int NT, class E>
int launch_rpa_as(long n_points, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream,
                  unsigned *status) {
  constexpr int N = NB * NB;
  const size_t smem = (size_t)N * N * 16 * (1 + NT) + (size_t)(N * N + N + 1) * sizeof(int) +
                      (size_t)N * NT * sizeof(int);
  if (smem > (size_t)max_smem_optin()) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH: nb too large");
  TPRF_CUDA(cudaFuncSetAttribute(rpa_lu_kernel<NB, NT, E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  long blocks = (n_points + NT - 1) / NT;
  const long cap = (long)num_sms() * 64;
  blocks = std::max(1L, std::min(blocks, cap));
  rpa_lu_kernel<NB, NT, E><<<(unsigned)blocks, NT, smem, stream>>>(n_points, chi0, U, chi, status);
  TPRF_LAUNCH_CHECK("rpa_lu_kernel");
  return TPRF_OK;
}

template <int NB, int NT>
int launch_rpa_nb(long n_points, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream,
                  unsigned *status) {
  // One thread per point leaves one warp per scheduler: enough for the FP64
  // pipe, too few to hide double-float's dependent chains, so FP64 is the
  // default here and double-float only on request.
  if (arith_mode() == kArithDF64All) return launch_rpa_as<NB, NT, cdf>(n_points, chi0, U, chi, stream, status);
  return launch_rpa_as<NB, NT, double2>(n_points, chi0, U, chi, stream, status);
}

// ---------------------------------------------------------------------------
// Cooperative variant: T adjacent lanes solve one point together. The point's
// A / LU factors sit in one shared-memory slice ([element][point] layout); in
// each elimination step the T lanes split the pivot search, the row swap and
// the trailing update by rows, then split the nb^2 right-hand sides by
// columns. With the same shared memory per point as one thread per point,
// the CTA holds T times more warps, which hides the latency of the dependent
// double-float chains. Lanes of one point synchronise with __syncwarp on
// their own mask; all of them take the same branches (the same point, the
// same conditioning estimate), so no lane waits for an absent partner.
template <int NB, int T, int PPB, class E>
__device__ double rpa_point_coop(const double2 *x, double2 *y, E *A, int *perm, const E *s_val, const int *s_off,
                                 const int *s_cs, unsigned mask, int tq, bool &singular) {
  constexpr int N = NB * NB;
#define AE(i, k) A[((i) * N + (k)) * PPB]
  double amax = 0.0;
  for (int r = tq; r < N; r += T) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
      E s = (r == c) ? el_one((E *)nullptr) : el_zero((E *)nullptr);
      float mag = (r == c) ? 1.f : 0.f;
      for (int t = s_cs[c]; t < s_cs[c + 1]; ++t) {
        const E xv = el_from(x[r * N + s_off[t]], (E *)nullptr);
        s = el_fms(xv, s_val[t], s);
        mag = fmaf(el_absf(xv), el_absf(s_val[t]), mag);
      }
      amax = fmax(amax, (double)mag * (double)mag);
      AE(r, c) = s;
    }
    perm[r * PPB] = r;
  }
  __syncwarp(mask);
  double pmin = 1e300;
  bool sing = false;
#pragma unroll 1
  for (int j = 0; j < N; ++j) {
    // pivot search: this lane's rows, then the best over the T lanes
    int p = j;
    double best = -1.0;
    for (int i = j + tq; i < N; i += T) {
      const double v = el_abs2(AE(i, j));
      if (v > best) {
        best = v;
        p = i;
      }
    }
#pragma unroll
    for (int o = 1; o < T; o <<= 1) {
      const double ob = __shfl_xor_sync(mask, best, o);
      const int op = __shfl_xor_sync(mask, p, o);
      if (ob > best || (ob == best && op < p)) {
        best = ob;
        p = op;
      }
    }
    if (best == 0.0) sing = true;
    pmin = fmin(pmin, best);
    if (p != j) {
      for (int k = tq; k < N; k += T) {
        const E t = AE(j, k);
        AE(j, k) = AE(p, k);
        AE(p, k) = t;
      }
      if (tq == 0) {
        const int t = perm[j * PPB];
        perm[j * PPB] = perm[p * PPB];
        perm[p * PPB] = t;
      }
    }
    __syncwarp(mask);
    const E inv = el_recip(AE(j, j));
    // rows below j, split over the lanes
    for (int i = j + 1 + tq; i < N; i += T) {
      const E f = cmul(AE(i, j), inv);
      AE(i, j) = f;
#pragma unroll
      for (int k = 0; k < N; ++k)
        if (k > j) AE(i, k) = el_fms(f, AE(j, k), AE(i, k));
    }
    __syncwarp(mask);
    if (tq == 0) AE(j, j) = inv;
    __syncwarp(mask);
  }
  singular = sing;
  // right-hand sides: columns split over the lanes
  for (int c = tq; c < N; c += T) {
    int z = 0;
    asm volatile("" : "+r"(z));
    const E *F = A + z;
    const int cm = colmap<NB>(c);
    E b[N];
#pragma unroll
    for (int r = 0; r < N; ++r) b[r] = el_from(x[perm[r * PPB] * N + cm], (E *)nullptr);
#pragma unroll
    for (int r = 1; r < N; ++r)
#pragma unroll
      for (int l = 0; l < r; ++l) b[r] = el_fms(F[(r * N + l) * PPB], b[l], b[r]);
#pragma unroll
    for (int rr = 0; rr < N; ++rr) {
      const int r = N - 1 - rr;
#pragma unroll
      for (int l = r + 1; l < N; ++l) b[r] = el_fms(F[(r * N + l) * PPB], b[l], b[r]);
      b[r] = cmul(b[r], F[(r * N + r) * PPB]);
    }
#pragma unroll
    for (int r = 0; r < N; ++r) y[r * N + cm] = el_to(b[r]);
  }
  // every lane of the point returns the same estimate
#pragma unroll
  for (int o = 1; o < T; o <<= 1) amax = fmax(amax, __shfl_xor_sync(mask, amax, o));
  __syncwarp(mask);
#undef AE
  return pmin > 0.0 ? amax / pmin : 1e300;
}

template <int NB, int T, int PPB, class E>
__global__ void __launch_bounds__(T *PPB, 1) rpa_coop_kernel(long n_points, const double2 *chi0,
                                                            const double2 *__restrict__ U, double2 *chi,
                                                            unsigned *status) {
  constexpr int N = NB * NB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  E *s_val = reinterpret_cast<E *>(smem_raw);
  unsigned char *lu_base = smem_raw + (size_t)N * N * sizeof(E);
  int *s_off = reinterpret_cast<int *>(lu_base + (size_t)N * N * PPB * 16);
  int *s_cs = s_off + N * N;
  int *perm_base = s_cs + N + 1;
  if (threadIdx.x == 0) {
    int t = 0;
    for (int c = 0; c < N; ++c) {
      s_cs[c] = t;
      for (int m = 0; m < N; ++m) {
        const double2 u = U[m * N + colmap<NB>(c)];
        if (u.x != 0.0 || u.y != 0.0) {
          s_off[t] = colmap<NB>(m);
          s_val[t] = el_from(u, (E *)nullptr);
          ++t;
        }
      }
    }
    s_cs[N] = t;
  }
  __syncthreads();
  const int pidx = threadIdx.x / T, tq = threadIdx.x % T;
  const unsigned mask = (T == 32) ? 0xffffffffu : (((1u << T) - 1u) << ((threadIdx.x & 31) & ~(T - 1)));
  for (long base = blockIdx.x * (long)PPB; base < n_points; base += (long)gridDim.x * PPB) {
    const long pt = base + pidx;
    if (pt >= n_points) continue;  // all T lanes of this point skip together
    const double2 *x = chi0 + pt * N * N;
    double2 *y = chi + pt * N * N;
    bool singular = false;
    const double cond2 = rpa_point_coop<NB, T, PPB, E>(x, y, reinterpret_cast<E *>(lu_base) + pidx,
                                                       perm_base + pidx, s_val, s_off, s_cs, mask, tq, singular);
    if (IsDf<E>::value && !(cond2 <= kDf64CondLimit2)) {
      double2 uval[N * N];
      for (int t = 0; t < s_cs[N]; ++t) {
        int c = 0;
        while (s_cs[c + 1] <= t) ++c;
        const int m = (s_off[t] % NB) * NB + s_off[t] / NB;
        uval[t] = U[m * N + colmap<NB>(c)];
      }
      rpa_point_coop<NB, T, PPB, double2>(x, y, reinterpret_cast<double2 *>(lu_base) + pidx, perm_base + pidx, uval,
                                          s_off, s_cs, mask, tq, singular);
    }
    if (singular && tq == 0) atomicOr(status, kDevErrSingular);
  }
}

template <int NB, int T, int PPB, class E>
int launch_rpa_coop_as(long n_points, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream,
                       unsigned *status) {
  constexpr int N = NB * NB;
  const size_t smem = (size_t)N * N * 16 * (1 + PPB) + (size_t)(N * N + N + 1) * sizeof(int) +
                      (size_t)N * PPB * sizeof(int);
  if (smem > (size_t)max_smem_optin()) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH: nb too large");
  TPRF_CUDA(cudaFuncSetAttribute(rpa_coop_kernel<NB, T, PPB, E>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
  long blocks = (n_points + PPB - 1) / PPB;
  const long cap = (long)num_sms() * 64;
  blocks = std::max(1L, std::min(blocks, cap));
  rpa_coop_kernel<NB, T, PPB, E><<<(unsigned)blocks, T * PPB, smem, stream>>>(n_points, chi0, U, chi, status);
  TPRF_LAUNCH_CHECK("rpa_coop_kernel");
  return TPRF_OK;
}

}  // namespace

int launch_rpa(long n_points, int nb, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream) {
  unsigned *status = device_status_word();
  if (!status) return TPRF_ERR_CUDA;
  switch (nb) {
    case 1: return launch_rpa_nb<1, 256>(n_points, chi0, U, chi, stream, status);
    case 2: return launch_rpa_nb<2, 256>(n_points, chi0, U, chi, stream, status);
    case 3:
      if (arith_mode() == kArithFP64) return launch_rpa_coop_as<3, 4, 128, double2>(n_points, chi0, U, chi, stream, status);
      return launch_rpa_coop_as<3, 4, 128, cdf>(n_points, chi0, U, chi, stream, status);
    case 4: return launch_rpa_nb<4, 32>(n_points, chi0, U, chi, stream, status);
    case 5: return launch_rpa_nb<5, 16>(n_points, chi0, U, chi, stream, status);
    default: return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH: nb must be 1..5");
  }
}

}  // namespace tprf

extern "C" int tprf_solve_rpa_PH(long n_points, int nb, const double *chi0, const double *U, double *chi,
                                 void *stream) {
  using namespace tprf;
  if (n_points < 1 || !chi0 || !U || !chi)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH: bad shape or null pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = launch_rpa(n_points, nb, reinterpret_cast<const double2 *>(chi0), reinterpret_cast<const double2 *>(U),
                      reinterpret_cast<double2 *>(chi), s);
  if (st) return st;
  return finish_with_checks(s, "solve_rpa_PH");
}

// ---- adjoint (differentiable path) ----------------------------------------------
// chi = A^-1 chi0 with A = I - chi0 U (PH-grouped matrices) gives
// d chi = A^-1 d chi0 (I + U chi) + chi dU chi. For a real loss with gradient
// Y = dL/d chi (conjugate Wirtinger convention): chi0_grad = A^-H Y (I + U chi)^H
// and U_grad = sum over points of chi^H Y chi^H. One thread per point, FP64;
// U_grad is accumulated with atomics into a caller-zeroed [nb^4] buffer.

namespace tprf {
namespace {

template <int NB>
__global__ void __launch_bounds__(128) rpa_adjoint_kernel(long n_points, const double2 *__restrict__ chi0,
                                                          const double2 *__restrict__ Uin,
                                                          const double2 *__restrict__ chi,
                                                          const double2 *__restrict__ chig,
                                                          double2 *__restrict__ chi0g, double2 *Ug, unsigned *status) {
  constexpr int N = NB * NB;
  __shared__ double2 Us[N * N];
  __shared__ double Uacc[2 * N * N];
  for (int w = threadIdx.x; w < N * N; w += blockDim.x) {
    Us[w] = Uin[(w / N) * N + colmap<NB>(w % N)];
    Uacc[2 * w] = Uacc[2 * w + 1] = 0.0;
  }
  __syncthreads();
  double2 ug[N][N];
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) ug[i][j] = make_double2(0.0, 0.0);
  for (long pt = blockIdx.x * (long)blockDim.x + threadIdx.x; pt < n_points; pt += (long)gridDim.x * blockDim.x) {
    const long o = pt * N * N;
    double2 A[N][N], Y[N][N], X[N][N];
    // A^H = I - U^H chi0^H, solved with partial pivoting: A^H Z = Y
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
      for (int j = 0; j < N; ++j) {
        double2 s = make_double2(i == j ? 1.0 : 0.0, 0.0);
#pragma unroll
        for (int m = 0; m < N; ++m) s = cfms(cconj(Us[m * N + i]), cconj(chi0[o + j * N + colmap<NB>(m)]), s);
        A[i][j] = s;
        Y[i][j] = chig[o + i * N + colmap<NB>(j)];
        X[i][j] = chi[o + i * N + colmap<NB>(j)];
      }
    bool singular = false;
#pragma unroll
    for (int j = 0; j < N; ++j) {
      int p = j;
      double best = cabs2(A[j][j]);
#pragma unroll
      for (int i = j + 1; i < N; ++i)
        if (cabs2(A[i][j]) > best) {
          best = cabs2(A[i][j]);
          p = i;
        }
      if (best == 0.0) singular = true;
#pragma unroll
      for (int i = j + 1; i < N; ++i)
        if (i == p) {
#pragma unroll
          for (int k = 0; k < N; ++k) {
            double2 t = A[i][k];
            A[i][k] = A[j][k];
            A[j][k] = t;
            t = Y[i][k];
            Y[i][k] = Y[j][k];
            Y[j][k] = t;
          }
        }
      const double2 inv = crecip(A[j][j]);
      A[j][j] = inv;
#pragma unroll
      for (int i = j + 1; i < N; ++i) {
        const double2 f = cmul(A[i][j], inv);
#pragma unroll
        for (int k = j + 1; k < N; ++k) A[i][k] = cfms(f, A[j][k], A[i][k]);
#pragma unroll
        for (int k = 0; k < N; ++k) Y[i][k] = cfms(f, Y[j][k], Y[i][k]);
      }
    }
#pragma unroll
    for (int jj = 0; jj < N; ++jj) {
      const int j = N - 1 - jj;
#pragma unroll
      for (int k = 0; k < N; ++k) {
        double2 s = Y[j][k];
#pragma unroll
        for (int l = j + 1; l < N; ++l) s = cfms(A[j][l], Y[l][k], s);
        Y[j][k] = cmul(s, A[j][j]);
      }
    }
    if (singular) atomicOr(status, kDevErrSingular);
    // B = I + U chi; chi0_grad = Z B^H
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
      for (int j = 0; j < N; ++j) {
        // (B^H)_{l j} = conj(B_{j l}) = delta + conj(sum_m U_{j m} chi_{m l})
        double2 s = make_double2(0.0, 0.0);
#pragma unroll
        for (int l = 0; l < N; ++l) {
          double2 bjl = make_double2(j == l ? 1.0 : 0.0, 0.0);
#pragma unroll
          for (int m = 0; m < N; ++m) bjl = cfma(Us[j * N + m], X[m][l], bjl);
          s = cfma(Y[i][l], cconj(bjl), s);
        }
        chi0g[o + i * N + colmap<NB>(j)] = s;
      }
    // U_grad += chi^H Y_in chi^H (Y_in re-read: Y now holds Z)
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
      for (int j = 0; j < N; ++j) {
        double2 s = make_double2(0.0, 0.0);
#pragma unroll
        for (int l = 0; l < N; ++l) {
          double2 t = make_double2(0.0, 0.0);  // (Y chi^H)_{l j}
#pragma unroll
          for (int m = 0; m < N; ++m) t = cfma(chig[o + l * N + colmap<NB>(m)], cconj(X[j][m]), t);
          s = cfma(cconj(X[l][i]), t, s);
        }
        ug[i][j] = cadd(ug[i][j], s);
      }
  }
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) {
      atomicAdd(&Uacc[2 * (i * N + j)], ug[i][j].x);
      atomicAdd(&Uacc[2 * (i * N + j) + 1], ug[i][j].y);
    }
  __syncthreads();
  for (int w = threadIdx.x; w < N * N; w += blockDim.x) {
    // grouped (m, c) -> tensor offset m * N + colmap(c)
    const int off = (w / N) * N + colmap<NB>(w % N);
    atomicAdd(&reinterpret_cast<double *>(Ug)[2 * off], Uacc[2 * w]);
    atomicAdd(&reinterpret_cast<double *>(Ug)[2 * off + 1], Uacc[2 * w + 1]);
  }
}

template <int NB>
int launch_rpa_adjoint_nb(long n_points, const double2 *chi0, const double2 *U, const double2 *chi,
                          const double2 *chig, double2 *chi0g, double2 *Ug, cudaStream_t s, unsigned *status) {
  long blocks = (n_points + 127) / 128;
  blocks = std::max(1L, std::min(blocks, (long)num_sms() * 8));
  rpa_adjoint_kernel<NB><<<(unsigned)blocks, 128, 0, s>>>(n_points, chi0, U, chi, chig, chi0g, Ug, status);
  TPRF_LAUNCH_CHECK("rpa_adjoint_kernel");
  return TPRF_OK;
}

}  // namespace
}  // namespace tprf

extern "C" int tprf_solve_rpa_PH_adjoint(long n_points, int nb, const double *chi0, const double *U, const double *chi,
                                         const double *chi_grad, double *chi0_grad, double *U_grad, void *stream) {
  using namespace tprf;
  if (n_points < 1 || !chi0 || !U || !chi || !chi_grad || !chi0_grad || !U_grad)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH_adjoint: bad shape or null pointer");
  unsigned *status = device_status_word();
  if (!status) return TPRF_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto c = [](const double *p) { return reinterpret_cast<const double2 *>(p); };
  double2 *g0 = reinterpret_cast<double2 *>(chi0_grad), *ug = reinterpret_cast<double2 *>(U_grad);
  int st;
  switch (nb) {
    case 1: st = launch_rpa_adjoint_nb<1>(n_points, c(chi0), c(U), c(chi), c(chi_grad), g0, ug, s, status); break;
    case 2: st = launch_rpa_adjoint_nb<2>(n_points, c(chi0), c(U), c(chi), c(chi_grad), g0, ug, s, status); break;
    case 3: st = launch_rpa_adjoint_nb<3>(n_points, c(chi0), c(U), c(chi), c(chi_grad), g0, ug, s, status); break;
    default: return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH_adjoint: nb must be 1..3");
  }
  if (st) return st;
  return finish_with_checks(s, "solve_rpa_PH_adjoint");
}
