// Kernel (d): the RPA solve chi = [I - chi0 U]^-1 chi0 per (omega, q) point.
//
// Restates c++/triqs_tprf/lattice/rpa.cpp:29-64: chi0 and U are grouped into
// nb^2 x nb^2 matrices with rows (a, b) and columns (d, c)
// (idx_group<0,1>, idx_group<3,2>, rpa.cpp:40,54-55) and
// chi = inverse(I - chi0 * U) * chi0 (rpa.cpp:57). Here the same system is
// solved without forming the inverse: A = I - chi0 U, then Gaussian
// elimination with partial pivoting on [A | chi0] and back substitution.
//
// Kernels by vertex size: nb = 1, 2 one thread per point (below); nb >= 3 a
// group of lanes per point (rpa_warp.cu, which also holds the adjoint).
//
// Design of the thread-per-point kernel: A = I - chi0 U is formed from the non-zeros of
// U only (compacted once per CTA into shared memory), LU-factorised with
// partial pivoting in the thread's slice of shared memory ([element][thread]
// layout: conflict-free although every thread pivots independently), and the
// nb^2 right-hand sides (columns of chi0, re-read from L1/L2 through the row
// permutation) are solved one at a time in registers. Keeping only the LU
// factors in shared memory halves the per-thread footprint of a full
// [A | chi0] elimination, which doubles the warps per SM.
#include <algorithm>
#include <cstdint>
#include <mutex>

#include "rpa_common.cuh"

namespace tprf {
namespace {

// One (w, q) point: A = I - chi0 U from the non-zeros of U, LU with partial
// pivoting in the thread's shared-memory slice, then the nb^2 right-hand
// sides in registers. Returns the conditioning estimate
// (max_ij s_ij / min_j |U_jj|)^2, where s_ij = delta_ij + sum_m |chi0_im| |U_mj|
// is the size of the terms that formed A_ij (so cancellation in forming
// 1 - chi0 U counts as well as small pivots); it sends ill-conditioned points
// from double-float to FP64.
template <int NB, int NT, class E>
__device__ double rpa_point(const double2 *x, double2 *y, E *A, int *perm, const E *s_val, const int *s_off,
                            const int *s_cs, bool &singular, double2 *y_conj = nullptr) {
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
    for (int r = 0; r < N; ++r) {
      const double2 v = el_to(b[r]);
      y[r * N + cm] = v;
      if (y_conj) y_conj[r * N + cm] = make_double2(v.x, -v.y);  // the conjugate system's solve
    }
  }
#undef AE
  return pmin > 0.0 ? amax / pmin : 1e300;
}


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

// Conjugate point pairs on a bosonic (w, q) mesh, one thread per unit (the
// pairing of rpa_pair_kernel in rpa_warp.cu): with U real and chi0(-w, -q) bit
// for bit conj(chi0(w, q)), the pair is solved once and both results stored.
template <int NB, int NT, class E>
__global__ void __launch_bounds__(NT) rpa_lu_pair_kernel(int nw, int d0, int d1, int d2, const double2 *chi0,
                                                         const double2 *__restrict__ U, PairOut out,
                                                         unsigned *status) {
  constexpr int N = NB * NB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  E *s_val = reinterpret_cast<E *>(smem_raw);
  unsigned char *lu_base = smem_raw + (size_t)N * N * sizeof(E);
  int *s_off = reinterpret_cast<int *>(lu_base + (size_t)N * N * NT * 16);
  int *s_cs = s_off + N * N;
  int *perm = s_cs + N + 1 + threadIdx.x;
  __shared__ int s_ureal;
  if (threadIdx.x == 0) {
    int t = 0, ureal = 1;
    for (int c = 0; c < N; ++c) {
      s_cs[c] = t;
      for (int m = 0; m < N; ++m) {
        const double2 u = U[m * N + colmap<NB>(c)];
        if (u.y != 0.0) ureal = 0;
        if (u.x != 0.0 || u.y != 0.0) {
          s_off[t] = colmap<NB>(m);
          s_val[t] = el_from(u, (E *)nullptr);
          ++t;
        }
      }
    }
    s_cs[N] = t;
    s_ureal = ureal;
  }
  __syncthreads();
  const bool ureal = s_ureal != 0;
  const long nk = (long)d0 * d1 * d2, units = (long)(out.mh1 - out.mh0) * nk;
  for (long un = blockIdx.x * (long)NT + threadIdx.x; un < units; un += (long)gridDim.x * NT) {
    const int mh = out.mh0 + (int)(un / nk);
    const long q = un - (long)(mh - out.mh0) * nk;
    const int q2 = (int)(q % d2), q1 = (int)((q / d2) % d1), q0 = (int)(q / ((long)d2 * d1));
    const long mq = ((long)((d0 - q0) % d0) * d1 + (d1 - q1) % d1) * d2 + (d2 - q2) % d2;
    if (mh == 0 && q > mq) continue;  // its partner (0, -q) holds this unit
    const long p = (long)(nw - 1 + mh) * nk + q, pm = (long)(nw - 1 - mh) * nk + mq;
    bool sym = ureal && pm != p;
    for (int o = 0; o < N * N && sym; ++o) {
      const double2 a = chi0[p * N * N + o], b = chi0[pm * N * N + o];
      sym = __double_as_longlong(a.x) == __double_as_longlong(b.x) &&
            __double_as_longlong(a.y) == __double_as_longlong(-b.y);
    }
    double2 *yp = out.pos + (long)(mh - out.mh0) * out.row + q * N * N;
    double2 *ypm = (mh == 0 ? out.pos + (long)(mh - out.mh0) * out.row : out.neg + (long)(mh - out.mh0) * out.neg_step) +
                   mq * N * N;
    for (int k = 0; k < 2; ++k) {
      if (k == 1 && (pm == p || sym)) break;
      const long pt = k ? pm : p;
      const double2 *x = chi0 + pt * N * N;
      double2 *y = k ? ypm : yp;
      double2 *yc = (k == 0 && sym) ? ypm : nullptr;
      bool singular = false;
      const double cond2 = rpa_point<NB, NT, E>(x, y, reinterpret_cast<E *>(lu_base) + threadIdx.x, perm, s_val,
                                                s_off, s_cs, singular, yc);
      if (IsDf<E>::value && !(cond2 <= kDf64CondLimit2)) {
        double2 uval[N * N];
        for (int t = 0; t < s_cs[N]; ++t) {
          int c = 0;
          while (s_cs[c + 1] <= t) ++c;
          const int m = (s_off[t] % NB) * NB + s_off[t] / NB;
          uval[t] = U[m * N + colmap<NB>(c)];
        }
        rpa_point<NB, NT, double2>(x, y, reinterpret_cast<double2 *>(lu_base) + threadIdx.x, perm, uval, s_off, s_cs,
                                   singular, yc);
      }
      if (singular) atomicOr(status, kDevErrSingular);
    }
  }
}

template <int NB, int NT, class E>
int launch_rpa_pair_as(int nw, const int dims[3], const double2 *chi0, const double2 *U, PairOut out,
                       cudaStream_t stream, unsigned *status) {
  constexpr int N = NB * NB;
  const size_t smem = (size_t)N * N * 16 * (1 + NT) + (size_t)(N * N + N + 1) * sizeof(int) +
                      (size_t)N * NT * sizeof(int);
  auto kern = rpa_lu_pair_kernel<NB, NT, E>;
  TPRF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const long units = (long)(out.mh1 - out.mh0) * dims[0] * dims[1] * dims[2];
  long blocks = (units + NT - 1) / NT;
  blocks = std::max(1L, std::min(blocks, (long)num_sms() * 64));
  kern<<<(unsigned)blocks, NT, smem, stream>>>(nw, dims[0], dims[1], dims[2], chi0, U, out, status);
  TPRF_KERNEL_LAUNCHED("rpa_lu_pair_kernel");
  return TPRF_OK;
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
  TPRF_KERNEL_LAUNCHED("rpa_lu_kernel");
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

}  // namespace

int launch_rpa_warp(long n_points, int nb, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream,
                    unsigned *status);

int launch_rpa(long n_points, int nb, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream) {
  unsigned *status = device_status_word();
  if (!status) return TPRF_ERR_CUDA;
  switch (nb) {
    case 1: return launch_rpa_nb<1, 256>(n_points, chi0, U, chi, stream, status);
    case 2: return launch_rpa_nb<2, 256>(n_points, chi0, U, chi, stream, status);
    default:
      if (nb < 1 || nb > 8) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH: nb must be 1..8");
      return launch_rpa_warp(n_points, nb, chi0, U, chi, stream, status);
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

// ---- RPA on a (w, q) mesh with conjugate pairs ----------------------------------------
namespace tprf {
int launch_rpa_warp_pairs(int nw, const int dims[3], int nb, const double2 *chi0, const double2 *U, PairOut out,
                          cudaStream_t stream, unsigned *status);

int launch_rpa_wk_block(int nw, const int dims[3], int nb, const double2 *chi0, const double2 *U, PairOut out,
                        cudaStream_t stream) {
  unsigned *status = device_status_word();
  if (!status) return TPRF_ERR_CUDA;
  if (nb < 1 || nb > 8) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH: nb must be 1..8");
  if (out.mh0 < 0 || out.mh1 > nw || out.mh0 >= out.mh1)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH: bad frequency range");
  const bool df = arith_mode() == kArithDF64All;  // as the point form: FP64 unless double-float everywhere
  if (nb == 1)
    return df ? launch_rpa_pair_as<1, 256, cdf>(nw, dims, chi0, U, out, stream, status)
              : launch_rpa_pair_as<1, 256, double2>(nw, dims, chi0, U, out, stream, status);
  if (nb == 2)
    return df ? launch_rpa_pair_as<2, 256, cdf>(nw, dims, chi0, U, out, stream, status)
              : launch_rpa_pair_as<2, 256, double2>(nw, dims, chi0, U, out, stream, status);
  return launch_rpa_warp_pairs(nw, dims, nb, chi0, U, out, stream, status);
}

int launch_rpa_wk(int nw, const int dims[3], int nb, const double2 *chi0, const double2 *U, double2 *chi,
                  cudaStream_t stream) {
  const long row = (long)dims[0] * dims[1] * dims[2] * nb * nb * nb * nb;
  const PairOut out{chi + (long)(nw - 1) * row, chi + (long)(nw - 1) * row, row, -row, 0, nw};
  return launch_rpa_wk_block(nw, dims, nb, chi0, U, out, stream);
}
}  // namespace tprf

extern "C" int tprf_solve_rpa_PH_wk(int nw, const int dims[3], int nb, const double *chi0, const double *U,
                                    double *chi, void *stream) {
  using namespace tprf;
  if (nw < 1 || !dims || dims[0] < 1 || dims[1] < 1 || dims[2] < 1 || !chi0 || !U || !chi)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH_wk: bad mesh or null pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = launch_rpa_wk(nw, dims, nb, reinterpret_cast<const double2 *>(chi0), reinterpret_cast<const double2 *>(U),
                         reinterpret_cast<double2 *>(chi), s);
  if (st) return st;
  return finish_with_checks(s, "solve_rpa_PH");
}

// ---- RPA with the result streamed to host memory -----------------------------------
// The reference returns chi as a host-side gf. Here the points are solved in chunks
// into a small device ring (the caller's workspace) and each chunk is copied to the
// host buffer on a second stream while the next chunk is solved, so the copy of the
// result (the largest transfer of the path) overlaps the RPA arithmetic. The caller's
// stream waits for the last copy: a synchronisation of `stream` means chi is on the host.
namespace tprf {
namespace {
constexpr int kMaxRingSlots = 16;
constexpr int kMaxDevices = 64;

struct HostOutCtx {
  bool ready = false;
  cudaStream_t copy = nullptr;
  cudaEvent_t computed[kMaxRingSlots], copied[kMaxRingSlots], done;
};
std::mutex g_host_out_mu;
HostOutCtx g_host_out[kMaxDevices];

int host_out_ctx(HostOutCtx **out) {
  int dev = 0;
  TPRF_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH_to_host: device id");
  HostOutCtx &c = g_host_out[dev];
  if (!c.ready) {
    TPRF_CUDA(cudaStreamCreateWithFlags(&c.copy, cudaStreamNonBlocking));
    for (int i = 0; i < kMaxRingSlots; ++i) {
      TPRF_CUDA(cudaEventCreateWithFlags(&c.computed[i], cudaEventDisableTiming));
      TPRF_CUDA(cudaEventCreateWithFlags(&c.copied[i], cudaEventDisableTiming));
    }
    TPRF_CUDA(cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming));
    c.ready = true;
  }
  *out = &c;
  return TPRF_OK;
}
}  // namespace
}  // namespace tprf

extern "C" size_t tprf_solve_rpa_PH_to_host_workspace_bytes(long chunk_points, int nb, int slots) {
  if (chunk_points < 1 || nb < 1 || slots < 1) return 0;
  return (size_t)slots * (size_t)chunk_points * (size_t)nb * nb * nb * nb * sizeof(double2) + 256;
}

extern "C" int tprf_solve_rpa_PH_to_host(long n_points, int nb, const double *chi0, const double *U, double *chi_host,
                                         long chunk_points, void *workspace, size_t workspace_bytes, void *stream) {
  using namespace tprf;
  if (n_points < 1 || chunk_points < 1 || nb < 1 || !chi0 || !U || !chi_host || !workspace)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH_to_host: bad shape or null pointer");
  const size_t per_point = (size_t)nb * nb * nb * nb;
  const size_t slot_bytes = (size_t)chunk_points * per_point * sizeof(double2);
  const uintptr_t base = (reinterpret_cast<uintptr_t>(workspace) + 255) & ~(uintptr_t)255;
  const size_t usable = workspace_bytes > (base - reinterpret_cast<uintptr_t>(workspace))
                            ? workspace_bytes - (base - reinterpret_cast<uintptr_t>(workspace))
                            : 0;
  const int slots = (int)std::min<size_t>(kMaxRingSlots, usable / slot_bytes);
  if (slots < 1)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH_to_host: workspace smaller than one chunk");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> lock(g_host_out_mu);
  HostOutCtx *c = nullptr;
  int st = host_out_ctx(&c);
  if (st) return st;
  const double2 *src = reinterpret_cast<const double2 *>(chi0);
  const double2 *u = reinterpret_cast<const double2 *>(U);
  double2 *host = reinterpret_cast<double2 *>(chi_host);
  const long n_chunks = (n_points + chunk_points - 1) / chunk_points;
  for (long k = 0; k < n_chunks; ++k) {
    const int slot = (int)(k % slots);
    const long p0 = k * chunk_points, np = std::min(chunk_points, n_points - p0);
    double2 *ring = reinterpret_cast<double2 *>(base + (size_t)slot * slot_bytes);
    if (k >= slots) TPRF_CUDA(cudaStreamWaitEvent(s, c->copied[slot], 0));  // the slot's last copy is done
    st = launch_rpa(np, nb, src + (size_t)p0 * per_point, u, ring, s);
    if (st) {
      // let the caller's stream wait for what was already queued, then report
      cudaEventRecord(c->done, c->copy);
      cudaStreamWaitEvent(s, c->done, 0);
      return st;
    }
    TPRF_CUDA(cudaEventRecord(c->computed[slot], s));
    TPRF_CUDA(cudaStreamWaitEvent(c->copy, c->computed[slot], 0));
    TPRF_CUDA(cudaMemcpyAsync(host + (size_t)p0 * per_point, ring, (size_t)np * per_point * sizeof(double2),
                              cudaMemcpyDeviceToHost, c->copy));
    TPRF_CUDA(cudaEventRecord(c->copied[slot], c->copy));
  }
  TPRF_CUDA(cudaEventRecord(c->done, c->copy));
  TPRF_CUDA(cudaStreamWaitEvent(s, c->done, 0));
  return finish_with_checks(s, "solve_rpa_PH_to_host");
}

// ---- adjoint (differentiable path) ------------------------------------------------
// nb = 1, 2: one thread per point (below); nb >= 3: the warp-per-point kernel of
// rpa_warp.cu. With the grouped matrices X0 (chi0), X (chi), Y (the gradient
// dL/d conj(chi)) and Ug, and A = I - X0 Ug (so X = A^-1 X0):
//   Z = A^-H Y,  P = Z X^H,
//   chi0_grad = Z (I + Ug X)^H = Z + P Ug^H,
//   U_grad    = sum over points of X0^H P  (= X^H Y X^H).
namespace tprf {
namespace {

__device__ __forceinline__ double2 ad_fma(double2 a, double2 b, double2 acc) { return cfma(a, b, acc); }
__device__ __forceinline__ cdf ad_fma(cdf a, cdf b, cdf acc) { return cfma_df(a, b, acc); }

// The thread-per-point adjoint needs no factorisation: A^-1 = (I - X0 Ug)^-1 =
// I + X Ug (push-through, X = A^-1 X0), so Z = A^-H Y = Y + Ug^H (X^H Y). Then
// P = Z X^H row by row, each row used at once by chi0_grad = Z + P Ug^H and by
// U_grad += X0^H P (row i of P meets row i of X0). Products only, with
// independent accumulators: double-float on the FP32 pipe by default (native
// FP64 in the FP64 mode), FP64 at the boundary.
template <int NB, int NT, class E>
__global__ void __launch_bounds__(NT) rpa_adjoint_point_kernel(long n_points, const double2 *chi0,
                                                               const double2 *__restrict__ U, const double2 *chi,
                                                               const double2 *chig, double2 *chi0g, double2 *Ug_out) {
  constexpr int N = NB * NB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // Layout: [N*N] grouped U, then per thread ([element][thread]: conflict-free)
  // the U_grad partial sums and conj(X) in the element type.
  E *ug = reinterpret_cast<E *>(smem_raw);
  E *acc = ug + N * N;
  E *xs = acc + N * N * NT;
  const int tid = threadIdx.x;
  for (int e = tid; e < N * N; e += NT) ug[e] = el_from(U[(e / N) * N + colmap<NB>(e % N)], (E *)nullptr);
#pragma unroll
  for (int e = 0; e < N * N; ++e) acc[e * NT + tid] = el_zero((E *)nullptr);
  __syncthreads();
#define ACC(i, k) acc[((i) * N + (k)) * NT + tid]
#define XC(i, k) xs[((i) * N + (k)) * NT + tid]
  for (long pt = blockIdx.x * (long)NT + tid; pt < n_points; pt += (long)gridDim.x * NT) {
    const double2 *x0 = chi0 + pt * N * N, *x = chi + pt * N * N, *y = chig + pt * N * N;
    // W = X^H Y, one row of X and Y at a time (conj(X) kept for P)
    E W[N][N];
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
      for (int j = 0; j < N; ++j) W[i][j] = el_zero((E *)nullptr);
#pragma unroll
    for (int l = 0; l < N; ++l) {
      E xr[N], yr[N];
#pragma unroll
      for (int m = 0; m < N; ++m) {
        xr[m] = cconj(el_from(x[l * N + colmap<NB>(m)], (E *)nullptr));
        yr[m] = el_from(y[l * N + colmap<NB>(m)], (E *)nullptr);
        XC(l, m) = xr[m];
      }
#pragma unroll
      for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j) W[i][j] = ad_fma(xr[i], yr[j], W[i][j]);
    }
    // Z = Y + Ug^H W
    E Z[N][N];
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
      for (int j = 0; j < N; ++j) {
        E s = el_from(y[i * N + colmap<NB>(j)], (E *)nullptr);
#pragma unroll
        for (int m = 0; m < N; ++m) s = ad_fma(cconj(ug[m * N + i]), W[m][j], s);
        Z[i][j] = s;
      }
    double2 *g = chi0g + pt * N * N;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      E pr[N];  // row i of P = Z X^H
#pragma unroll
      for (int m = 0; m < N; ++m) {
        E s = el_zero((E *)nullptr);
#pragma unroll
        for (int l = 0; l < N; ++l) s = ad_fma(Z[i][l], XC(m, l), s);
        pr[m] = s;
      }
#pragma unroll
      for (int j = 0; j < N; ++j) {
        E s = Z[i][j];
#pragma unroll
        for (int m = 0; m < N; ++m) s = ad_fma(pr[m], cconj(ug[j * N + m]), s);
        g[i * N + colmap<NB>(j)] = el_to(s);
      }
#pragma unroll
      for (int k = 0; k < N; ++k) {
        const E xk = cconj(el_from(x0[i * N + colmap<NB>(k)], (E *)nullptr));
#pragma unroll
        for (int j = 0; j < N; ++j) ACC(k, j) = ad_fma(xk, pr[j], ACC(k, j));
      }
    }
  }
#undef ACC
#undef XC
  __syncthreads();
  // CTA sum of the partials, one atomic per entry: grouped (m, c) -> offset m * N + colmap(c)
  for (int e = tid; e < N * N; e += NT) {
    E s = el_zero((E *)nullptr);
    for (int t = 0; t < NT; ++t) s = cadd(s, acc[e * NT + t]);
    const double2 v = el_to(s);
    const int off = (e / N) * N + colmap<NB>(e % N);
    atomicAdd(&reinterpret_cast<double *>(Ug_out)[2 * off], v.x);
    atomicAdd(&reinterpret_cast<double *>(Ug_out)[2 * off + 1], v.y);
  }
}

template <int NB, class E>
int launch_rpa_adjoint_point_as(long n_points, const double2 *chi0, const double2 *U, const double2 *chi,
                                const double2 *chig, double2 *chi0g, double2 *Ug, cudaStream_t stream) {
  constexpr int N = NB * NB, NT = 128;
  const size_t smem = (size_t)N * N * 16 * (1 + 2 * NT);
  auto kern = rpa_adjoint_point_kernel<NB, NT, E>;
  TPRF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  TPRF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem));
  long blocks = (n_points + NT - 1) / NT;
  blocks = std::max(1L, std::min(blocks, (long)num_sms() * std::max(1, per_sm)));
  kern<<<(unsigned)blocks, NT, smem, stream>>>(n_points, chi0, U, chi, chig, chi0g, Ug);
  TPRF_KERNEL_LAUNCHED("rpa_adjoint_point_kernel");
  return TPRF_OK;
}

template <int NB>
int launch_rpa_adjoint_point(long n_points, const double2 *chi0, const double2 *U, const double2 *chi,
                             const double2 *chig, double2 *chi0g, double2 *Ug, cudaStream_t stream, unsigned *) {
  return arith_mode() == kArithFP64
             ? launch_rpa_adjoint_point_as<NB, double2>(n_points, chi0, U, chi, chig, chi0g, Ug, stream)
             : launch_rpa_adjoint_point_as<NB, cdf>(n_points, chi0, U, chi, chig, chi0g, Ug, stream);
}

}  // namespace

int launch_rpa_adjoint_warp(long n_points, int nb, const double2 *chi0, const double2 *U, const double2 *chi,
                            const double2 *chig, double2 *chi0g, double2 *Ug, cudaStream_t stream, unsigned *status);

// The RPA adjoint by vertex size (U_grad is accumulated: the caller zeroes it).
int launch_rpa_adjoint(long n_points, int nb, const double2 *chi0, const double2 *U, const double2 *chi,
                       const double2 *chig, double2 *chi0g, double2 *Ug, cudaStream_t stream, unsigned *status) {
  switch (nb) {
    case 1: return launch_rpa_adjoint_point<1>(n_points, chi0, U, chi, chig, chi0g, Ug, stream, status);
    case 2: return launch_rpa_adjoint_point<2>(n_points, chi0, U, chi, chig, chi0g, Ug, stream, status);
    default:
      if (nb < 1 || nb > 8) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH_adjoint: nb must be 1..8");
      return launch_rpa_adjoint_warp(n_points, nb, chi0, U, chi, chig, chi0g, Ug, stream, status);
  }
}

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
  const int st = launch_rpa_adjoint(n_points, nb, c(chi0), c(U), c(chi), c(chi_grad), g0, ug, s, status);
  if (st) return st;
  return finish_with_checks(s, "solve_rpa_PH_adjoint");
}
