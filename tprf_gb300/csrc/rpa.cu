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

template <int NB, int NT>
__global__ void __launch_bounds__(NT) rpa_lu_kernel(long n_points, const double2 *chi0, const double2 *__restrict__ U,
                                                    double2 *chi, unsigned *status) {
  constexpr int N = NB * NB;
  extern __shared__ double2 smem[];
  double2 *s_val = smem;                                     // [nnz] non-zeros of the grouped U
  double2 *A = smem + N * N + threadIdx.x;                   // per thread LU, [N*N][NT]
  int *s_off = reinterpret_cast<int *>(smem + N * N + (size_t)N * N * NT);  // [nnz]
  int *s_cs = s_off + N * N;                                 // [N + 1] column starts
  int *perm = s_cs + N + 1 + threadIdx.x;                    // per thread row permutation, [N][NT]
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
          s_val[t] = u;
          ++t;
        }
      }
    }
    s_cs[N] = t;
  }
  __syncthreads();
#define AE(i, k) A[((i) * N + (k)) * NT]
  for (long base = blockIdx.x * (long)NT; base < n_points; base += (long)gridDim.x * NT) {
    const long pt = base + threadIdx.x;
    if (pt >= n_points) continue;
    const double2 *x = chi0 + pt * N * N;
    // A = I - chi0 U over the non-zeros of U
#pragma unroll
    for (int r = 0; r < N; ++r) {
#pragma unroll
      for (int c = 0; c < N; ++c) {
        double2 s = make_double2(r == c ? 1.0 : 0.0, 0.0);
        for (int t = s_cs[c]; t < s_cs[c + 1]; ++t) s = cfms(x[r * N + s_off[t]], s_val[t], s);
        AE(r, c) = s;
      }
      perm[r * NT] = r;
    }
    // LU with partial pivoting; the step loop stays rolled so that the factors
    // live in shared memory, not in registers.
    bool singular = false;
#pragma unroll 1
    for (int j = 0; j < N; ++j) {
      int p = j;
      double best = cabs2(AE(j, j));
#pragma unroll
      for (int i = 0; i < N; ++i) {
        if (i > j) {
          const double v = cabs2(AE(i, j));
          if (v > best) {
            best = v;
            p = i;
          }
        }
      }
      if (best == 0.0) singular = true;
      if (p != j) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
          const double2 t = AE(j, k);
          AE(j, k) = AE(p, k);
          AE(p, k) = t;
        }
        const int t = perm[j * NT];
        perm[j * NT] = perm[p * NT];
        perm[p * NT] = t;
      }
      const double2 inv = crecip(AE(j, j));
      AE(j, j) = inv;
      double2 pr[N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        if (k > j) pr[k] = AE(j, k);
#pragma unroll
      for (int i = 0; i < N; ++i) {
        if (i > j) {
          const double2 f = cmul(AE(i, j), inv);
          AE(i, j) = f;
#pragma unroll
          for (int k = 0; k < N; ++k)
            if (k > j) AE(i, k) = cfms(f, pr[k], AE(i, k));
        }
      }
    }
    if (singular) atomicOr(status, kDevErrSingular);
    // one right-hand side (a column of chi0) at a time, in registers
    double2 *y = chi + pt * N * N;
#pragma unroll 1
    for (int c = 0; c < N; ++c) {
      // An opaque zero added to the factor offsets keeps the compiler from
      // hoisting all N^2 factor loads out of this loop into registers.
      int z = 0;
      asm volatile("" : "+r"(z));
      const double2 *F = A + z;
      const int cm = colmap<NB>(c);
      double2 b[N];
#pragma unroll
      for (int r = 0; r < N; ++r) b[r] = x[perm[r * NT] * N + cm];
#pragma unroll
      for (int r = 1; r < N; ++r)
#pragma unroll
        for (int l = 0; l < r; ++l) b[r] = cfms(F[(r * N + l) * NT], b[l], b[r]);
#pragma unroll
      for (int rr = 0; rr < N; ++rr) {
        const int r = N - 1 - rr;
#pragma unroll
        for (int l = r + 1; l < N; ++l) b[r] = cfms(F[(r * N + l) * NT], b[l], b[r]);
        b[r] = cmul(b[r], F[(r * N + r) * NT]);
      }
#pragma unroll
      for (int r = 0; r < N; ++r) y[r * N + cm] = b[r];
    }
  }
#undef AE
}

template <int NB, int NT>
int launch_rpa_nb(long n_points, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream,
                  unsigned *status) {
  constexpr int N = NB * NB;
  const size_t smem = (size_t)N * N * sizeof(double2) * (1 + NT) + (size_t)(N * N + N + 1) * sizeof(int) +
                      (size_t)N * NT * sizeof(int);
  if (smem > (size_t)max_smem_optin()) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH: nb too large");
  TPRF_CUDA(cudaFuncSetAttribute(rpa_lu_kernel<NB, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  long blocks = (n_points + NT - 1) / NT;
  const long cap = (long)num_sms() * 64;
  blocks = std::max(1L, std::min(blocks, cap));
  rpa_lu_kernel<NB, NT><<<(unsigned)blocks, NT, smem, stream>>>(n_points, chi0, U, chi, status);
  TPRF_LAUNCH_CHECK("rpa_lu_kernel");
  return TPRF_OK;
}

}  // namespace

int launch_rpa(long n_points, int nb, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream) {
  unsigned *status = device_status_word();
  if (!status) return TPRF_ERR_CUDA;
  switch (nb) {
    case 1: return launch_rpa_nb<1, 256>(n_points, chi0, U, chi, stream, status);
    case 2: return launch_rpa_nb<2, 256>(n_points, chi0, U, chi, stream, status);
    case 3: return launch_rpa_nb<3, 128>(n_points, chi0, U, chi, stream, status);
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
