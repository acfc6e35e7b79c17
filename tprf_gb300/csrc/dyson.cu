// Kernel (a): the Dyson equation G(iv_n, k) = [(iv_n + mu) I - e(k) - Sigma]^-1,
// one complex128 nb x nb inversion per (v, k) point.
//
// Restates c++/triqs_tprf/lattice/gf.cpp:42-58 (lattice_dyson_g0_Xk) and
// gf.cpp:91-123 (lattice_dyson_g_Xk): same matrix, (w + mu) I - e_k[k] - sigma,
// inverted per point (the reference calls nda::inverse, an LU-based inverse).
//
// Design: one thread per point; the matrix lives in registers and is inverted
// in place by Gauss-Jordan elimination with partial pivoting. Row swaps use
// compile-time indices with predicated selects and the final column
// permutation is folded into the store addresses, so the matrix stays in
// registers (nb <= 5; larger nb spill but stay correct). The elimination runs
// in double-float on the FP32 pipe (about 48 significant bits; the matrix is
// (iv + mu) I - e(k) - Sigma, whose inverse is well conditioned for the
// Matsubara frequencies, |Im| >= pi / beta) and in FP64 in the FP64
// arithmetic mode; the input is read and the output written as complex128.
#include <algorithm>

#include "rpa_common.cuh"

namespace tprf {
namespace {

template <int NB, class E>
__device__ __forceinline__ void swap_rows_if(E (&M)[NB][NB], int j, int p) {
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    if (i > j && i == p) {
#pragma unroll
      for (int c = 0; c < NB; ++c) {
        E t = M[i][c];
        M[i][c] = M[j][c];
        M[j][c] = t;
      }
    }
  }
}

// In-place Gauss-Jordan inverse of the row-pivoted matrix. The inverse of the
// original matrix is M with its columns permuted; the permutation is returned
// packed (destination column of column c in bits [4c, 4c+4)) and applied by
// the caller when storing, so no register array is indexed at run time.
// Returns false on an exactly zero pivot.
// Pivot magnitudes: |z|^2 in FP64, or from the high words of a double-float
// element (the choice of pivot only needs the order of magnitudes).
__device__ __forceinline__ double pivot_mag(double2 z) { return cabs2(z); }
__device__ __forceinline__ float pivot_mag(cdf z) { return __fmaf_rn(z.x.hi, z.x.hi, z.y.hi * z.y.hi); }

template <int NB, class E>
__device__ __forceinline__ bool invert_in_place(E (&M)[NB][NB], unsigned &dest) {
  unsigned perm = 0u;  // pivot row of step j in bits [4j, 4j+4)
  bool ok = true;
#pragma unroll
  for (int j = 0; j < NB; ++j) {
    int p = j;
    auto best = pivot_mag(M[j][j]);
#pragma unroll
    for (int i = j + 1; i < NB; ++i) {
      const auto v = pivot_mag(M[i][j]);
      if (v > best) {
        best = v;
        p = i;
      }
    }
    perm |= (unsigned)p << (4 * j);
    swap_rows_if<NB>(M, j, p);
    if (best == 0) ok = false;
    const E inv = el_recip(M[j][j]);
    M[j][j] = el_one((E *)nullptr);
#pragma unroll
    for (int c = 0; c < NB; ++c) M[j][c] = cmul(M[j][c], inv);
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      if (i != j) {
        const E f = M[i][j];
        M[i][j] = el_zero((E *)nullptr);
#pragma unroll
        for (int c = 0; c < NB; ++c) M[i][c] = el_fms(f, M[j][c], M[i][c]);
      }
    }
  }
  // The row swaps become column swaps of the inverse, applied last pivot first.
  dest = 0u;
#pragma unroll
  for (int c = 0; c < NB; ++c) dest |= (unsigned)c << (4 * c);
#pragma unroll
  for (int jj = 0; jj < NB; ++jj) {
    const unsigned j = NB - 1 - jj;
    const unsigned p = (perm >> (4 * j)) & 15u;
#pragma unroll
    for (int c = 0; c < NB; ++c) {
      const unsigned d = (dest >> (4 * c)) & 15u;
      const unsigned nd = (d == j) ? p : ((d == p) ? j : d);
      dest = (dest & ~(15u << (4 * c))) | (nd << (4 * c));
    }
  }
  return ok;
}

template <int NB, class E>
__global__ void __launch_bounds__(128) dyson_kernel(double beta, int n_iw, long n_k, double mu,
                                                    const double2 *__restrict__ e_k,
                                                    const double2 *__restrict__ sigma, int sigma_kind,
                                                    double2 *__restrict__ g, unsigned *status) {
  const long total = 2L * n_iw * n_k;
  for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
    const int n = (int)(idx / n_k);
    const long k = idx - (long)n * n_k;
    const double nu = (2.0 * (n - n_iw) + 1.0) * M_PI / beta;
    E M[NB][NB];
    const double2 *ek = e_k + k * NB * NB;
    // the matrix in FP64 (the diagonal shift and Sigma), then one conversion
#pragma unroll
    for (int i = 0; i < NB; ++i)
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        const double2 e = ek[i * NB + j];
        double2 m = (i == j) ? make_double2(mu - e.x, nu - e.y) : make_double2(-e.x, -e.y);
        if (sigma_kind != 0) {
          const double2 *s = (sigma_kind == 1) ? sigma + (long)n * NB * NB : sigma + idx * NB * NB;
          m = csub(m, s[i * NB + j]);
        }
        M[i][j] = el_from(m, (E *)nullptr);
      }
    unsigned dest;
    if (!invert_in_place<NB>(M, dest)) atomicOr(status, kDevErrSingular);
    double2 *out = g + idx * NB * NB;
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      const int dj = (int)((dest >> (4 * j)) & 15u);
#pragma unroll
      for (int i = 0; i < NB; ++i) out[i * NB + dj] = el_to(M[i][j]);
    }
  }
}

template <int NB>
int launch_dyson_nb(double beta, int n_iw, long n_k, double mu, const double2 *e_k, const double2 *sigma,
                    int sigma_kind, double2 *g, cudaStream_t stream, unsigned *status) {
  const long total = 2L * n_iw * n_k;
  // threads per CTA (at most the kernel's bound of 128): 128 unless the
  // autotuner measured another (the kernel is out of place, so a trial run
  // recomputes the same G)
  const bool fp64 = arith_mode() == kArithFP64;
  auto launch = [&](int threads) -> int {
    long blocks = (total + threads - 1) / threads;
    const long cap = (long)num_sms() * 2048 / threads;
    if (blocks > cap) blocks = cap;
    if (fp64)
      dyson_kernel<NB, double2><<<(unsigned)blocks, threads, 0, stream>>>(beta, n_iw, n_k, mu, e_k, sigma, sigma_kind,
                                                                          g, status);
    else
      dyson_kernel<NB, cdf><<<(unsigned)blocks, threads, 0, stream>>>(beta, n_iw, n_k, mu, e_k, sigma, sigma_kind, g,
                                                                      status);
    TPRF_KERNEL_LAUNCHED("dyson_kernel");
    return TPRF_OK;
  };
  int threads = 128;
  if ((const void *)e_k != (const void *)g && (const void *)sigma != (const void *)g) {
    int st = tune_pick(tune_key("dyson", {NB, sigma_kind}), {32, 64, 128}, 128, stream, launch, &threads);
    if (st) return st;
  }
  return launch(threads);
}

}  // namespace

int launch_dyson(double beta, int n_iw, long n_k, int nb, double mu, const double2 *e_k, const double2 *sigma,
                 int sigma_kind, double2 *g, cudaStream_t stream) {
  unsigned *status = device_status_word();
  if (!status) return TPRF_ERR_CUDA;
  switch (nb) {
    case 1: return launch_dyson_nb<1>(beta, n_iw, n_k, mu, e_k, sigma, sigma_kind, g, stream, status);
    case 2: return launch_dyson_nb<2>(beta, n_iw, n_k, mu, e_k, sigma, sigma_kind, g, stream, status);
    case 3: return launch_dyson_nb<3>(beta, n_iw, n_k, mu, e_k, sigma, sigma_kind, g, stream, status);
    case 4: return launch_dyson_nb<4>(beta, n_iw, n_k, mu, e_k, sigma, sigma_kind, g, stream, status);
    case 5: return launch_dyson_nb<5>(beta, n_iw, n_k, mu, e_k, sigma, sigma_kind, g, stream, status);
    case 6: return launch_dyson_nb<6>(beta, n_iw, n_k, mu, e_k, sigma, sigma_kind, g, stream, status);
    case 7: return launch_dyson_nb<7>(beta, n_iw, n_k, mu, e_k, sigma, sigma_kind, g, stream, status);
    case 8: return launch_dyson_nb<8>(beta, n_iw, n_k, mu, e_k, sigma, sigma_kind, g, stream, status);
    default: return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice_dyson_g_wk: nb must be 1..8");
  }
}

}  // namespace tprf

extern "C" int tprf_lattice_dyson_g_wk(double beta, int n_iw, long n_k, int nb, double mu, const double *e_k,
                                       const double *sigma, int sigma_kind, double *g_wk, void *stream) {
  using namespace tprf;
  if (!(beta > 0.0) || n_iw < 1 || n_k < 1 || !e_k || !g_wk)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice_dyson_g_wk: bad mesh or null pointer");
  if (sigma_kind < 0 || sigma_kind > 2 || (sigma_kind != 0 && !sigma))
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice_dyson_g_wk: bad sigma_kind / sigma");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = launch_dyson(beta, n_iw, n_k, nb, mu, reinterpret_cast<const double2 *>(e_k),
                        reinterpret_cast<const double2 *>(sigma), sigma_kind, reinterpret_cast<double2 *>(g_wk), s);
  if (st) return st;
  return finish_with_checks(s, "lattice_dyson_g_wk");
}

// ---- adjoint (differentiable path) ----------------------------------------------
// G = [(iv + mu) I - e(k)]^-1 gives dG = G de G, so for a real loss with gradient
// Gg = dL/dG (conjugate Wirtinger convention, as torch uses) the gradient of e(k)
// is sum_v G^H Gg G^H. A CTA takes 32 consecutive k (one per lane) and a slice
// of the frequencies (every warp of the grid's slices a different frequency,
// so a warp's loads are 32 consecutive k of one frequency); the partial sums
// meet in e_grad through FP64 atomics (the launcher zeroes it first).

namespace tprf {
namespace {

template <int NB>
__global__ void __launch_bounds__(256) dyson_adjoint_kernel(int n_nu, long n_k, const double2 *__restrict__ g,
                                                            const double2 *__restrict__ gg, double2 *__restrict__ ekg) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, n_warps = blockDim.x >> 5;
  const long k = blockIdx.x * 32L + lane;
  if (k >= n_k) return;
  const int stride = gridDim.y * n_warps;
  double2 acc[NB][NB];
#pragma unroll
  for (int i = 0; i < NB; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j) acc[i][j] = make_double2(0.0, 0.0);
  for (int n = blockIdx.y * n_warps + warp; n < n_nu; n += stride) {
    const double2 *G = g + ((long)n * n_k + k) * NB * NB;
    const double2 *Y = gg + ((long)n * n_k + k) * NB * NB;
    // T = Gg G^H, then acc += G^H T
    double2 T[NB][NB];
#pragma unroll
    for (int i = 0; i < NB; ++i)
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        double2 s = make_double2(0.0, 0.0);
#pragma unroll
        for (int l = 0; l < NB; ++l) s = cfma(Y[i * NB + l], cconj(G[j * NB + l]), s);
        T[i][j] = s;
      }
#pragma unroll
    for (int i = 0; i < NB; ++i)
#pragma unroll
      for (int j = 0; j < NB; ++j)
#pragma unroll
        for (int l = 0; l < NB; ++l) acc[i][j] = cfma(cconj(G[l * NB + i]), T[l][j], acc[i][j]);
  }
  double *out = reinterpret_cast<double *>(ekg + k * NB * NB);
#pragma unroll
  for (int i = 0; i < NB; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      atomicAdd(out + 2 * (i * NB + j), acc[i][j].x);
      atomicAdd(out + 2 * (i * NB + j) + 1, acc[i][j].y);
    }
}

template <int NB>
int launch_dyson_adjoint_nb(int n_nu, long n_k, const double2 *g, const double2 *gg, double2 *ekg, cudaStream_t s) {
  TPRF_CUDA(cudaMemsetAsync(ekg, 0, (size_t)n_k * NB * NB * sizeof(double2), s));
  const long k_tiles = (n_k + 31) / 32;
  constexpr int kWarps = 8;
  const long target = (long)num_sms() * 8;  // CTAs for a full GPU
  const long slices = std::max(1L, std::min((long)((n_nu + kWarps - 1) / kWarps), (target + k_tiles - 1) / k_tiles));
  if (k_tiles > 0x7fffffffL) return set_error(TPRF_ERR_UNSUPPORTED_SIZE, "lattice_dyson_g_wk_adjoint: too many k");
  dyson_adjoint_kernel<NB><<<dim3((unsigned)k_tiles, (unsigned)slices), 32 * kWarps, 0, s>>>(n_nu, n_k, g, gg, ekg);
  TPRF_KERNEL_LAUNCHED("dyson_adjoint_kernel");
  return TPRF_OK;
}

}  // namespace

int launch_dyson_adjoint(int n_iw, long n_k, int nb, const double2 *g, const double2 *gg, double2 *out,
                         cudaStream_t s) {
  switch (nb) {
    case 1: return launch_dyson_adjoint_nb<1>(2 * n_iw, n_k, g, gg, out, s);
    case 2: return launch_dyson_adjoint_nb<2>(2 * n_iw, n_k, g, gg, out, s);
    case 3: return launch_dyson_adjoint_nb<3>(2 * n_iw, n_k, g, gg, out, s);
    case 4: return launch_dyson_adjoint_nb<4>(2 * n_iw, n_k, g, gg, out, s);
    case 5: return launch_dyson_adjoint_nb<5>(2 * n_iw, n_k, g, gg, out, s);
    default: return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice_dyson_g_wk_adjoint: nb must be 1..5");
  }
}

}  // namespace tprf

extern "C" int tprf_lattice_dyson_g_wk_adjoint(int n_iw, long n_k, int nb, const double *g_wk, const double *g_wk_grad,
                                               double *e_k_grad, void *stream) {
  using namespace tprf;
  if (n_iw < 1 || n_k < 1 || !g_wk || !g_wk_grad || !e_k_grad)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice_dyson_g_wk_adjoint: bad shape or null pointer");
  return launch_dyson_adjoint(n_iw, n_k, nb, reinterpret_cast<const double2 *>(g_wk),
                              reinterpret_cast<const double2 *>(g_wk_grad), reinterpret_cast<double2 *>(e_k_grad),
                              static_cast<cudaStream_t>(stream));
}
