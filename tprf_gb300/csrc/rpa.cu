// Kernel (d): the RPA solve chi = [I - chi0 U]^-1 chi0 per (omega, q) point.
//
// Restates c++/triqs_tprf/lattice/rpa.cpp:29-64: chi0 and U are grouped into
// nb^2 x nb^2 matrices with rows (a, b) and columns (d, c)
// (idx_group<0,1>, idx_group<3,2>, rpa.cpp:40,54-55) and
// chi = inverse(I - chi0 * U) * chi0 (rpa.cpp:57). Here the same system is
// solved without forming the inverse: A = I - chi0 U, then Gaussian
// elimination with partial pivoting on [A | chi0] and back substitution.
//
// Design: one thread per point; the grouped U is shared by the CTA in shared
// memory; each thread's A and right-hand sides live in shared memory laid out
// [element][thread], so every access is conflict-free although each thread
// pivots independently. All loops are unrolled for the compile-time size.
#include <algorithm>

#include "common.cuh"

namespace tprf {
namespace {

template <int NB>
__device__ __forceinline__ int colmap(int c) {  // grouped column (d, c') -> offset c' * nb + d
  return (c % NB) * NB + c / NB;
}

template <int NB, int NT>
__global__ void __launch_bounds__(NT) rpa_kernel(long n_points, const double2 *chi0,
                                                 const double2 *__restrict__ U, double2 *chi,
                                                 unsigned *status) {
  constexpr int N = NB * NB;
  constexpr int UNR = (N <= 9) ? 32 : 1;  // full unroll only for the small systems
  extern __shared__ double2 smem[];
  double2 *Ug = smem;  // [N][N], shared by the CTA
  // Per-thread systems, [element][thread], real and imaginary planes. Declared
  // volatile so each access is a real shared-memory access: without it the
  // compiler may keep a thread's private rows in registers and spill them.
  volatile double *ws = reinterpret_cast<volatile double *>(smem + N * N);
  const int tid = threadIdx.x;
  volatile double *Ar = ws + tid;
  volatile double *Ai = Ar + (size_t)N * N * NT;
  volatile double *Br = Ai + (size_t)N * N * NT;
  volatile double *Bi = Br + (size_t)N * N * NT;
  for (int w = tid; w < N * N; w += NT) {
    const int m = w / N, c = w % N;
    Ug[w] = U[m * N + colmap<NB>(c)];
  }
  __syncthreads();
#define AOFF(i, j) (((i) * N + (j)) * NT)
#define LDA(i, j) make_double2(Ar[AOFF(i, j)], Ai[AOFF(i, j)])
#define LDB(i, j) make_double2(Br[AOFF(i, j)], Bi[AOFF(i, j)])
#define STA(i, j, v) (Ar[AOFF(i, j)] = (v).x, Ai[AOFF(i, j)] = (v).y)
#define STB(i, j, v) (Br[AOFF(i, j)] = (v).x, Bi[AOFF(i, j)] = (v).y)
  for (long base = blockIdx.x * (long)NT; base < n_points; base += (long)gridDim.x * NT) {
    const long pt = base + tid;
    if (pt < n_points) {
      const double2 *x = chi0 + pt * N * N;
#pragma unroll UNR
      for (int r = 0; r < N; ++r)
#pragma unroll
        for (int c = 0; c < N; ++c) STB(r, c, x[r * N + colmap<NB>(c)]);
      // A = I - chi0 U
#pragma unroll UNR
      for (int r = 0; r < N; ++r) {
#pragma unroll UNR
        for (int c = 0; c < N; ++c) {
          double2 s = make_double2(r == c ? 1.0 : 0.0, 0.0);
#pragma unroll
          for (int m = 0; m < N; ++m) s = cfms(LDB(r, m), Ug[m * N + c], s);
          STA(r, c, s);
        }
      }
      bool singular = false;
#pragma unroll UNR
      for (int j = 0; j < N; ++j) {
        int p = j;
        double best = cabs2(LDA(j, j));
#pragma unroll UNR
        for (int i = j + 1; i < N; ++i) {
          const double v = cabs2(LDA(i, j));
          if (v > best) {
            best = v;
            p = i;
          }
        }
        if (best == 0.0) singular = true;
        if (p != j) {
#pragma unroll UNR
          for (int k = j; k < N; ++k) {
            const double2 t = LDA(j, k);
            STA(j, k, LDA(p, k));
            STA(p, k, t);
          }
#pragma unroll UNR
          for (int k = 0; k < N; ++k) {
            const double2 t = LDB(j, k);
            STB(j, k, LDB(p, k));
            STB(p, k, t);
          }
        }
        const double2 inv = crecip(LDA(j, j));
        STA(j, j, inv);
#pragma unroll UNR
        for (int i = j + 1; i < N; ++i) {
          const double2 f = cmul(LDA(i, j), inv);
#pragma unroll UNR
          for (int k = j + 1; k < N; ++k) STA(i, k, cfms(f, LDA(j, k), LDA(i, k)));
#pragma unroll UNR
          for (int k = 0; k < N; ++k) STB(i, k, cfms(f, LDB(j, k), LDB(i, k)));
        }
      }
      if (singular) atomicOr(status, kDevErrSingular);
      double2 *y = chi + pt * N * N;
#pragma unroll UNR
      for (int j = N - 1; j >= 0; --j) {
        const double2 inv = LDA(j, j);
#pragma unroll UNR
        for (int k = 0; k < N; ++k) {
          double2 s = LDB(j, k);
#pragma unroll UNR
          for (int l = j + 1; l < N; ++l) s = cfms(LDA(j, l), LDB(l, k), s);
          s = cmul(s, inv);
          STB(j, k, s);
          y[j * N + colmap<NB>(k)] = s;
        }
      }
    }
  }
#undef AOFF
#undef LDA
#undef LDB
#undef STA
#undef STB
}

template <int NB, int NT>
int launch_rpa_nb(long n_points, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream,
                  unsigned *status) {
  constexpr int N = NB * NB;
  const size_t smem = (size_t)N * N * sizeof(double2) * (1 + 2 * NT);
  if (smem > (size_t)max_smem_optin()) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH: nb too large");
  TPRF_CUDA(cudaFuncSetAttribute(rpa_kernel<NB, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  long blocks = (n_points + NT - 1) / NT;
  const long cap = (long)num_sms() * 64;
  blocks = std::max(1L, std::min(blocks, cap));
  rpa_kernel<NB, NT><<<(unsigned)blocks, NT, smem, stream>>>(n_points, chi0, U, chi, status);
  TPRF_LAUNCH_CHECK("rpa_kernel");
  return TPRF_OK;
}

}  // namespace

int launch_rpa(long n_points, int nb, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream) {
  unsigned *status = device_status_word();
  if (!status) return TPRF_ERR_CUDA;
  switch (nb) {
    case 1: return launch_rpa_nb<1, 256>(n_points, chi0, U, chi, stream, status);
    case 2: return launch_rpa_nb<2, 256>(n_points, chi0, U, chi, stream, status);
    case 3: return launch_rpa_nb<3, 64>(n_points, chi0, U, chi, stream, status);
    case 4: return launch_rpa_nb<4, 16>(n_points, chi0, U, chi, stream, status);
    case 5: return launch_rpa_nb<5, 8>(n_points, chi0, U, chi, stream, status);
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
