// Analytic Lindhard bubble chi00(i w, q) (c++/triqs_tprf/lattice/lindhard_chi00.cpp:34-94):
//
//   chi_abcd(w, q) = 1/N_k sum_k sum_ij U_k(a,i) U_k^*(d,i) U_{k+q}(c,j) U_{k+q}^*(b,j)
//                    (f(e_ki) - f(e_{k+q},j)) / (i w + e_{k+q},j - e_ki),
//
// e_ki, U_k the eigen-decomposition of e(k) - mu, f the Fermi function of
// beta e, and beta / (4 cosh^2(beta e_ki / 2)) where w = 0 and the energies
// coincide (|de| < 1e-10). A validation tool: its cost is N_k^2.
//
// Design: one thread per k diagonalises e(k) - mu by cyclic Jacobi rotations
// (complex Hermitian, FP64; the eigenvector phases and order do not matter,
// only the projectors U(a,i) U^*(d,i) enter). Then one CTA per q accumulates
// all (w, abcd) outputs of that q over k, with the eigen data of k and k + q
// staged in shared memory.
#include <algorithm>
#include <cmath>
#include <cstdint>

#include "common.cuh"

namespace tprf {
namespace {

constexpr int kMaxNb = 8;

__device__ __forceinline__ double fermi_of(double e) {  // lattice_utility.cpp:146-153
  if (e < 0) return 1.0 / (exp(e) + 1.0);
  const double x = exp(-e);
  return x / (1.0 + x);
}

__global__ void __launch_bounds__(128) hermitian_eig_kernel(long nk, int nb, const double2 *__restrict__ ek,
                                                            double mu, double *__restrict__ evals,
                                                            double2 *__restrict__ evecs) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < nk; k += (long)gridDim.x * blockDim.x) {
    double2 A[kMaxNb][kMaxNb], V[kMaxNb][kMaxNb];
    double scale = 0.0;
    for (int i = 0; i < nb; ++i)
      for (int j = 0; j < nb; ++j) {
        A[i][j] = ek[(k * nb + i) * nb + j];
        if (i == j) A[i][j].x -= mu;
        V[i][j] = make_double2(i == j ? 1.0 : 0.0, 0.0);
        scale = fmax(scale, cabs2(A[i][j]));
      }
    const double tiny = 1e-30 * (scale + 1e-300);
    for (int sweep = 0; sweep < 60; ++sweep) {
      double off = 0.0;
      for (int p = 0; p < nb; ++p)
        for (int q = p + 1; q < nb; ++q) off = fmax(off, cabs2(A[p][q]));
      if (off <= tiny) break;
      for (int p = 0; p < nb; ++p)
        for (int q = p + 1; q < nb; ++q) {
          const double b2 = cabs2(A[p][q]);
          if (b2 <= tiny) continue;
          const double b = sqrt(b2);
          const double2 ph = make_double2(A[p][q].x / b, A[p][q].y / b);  // e^{i phi}
          const double app = A[p][p].x, aqq = A[q][q].x;
          const double theta = (aqq - app) / (2.0 * b);
          const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
          const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
          // J = diag(1, e^{-i phi}) [[c, s], [-s, c]]: A <- J^H A J, V <- V J
          const double2 mph = cconj(ph);  // e^{-i phi}
          for (int r = 0; r < nb; ++r) {
            const double2 arp = A[r][p], arq = A[r][q];
            A[r][p] = csub(cscale(arp, c), cscale(cmul(arq, mph), s));
            A[r][q] = cadd(cscale(arp, s), cscale(cmul(arq, mph), c));
            const double2 vrp = V[r][p], vrq = V[r][q];
            V[r][p] = csub(cscale(vrp, c), cscale(cmul(vrq, mph), s));
            V[r][q] = cadd(cscale(vrp, s), cscale(cmul(vrq, mph), c));
          }
          for (int r = 0; r < nb; ++r) {
            const double2 apr = A[p][r], aqr = A[q][r];
            A[p][r] = csub(cscale(apr, c), cscale(cmul(aqr, ph), s));
            A[q][r] = cadd(cscale(apr, s), cscale(cmul(aqr, ph), c));
          }
          A[p][q] = A[q][p] = make_double2(0.0, 0.0);
          A[p][p] = make_double2(A[p][p].x, 0.0);
          A[q][q] = make_double2(A[q][q].x, 0.0);
        }
    }
    for (int i = 0; i < nb; ++i) {
      evals[k * nb + i] = A[i][i].x;
      for (int a = 0; a < nb; ++a) evecs[(k * nb + a) * nb + i] = V[a][i];
    }
  }
}

constexpr int kPer = 8;  // outputs per thread: a block covers 256 * kPer of one q

__global__ void __launch_bounds__(256) lindhard_kernel(long nk, int d0, int d1, int d2, int nb, int nw, double beta,
                                                       const double *__restrict__ evals,
                                                       const double2 *__restrict__ evecs, double2 *__restrict__ chi) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *Uk = reinterpret_cast<double2 *>(smem_raw), *Ukq = Uk + nb * nb;
  double *ek = reinterpret_cast<double *>(Ukq + nb * nb), *ekq = ek + nb, *fk = ekq + nb, *fkq = fk + nb;
  const int nb4 = nb * nb * nb * nb, nwt = 2 * nw - 1;
  const int n_out = nwt * nb4;
  const int n_chunks = (n_out + 256 * kPer - 1) / (256 * kPer);
  const long q = blockIdx.x / n_chunks;
  const int o0 = (int)(blockIdx.x % n_chunks) * 256 * kPer;
  const int q2 = (int)(q % d2), q1 = (int)((q / d2) % d1), q0 = (int)(q / ((long)d2 * d1));
  double2 acc[kPer];
  for (int u = 0; u < kPer; ++u) acc[u] = make_double2(0.0, 0.0);
  for (long k = 0; k < nk; ++k) {
    const int k2 = (int)(k % d2), k1 = (int)((k / d2) % d1), k0 = (int)(k / ((long)d2 * d1));
    const long kq = ((long)((k0 + q0) % d0) * d1 + (k1 + q1) % d1) * d2 + (k2 + q2) % d2;
    __syncthreads();
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
      Uk[e] = evecs[k * nb * nb + e];
      Ukq[e] = evecs[kq * nb * nb + e];
    }
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
      ek[i] = evals[k * nb + i];
      ekq[i] = evals[kq * nb + i];
      fk[i] = fermi_of(beta * ek[i]);
      fkq[i] = fermi_of(beta * ekq[i]);
    }
    __syncthreads();
    for (int u = 0; u < kPer; ++u) {
      const int o = o0 + threadIdx.x + u * blockDim.x;
      if (o >= n_out) break;
      const int mi = o / nb4, abcd = o % nb4;
      const int d = abcd % nb, c = (abcd / nb) % nb, b = (abcd / (nb * nb)) % nb, a = abcd / (nb * nb * nb);
      const double w = 2.0 * (mi - (nw - 1)) * M_PI / beta;
      double2 s = make_double2(0.0, 0.0);
      for (int i = 0; i < nb; ++i) {
        const double2 A = cmul(Uk[a * nb + i], cconj(Uk[d * nb + i]));
        for (int j = 0; j < nb; ++j) {
          const double de = ekq[j] - ek[i];
          double2 fac;
          if (fabs(w) < 1e-10 && fabs(de) < 1e-10) {
            const double ch = cosh(0.5 * beta * ek[i]);
            fac = make_double2(beta / (4.0 * ch * ch), 0.0);
          } else {
            const double dn = fk[i] - fkq[j];
            // dn / (de + i w)
            const double den = de * de + w * w;
            fac = make_double2(dn * de / den, -dn * w / den);
          }
          const double2 B = cmul(Ukq[c * nb + j], cconj(Ukq[b * nb + j]));
          s = cfma(cmul(A, B), fac, s);
        }
      }
      acc[u] = cadd(acc[u], s);
    }
  }
  for (int u = 0; u < kPer; ++u) {
    const int o = o0 + threadIdx.x + u * blockDim.x;
    if (o >= n_out) break;
    const int mi = o / nb4, abcd = o % nb4;
    chi[((long)mi * nk + q) * nb4 + abcd] = cscale(acc[u], 1.0 / (double)nk);
  }
}

}  // namespace
}  // namespace tprf

using namespace tprf;

extern "C" size_t tprf_lindhard_chi00_workspace_bytes(long n_k, int nb) {
  if (n_k < 1 || nb < 1) return 0;
  return (size_t)n_k * nb * (sizeof(double) + nb * sizeof(double2)) + 512;
}

extern "C" int tprf_lindhard_chi00(long n_k, const int dims[3], int nb, const double *e_k, double beta, double mu,
                                   int nw, double *chi_wk, void *workspace, size_t workspace_bytes, void *stream) {
  if (!dims || !e_k || !chi_wk || !workspace || n_k < 1 || nb < 1 || nb > kMaxNb || nw < 1 || !(beta > 0.0))
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "lindhard_chi00: bad shape or null pointer");
  if ((long)dims[0] * dims[1] * dims[2] != n_k || dims[0] < 1 || dims[1] < 1 || dims[2] < 1)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "lindhard_chi00: dims do not match n_k");
  if (workspace_bytes < tprf_lindhard_chi00_workspace_bytes(n_k, nb))
    return set_error(TPRF_ERR_ALLOC, "lindhard_chi00: workspace too small");
  const uintptr_t base = (reinterpret_cast<uintptr_t>(workspace) + 255) & ~(uintptr_t)255;
  double2 *evecs = reinterpret_cast<double2 *>(base);
  double *evals = reinterpret_cast<double *>(evecs + (size_t)n_k * nb * nb);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long eb = std::max(1L, std::min((n_k + 127) / 128, (long)num_sms() * 16));
  hermitian_eig_kernel<<<(unsigned)eb, 128, 0, s>>>(n_k, nb, reinterpret_cast<const double2 *>(e_k), mu, evals, evecs);
  TPRF_KERNEL_LAUNCHED("hermitian_eig_kernel");
  const size_t smem = 2 * nb * nb * sizeof(double2) + 4 * nb * sizeof(double);
  const long n_out = (2L * nw - 1) * nb * nb * nb * nb;
  const long blocks = n_k * ((n_out + 256 * kPer - 1) / (256 * kPer));
  if (blocks > 0x7fffffffL) return set_error(TPRF_ERR_UNSUPPORTED_SIZE, "lindhard_chi00: mesh too large");
  lindhard_kernel<<<(unsigned)blocks, 256, smem, s>>>(n_k, dims[0], dims[1], dims[2], nb, nw, beta, evals, evecs,
                                                   reinterpret_cast<double2 *>(chi_wk));
  TPRF_KERNEL_LAUNCHED("lindhard_kernel");
  return TPRF_OK;
}
