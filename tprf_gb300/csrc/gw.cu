// GW consumers of the bubble chain.
//
//  * gw_dynamic_sigma: sigma_ab(tau, r) = - sum_cd W_acdb(tau, r) G_cd(tau, r)
//    (c++/triqs_tprf/lattice/gw.cpp:66-84), a streaming product per (tau, r).
//  * dynamical_screened_interaction_W: the per-(w, k) solve of
//    lattice/dynamical_screened_interaction.cpp (kernel in rpa_warp.cu).
//  * split_into_dynamic_wk_and_constant_k (lattice/lattice_utility.cpp:57-85):
//    chi_const(k) = the constant moment of the tail fit of chi(iw, k) on the
//    bosonic mesh, chi_dyn = chi - chi_const.
// bubble_PI_wk (python/triqs_tprf/gw.py:56-91) is the bubble chain itself with
// nw = n_max and needs no kernel of its own.
#include <algorithm>

#include "common.cuh"

namespace tprf {
int launch_screened_w(long n_points, long nk, int nb, bool swap, bool v_per_point, const double2 *PI, const double2 *V,
                      double2 *W, cudaStream_t stream, unsigned *status);

namespace {

// one thread per output element (point, a, b); consecutive threads run over b,
// so the W reads W[point][a][c][d][b] are coalesced
__global__ void __launch_bounds__(256) gw_sigma_kernel(long n_out, int nb, const double2 *__restrict__ W,
                                                       const double2 *__restrict__ g, double2 *__restrict__ sigma) {
  const int nb2 = nb * nb;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n_out; i += (long)gridDim.x * blockDim.x) {
    const long pt = i / nb2;
    const int ab = (int)(i - pt * nb2), a = ab / nb, b = ab % nb;
    const double2 *w = W + pt * nb2 * nb2 + (long)a * nb2 * nb + b;
    const double2 *gp = g + pt * nb2;
    double2 s = make_double2(0.0, 0.0);
    for (int cd = 0; cd < nb2; ++cd) s = cfma(w[(long)cd * nb], gp[cd], s);
    sigma[i] = make_double2(-s.x, -s.y);
  }
}

// one thread per column (k, target): c0 = sum_i F[0][i] chi[rows[i]][col]
__global__ void __launch_bounds__(256) split_const_kernel(long ncols, int n_freq, TailFitPlan fit,
                                                          const double2 *__restrict__ chi, double2 *__restrict__ dyn,
                                                          double2 *__restrict__ cst) {
  for (long col = blockIdx.x * (long)blockDim.x + threadIdx.x; col < ncols; col += (long)gridDim.x * blockDim.x) {
    double2 c0 = make_double2(0.0, 0.0);
    for (int i = 0; i < fit.n_fit; ++i) c0 = cfma(fit.F[i], chi[(long)fit.rows[i] * ncols + col], c0);
    cst[col] = c0;
    for (int m = 0; m < n_freq; ++m) dyn[(long)m * ncols + col] = csub(chi[(long)m * ncols + col], c0);
  }
}

long grid_of(long work) {
  const long blocks = (work + 255) / 256;
  return std::max(1L, std::min(blocks, (long)num_sms() * 32));
}

}  // namespace
}  // namespace tprf

using namespace tprf;

extern "C" int tprf_gw_dynamic_sigma(long n_tau, long n_r, int nb, const double *W_tr, const double *g_tr,
                                     double *sigma_tr, void *stream) {
  if (!W_tr || !g_tr || !sigma_tr || n_tau < 1 || n_r < 1 || nb < 1 || nb > 16)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "gw_dynamic_sigma: bad shape or null pointer");
  const long n_out = n_tau * n_r * nb * nb;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  gw_sigma_kernel<<<(unsigned)grid_of(n_out), 256, 0, s>>>(n_out, nb, reinterpret_cast<const double2 *>(W_tr),
                                                          reinterpret_cast<const double2 *>(g_tr),
                                                          reinterpret_cast<double2 *>(sigma_tr));
  TPRF_KERNEL_LAUNCHED("gw_sigma_kernel");
  return TPRF_OK;
}

extern "C" int tprf_dynamical_screened_interaction_W(long n_w, long n_k, int nb, const double *PI_wk,
                                                     const double *V, int v_kind, double *W_wk, void *stream) {
  if (!PI_wk || !V || !W_wk || n_w < 1 || n_k < 1 || nb < 1 || nb > 8 || (v_kind != 0 && v_kind != 1))
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "dynamical_screened_interaction_W: bad shape or null pointer");
  unsigned *status = device_status_word();
  if (!status) return TPRF_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // v_kind 0: static V(k) (pair-swapped contraction), 1: dynamic V(w, k)
  int st = launch_screened_w(n_w * n_k, n_k, nb, v_kind == 0, v_kind == 1, reinterpret_cast<const double2 *>(PI_wk),
                             reinterpret_cast<const double2 *>(V), reinterpret_cast<double2 *>(W_wk), s, status);
  if (st) return st;
  return finish_with_checks(s, "dynamical_screened_interaction_W");
}

extern "C" int tprf_split_into_dynamic_wk_and_constant_k(double beta, int nw, long n_k, long n_target,
                                                         const double *chi_wk, double *chi_dyn_wk,
                                                         double *chi_const_k, void *stream) {
  if (!chi_wk || !chi_dyn_wk || !chi_const_k || !(beta > 0.0) || nw < 2 || n_k < 1 || n_target < 1)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "split_into_dynamic_wk_and_constant_k: bad shape or null pointer");
  const TailFitPlan *p = nullptr;
  int st = get_tail_fit_plan(beta, nw, false, &p);
  if (st) return st;
  const long ncols = n_k * n_target;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  split_const_kernel<<<(unsigned)grid_of(ncols), 256, 0, s>>>(ncols, 2 * nw - 1, *p,
                                                               reinterpret_cast<const double2 *>(chi_wk),
                                                               reinterpret_cast<double2 *>(chi_dyn_wk),
                                                               reinterpret_cast<double2 *>(chi_const_k));
  TPRF_KERNEL_LAUNCHED("split_const_kernel");
  return TPRF_OK;
}
