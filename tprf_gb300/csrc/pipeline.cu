// The whole bubble chain g_wk -> chi0_wk, as the Python driver
// python/triqs_tprf/lattice_utils.py:191-269 (imtime_bubble_chi0_wk) chains it:
// fourier_wk_to_wr, fourier_wr_to_tr, then the static trapezoid branch
// (nw == 1, chi0_w0r_from_grt_PH) or the bubble + tau -> w transform, then
// chi_wk_from_chi_wr. The reference's save_memory switch only changes how
// much it stores; here the bubble is always fused with tau -> w, so chi0(tau, r)
// is never stored and both settings give the same numbers.
//
// The caller provides all memory: G(iv, r) and G(tau, r) in `workspace`
// (tprf_imtime_bubble_workspace_bytes), chi0(w, r) is built in the output
// buffer and transformed r -> q in place.
#include "common.cuh"

namespace tprf {
int launch_lattice_fft(bool forward, long n_w, const int dims[3], long n_target, const double2 *in, double2 *out,
                       cudaStream_t stream);
int launch_nu_to_tau(double beta, int n_iw, int n_tau, long C, const double2 *gw, const double2 *mom, double2 *gt,
                     cudaStream_t stream);
int launch_chi0_wr_from_grt(double beta, int n_tau, int nw, const int dims[3], int nb, const double2 *g,
                            double2 *chi0_wr, cudaStream_t stream);
int launch_chi0_w0r_from_grt(double beta, int n_tau, const int dims[3], int nb, const double2 *g, double2 *chi0_wr,
                             cudaStream_t stream);
}  // namespace tprf

using namespace tprf;

extern "C" size_t tprf_imtime_bubble_workspace_bytes(int n_iw, int n_tau, const int dims[3], int nb) {
  if (n_tau < 0) n_tau = default_n_tau(n_iw);
  const size_t nk = (size_t)dims[0] * dims[1] * dims[2];
  const size_t t = (size_t)nb * nb * nk;
  const size_t g_wr = 2ull * n_iw * t, g_tr = (size_t)n_tau * t;
  // G(iv, r), G(tau, r) and its double-float copy (16 bytes per element each),
  // then 256 bytes for the max |G|, max |Im G| words of the real-pair test
  return (g_wr + 2 * g_tr) * sizeof(double2) + 512;
}

extern "C" int tprf_imtime_bubble_chi0_wk(double beta, int n_iw, int n_tau, int nw, const int dims[3], int nb,
                                          const double *g_wk, const double *moments, double *chi0_wk,
                                          void *workspace, size_t workspace_bytes, void *stream) {
  return tprf_imtime_bubble_chi0_wk_timed(beta, n_iw, n_tau, nw, dims, nb, g_wk, moments, chi0_wk, workspace,
                                          workspace_bytes, nullptr, stream);
}

namespace tprf {

// The chain up to chi0(w, r) in `out` (k -> r, iv -> tau, the fused bubble);
// events[0..3] (nullable) are recorded before and after each stage. *chi_df:
// chi0(w, r) was written as double-float pairs; *gmax_out: the real-input words
// of the bubble, which the r -> q mirror and the pair solves use.
// cc (nullable): the caller transforms r -> q next with launch_lattice_fft_fmt
// and can take the compact canonical orbital columns (CompactChi); where they
// apply, *cc is filled (cc->gmax set) and the bubble writes them when its words
// say canon_says_yes. They live in rows 9 .. n_tau - 10 of the complex128
// G(tau, r), which the bubble does not read on that path (it reads the
// double-float copy and the 18 sampled rows at both ends).
int bubble_to_wr(double beta, int n_iw, int n_tau, int nw, const int dims[3], int nb, const double *g_wk,
                 const double *moments, double2 *out, void *workspace, size_t workspace_bytes, void *const *events,
                 cudaStream_t s, bool *chi_df, unsigned **gmax_out, CompactChi *cc) {
  if (!dims || !g_wk || !out || !workspace || nb < 1 || nb > 8 || nw < 1 || n_iw < 1)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "imtime_bubble_chi0_wk: bad shape or null pointer");
  if (n_tau < 0) n_tau = default_n_tau(n_iw);
  const size_t need = tprf_imtime_bubble_workspace_bytes(n_iw, n_tau, dims, nb);
  if (workspace_bytes < need)
    return set_error(TPRF_ERR_ALLOC, "imtime_bubble_chi0_wk: workspace smaller than tprf_imtime_bubble_workspace_bytes");
  const long nk = (long)dims[0] * dims[1] * dims[2];
  const long nb2 = (long)nb * nb;
  uintptr_t ws = (reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255);
  double2 *g_wr = reinterpret_cast<double2 *>(ws);
  double2 *g_tr = g_wr + 2L * n_iw * nk * nb2;
  double2 *g_tr_df = g_tr + (long)n_tau * nk * nb2;  // double-float copy, same element size
  unsigned *gmax = reinterpret_cast<unsigned *>(g_tr_df + (long)n_tau * nk * nb2);
  *gmax_out = gmax;
  auto mark = [&](int i) -> int {
    if (events && events[i]) TPRF_CUDA(cudaEventRecord(static_cast<cudaEvent_t>(events[i]), s));
    return TPRF_OK;
  };
  int st;
  if ((st = mark(0))) return st;
  st = launch_lattice_fft(true, 2L * n_iw, dims, nb2, reinterpret_cast<const double2 *>(g_wk), g_wr, s);
  if (st || (st = mark(1))) return st;
  // gmax[0..1]: the real-input test of G(tau, r); gmax[2..3]: the Hermitian
  // test of G(iv, r), which lets iv -> tau pair real columns;
  // gmax[4]: the transposition test of G(iv, r), which lets iv -> tau and the
  // bubble transform one column of each transposition pair
  TPRF_CUDA(cudaMemsetAsync(gmax, 0, 8 * sizeof(unsigned), s));
  if ((st = launch_hermitian_check(n_iw, nk * nb2, g_wr, gmax + 2, s, dims, nb))) return st;
  const TransposePairs *tp2 = nullptr;
  if ((st = get_transpose_pairs(dims, nb, 2, &tp2))) return st;
  st = launch_nu_to_tau_df(beta, n_iw, n_tau, nk * nb2, g_wr, reinterpret_cast<const double2 *>(moments), g_tr,
                           g_tr_df, s, gmax, gmax + 2, nw > 1, tp2);
  if (st || (st = mark(2))) return st;
  // chi0(w, r) goes from the bubble to the r -> q transform as double-float
  // pairs (same bytes) on the double-float path: no conversion in between
  *chi_df = false;
  if (cc) {
    *cc = CompactChi{};
    const OrbCanon *oc = nullptr;
    const long nb4 = nb2 * nb2;
    if (nw >= 2 && nk > 1 && arith_mode() != kArithFP64 && compact_r_to_q_applies(dims, nb4) && n_tau >= 19) {
      if ((st = get_orb_canon(nb, &oc))) return st;
      if ((long)nw * oc->nc <= (long)(n_tau - 18) * nb2)
        *cc = CompactChi{gmax, g_tr + 9L * nk * nb2, (long)nw, oc};
    }
  }
  if (nw == 1)
    st = launch_chi0_w0r_from_grt(beta, n_tau, dims, nb, g_tr, out, s);
  else
    st = launch_chi0_wr_from_grt_df(beta, n_tau, nw, dims, nb, g_tr, g_tr_df, out, s, nk > 1, chi_df, gmax, nk > 1,
                                    cc && cc->gmax ? cc : nullptr);
  if (st || (st = mark(3))) return st;
  return TPRF_OK;
}

}  // namespace tprf

extern "C" int tprf_imtime_bubble_chi0_wk_timed(double beta, int n_iw, int n_tau, int nw, const int dims[3], int nb,
                                                const double *g_wk, const double *moments, double *chi0_wk,
                                                void *workspace, size_t workspace_bytes, void *const *events,
                                                void *stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double2 *out = reinterpret_cast<double2 *>(chi0_wk);
  bool chi_df = false;
  unsigned *gmax = nullptr;
  CompactChi cc;
  int st = bubble_to_wr(beta, n_iw, n_tau, nw, dims, nb, g_wk, moments, out, workspace, workspace_bytes, events, s,
                        &chi_df, &gmax, &cc);
  if (st) return st;
  const long nb4 = (long)nb * nb * nb * nb;
  // on a real bubble (the same words) only the non-negative frequencies are
  // transformed; the others follow by symmetry; on a transpose-symmetric one
  // only the canonical orbital columns (cc)
  st = launch_lattice_fft_fmt(false, 2L * nw - 1, dims, nb4, out, chi_df, out, false, 1.0, s, chi_df ? gmax : nullptr,
                              false, 0, chi_df && cc.gmax ? &cc : nullptr);
  if (st) return st;
  if (events && events[4]) TPRF_CUDA(cudaEventRecord(static_cast<cudaEvent_t>(events[4]), s));
  return finish_with_checks(s, "imtime_bubble_chi0_wk");
}
