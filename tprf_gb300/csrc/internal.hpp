// Internal declarations shared by the tprf_gb300 CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <functional>
#include <initializer_list>
#include <string>
#include <vector>

#include "../../include/tprf_gb300.h"

namespace tprf {

// ---------------------------------------------------------------------------
// Errors: every entry point returns a status; a one-line reason is kept per
// thread for tprf_last_error().
int set_error(int status, const std::string &msg);
int cuda_status(cudaError_t e, const char *what);
#define TPRF_CUDA(call)                                              \
  do {                                                               \
    cudaError_t e_ = (call);                                         \
    if (e_ != cudaSuccess) return ::tprf::cuda_status(e_, #call);    \
  } while (0)
#define TPRF_LAUNCH_CHECK(what)                                      \
  do {                                                               \
    cudaError_t e_ = cudaGetLastError();                             \
    if (e_ != cudaSuccess) return ::tprf::cuda_status(e_, what);     \
  } while (0)

// Kernel launches of this library (tprf_kernel_launches): count_launch() at
// every launch site; while this thread captures one of the library's own
// graphs the launches go to its capture tally instead, and every launch of
// such a graph adds the kernels it holds (count_graph_launch).
void count_launch();
void count_graph_launch(unsigned long long kernels);
void begin_capture_tally();
unsigned long long end_capture_tally();
#define TPRF_KERNEL_LAUNCHED(what) \
  do {                             \
    ::tprf::count_launch();        \
    TPRF_LAUNCH_CHECK(what);       \
  } while (0)

bool sync_checks_enabled();
// Bound (ns of the GPU's global timer) of the device-side waits on copies in
// flight (the TMA-staged passes); tprf_set_device_wait_limit_ns.
unsigned long long device_wait_limit_ns();

// Device-side error word (one per device). Kernels OR flag bits into it.
enum : unsigned {
  kDevErrTailFit = 1u,      // tail-fit residual above 1e-3
  kDevErrSingular = 2u,     // zero pivot in Dyson / RPA
  kDevErrNonFinite = 4u,    // NaN / Inf in a result
  kDevErrTimeout = 8u,      // bounded wait expired (persistent kernels)
  kDevErrRange = 16u,       // data outside the double-float chain's exponent range
};
// The double-float chain keeps FP32's exponent range (~1e+-38): the bubble's
// products of G and their transforms stay inside it, with their low words, while
// max |G(iv, r)| lies in [kDfGMin, kDfGMax] (or G is zero).
constexpr float kDfGMin = 1e-15f, kDfGMax = 1e15f;
unsigned *device_status_word();  // nullptr on failure (error set)
// The current device's context as a cache key: its unique id (cuCtxGetId). The
// plans, the status word and the copy stream belong to a context, which
// cudaDeviceReset destroys; the device's next context has another id, so
// nothing cached for the old one is handed out. The device number (with the top
// bit set) where the driver has no cuCtxGetId.
int current_context_key(unsigned long long *key);
// Reads and clears the device word after synchronising `stream`.
int finish_with_checks(cudaStream_t stream, const char *what);

// ---------------------------------------------------------------------------
// FFT plans. A length-n transform is a list of radix stages (Stockham,
// self-sorting) and a table tw[t] = exp(-2 pi i t / n), t < n.
constexpr int kMaxStages = 24;
struct FftDesc {
  int n;
  int nst;
  int has_generic;  // a stage with a prime radix > 7 (needs a second buffer)
  int radix[kMaxStages];
  const double2 *tw;  // device, exp(-2 pi i t / n) in FP64
  const float4 *twf;  // device, the same roots as double-float pairs (re.hi, re.lo, im.hi, im.lo)
  const int *rev;     // device, position of natural index t in the digit-reversed input order
};
// Returns 0 or a status; fills *out. Cached per (device, n).
int get_fft(int n, FftDesc *out);
// The same factors of n in radix order `variant` (0 = get_fft's; see
// factorize_variant in plans.cu); fft_variants(n): the variants giving distinct
// stage sequences for n (the autotuner's candidates).
constexpr int kFftVariants = 4;
int get_fft_variant(int n, int variant, FftDesc *out);
std::vector<int> fft_variants(int n);

// Matsubara -> tau tables for one (beta, n, n_tau, statistic). Fermion: n = n_max,
// inputs iv_n for n = -n_max .. n_max-1; boson: n = nw, inputs iw_m for
// m = -(nw-1) .. nw-1.
struct NuTauPlan {
  double beta;
  int n_iw, n_tau, L;
  int fermion, n_in, in0;  // statistic, input count, frequency integer of input 0
  FftDesc fft;
  const double2 *den;    // [3][n_in]: 1/(iw - b_j), b = (0, 1, -1) fermion, (-1/2, -1, 1) boson
  const double2 *phase;  // [L]: exp(-i pi tau_t / beta) (fermion), 1 (boson)
  const double *ftail;   // [3][L]: oneFermion / oneBoson(1, b_j, tau_t)
  int n_fit, n_mom;      // fit points, number of fitted moments (P+1)
  const int *fit_row;    // [n_fit]: data index of each fit point
  const double2 *fitF;   // [n_mom][n_fit]: moments = F g
  const double2 *fitG;   // [n_fit][n_mom]: model value = sum_p c_p G[i][p]
  // Tail model folded after the FFT (linear in the moments):
  //   G(tau_t) = P[t] FFT(g)[t] + sum_j a_j Q[j][t],  P = phase / beta,
  //   Q[j][t] = ftail[j][t] - P[t] FFT(den[j])[t].
  const double2 *P, *Q;     // [L], [3][L]
  const float4 *Pf, *Qf;    // the same as double-float pairs
  const float4 *fitFf, *fitGf;
};
int get_nu_tau_plan(double beta, int n_iw, int n_tau, const NuTauPlan **out);
int get_nu_tau_plan_stat(double beta, int n, int n_tau, bool fermion, const NuTauPlan **out);

// tau -> Matsubara tables for one (beta, n_tau, n, statistic). Boson: n = nw,
// outputs m = -(nw-1) .. nw-1; fermion: n = n_max, outputs n = -n_max .. n_max-1.
struct TauWPlan {
  double beta;
  int n_tau, nw, L;
  int fermion, n_out, out0;  // statistic, output count, frequency integer of output 0
  FftDesc fft;
  const double *btail;   // [3][L]: oneBoson / oneFermion(1, b_j, tau_t)
  const double2 *den;    // [3][n_out]: 1/(i w_m - b_j)
  const double2 *ph;     // [L]: input phase exp(i pi tau_t / beta) (fermion), 1 (boson)
  // Tail model folded after the FFT: chi(i w_m) = (beta/L) FFT(ph chi)[k_m] + sum_j a_j K[j][m],
  //   K[j][m] = den[j][m] - (beta/L) FFT(ph btail[j])[k_m],  k_m = (m + L) % L.
  const double2 *K;      // [3][n_out]
  const float4 *Kf;
};

// Arithmetic mode. kArithDF64 (default): double-float on the FP32 pipe in the
// FFT stages, the bubble, the Dyson inversion and the nb >= 3 (warp-group) RPA
// solve, FP64 in the tail fits and the nb <= 2 thread-per-point RPA; kArithFP64:
// native FP64 everywhere; kArithDF64All: kArithDF64 with the nb <= 2 RPA in
// double-float as well.
enum Arith : int { kArithDF64 = 0, kArithFP64 = 1, kArithDF64All = 2 };
int arith_mode();
int get_tau_w_plan(double beta, int n_tau, int nw, const TauWPlan **out);
int get_tau_w_plan_stat(double beta, int n_tau, int n, bool fermion, const TauWPlan **out);

// The tail-fit definition of one mesh on the device: moments c = F g[rows].
struct TailFitPlan {
  int n_fit, n_mom;
  const int *rows;      // [n_fit]
  const double2 *F;     // [n_mom][n_fit]
};
int get_tail_fit_plan(double beta, int n, bool fermion, const TailFitPlan **out);

// Exact inverse of the 8x8 Vandermonde V[m][j] = m^j (m = 1..8), uploaded to
// __constant__ memory of the TU that needs it.
void vandermonde_inverse8(double out[64]);
// rows 0 and 1 of the inverse Vandermonde table as TPRF hard-codes it (fit_derivatives)
void fit_derivative_rows(double r0[8], double r1[8]);

// Transposition pairs of the columns (r, e) of a function on a periodic mesh
// with nb^rank target elements e: column c = r * nb^rank + e and its partner
// t(c) = (-r) * nb^rank + e', e' the element with its indices reversed (ab ->
// ba for rank 2, abcd -> dcba for rank 4). With real hoppings G(tau, -r)_ab =
// G(tau, r)_ba and chi0(tau, -r)_dcba = chi0(tau, r)_abcd, so a transform of the
// canonical columns (c <= t(c)) stored at c and t(c) gives every column.
// pairs[i] = {c, t(c)} for the n_can canonical columns in increasing order.
struct TransposePairs {
  long n_can;
  const int2 *pairs;  // device
};
int get_transpose_pairs(const int dims[3], int nb, int rank, const TransposePairs **out);

// Default time mesh of the reference's make_adjoint_mesh for a fermionic
// mesh with n_iw positive frequencies.
inline int default_n_tau(int n_iw) { return 6 * n_iw + 1; }

int max_smem_optin();
int num_sms();

// Real-input test of the bubble chain: G(tau, r) counts as real when
// max |Im G| <= kRealInputTol max |G| (both recorded by the iv -> tau pass as
// float bits in two words); see the real-pair bubble in matsubara.cu.
constexpr float kRealInputTol = 1e-11f;
// Smallest max |G| for which the FP32 ratio test means something (kRealInputTol
// times it is a normal float); the words of a G that is zero, tiny, infinite or
// NaN never say real, so such inputs take the general complex path.
constexpr float kRealInputMin = 1e-26f;
__host__ __device__ __forceinline__ bool real_input_ratio(float max_abs, float max_im) {
  return max_abs >= kRealInputMin && max_abs <= 3.4028234e38f && max_im <= kRealInputTol * max_abs;
}
#ifdef __CUDACC__
__device__ __forceinline__ bool gmax_says_real(const unsigned *gmax) {
  return gmax != nullptr && real_input_ratio(__uint_as_float(gmax[0]), __uint_as_float(gmax[1]));
}
// The same test on G(iv, r): words [max |G|, max |G(iv) - conj(G(-iv))|]
// (hermitian_check_kernel); Hermitian in iv means G(tau, r) is real.
__device__ __forceinline__ bool hermitian_says_yes(const unsigned *hw) { return gmax_says_real(hw); }
// And its third word, max |G_ab(iv, -r) - G_ba(iv, r)|: G(iv, -r) = G(iv, r)^T
// (real hoppings), so that G(tau, -r) = G(tau, r)^T and the bubble columns
// (r, abcd) and (-r, dcba) are equal (the transposition pairs below).
__device__ __forceinline__ bool transpose_says_yes(const unsigned *hw) {
  return hw != nullptr && real_input_ratio(__uint_as_float(hw[0]), __uint_as_float(hw[2]));
}
#endif

// Stream-ordered launchers shared by the C-ABI entry points and the batched
// graphs (no synchronisation; plans must exist before a graph capture).
int launch_lattice_fft(bool forward, long n_w, const int dims[3], long n_target, const double2 *in, double2 *out,
                       cudaStream_t stream);
int launch_lattice_fft_scaled(bool forward, long n_w, const int dims[3], long n_target, const double2 *in,
                              double2 *out, double scale, cudaStream_t stream);
// Canonical orbital columns of a rank-4 bubble: the column o = abcd (a slowest,
// o = ((a nb + b) nb + c) nb + d) is canonical when o <= rev(o) = dcba. When
// the bubble's transposition pairs hold (chi0(w, -r)_dcba = chi0(w, r)_abcd bit
// for bit), its r -> q transform gives chi0(w, -q)_dcba = chi0(w, q)_abcd, so
// only the (nb^4 + nb^2) / 2 canonical columns need a transform.
struct OrbCanon {
  int nc;            // canonical columns
  const int *ocan;   // device [nc]: the canonical columns in increasing order
  const int *orev;   // device [nc]: rev(ocan[j])
  const int *ocomp;  // device [nb^4]: j with ocan[j] == o, or -1
};
int get_orb_canon(int nb, const OrbCanon **out);
// The points k = (k1, k2) of a d1 x d2 mesh (k = k1 d2 + k2) ordered so that each
// k is followed by -k (unless k = -k): the last r -> q pass on compact columns
// writes the columns of k and of -k from one tile or two neighbouring ones.
int get_k_pair_order(int d1, int d2, const int **out);

// The compact form of chi0(w, r) on a real, transpose-symmetric bubble: the
// rows w = 0 .. nw - 1 of the canonical columns, [nw][N_r][nc] as double-float
// pairs in caller memory. The bubble writes it (instead of its output) and the
// r -> q passes read it when the chain's words say so on the device
// (canon_says_yes); otherwise it is left untouched and the full path runs.
struct CompactChi {
  const unsigned *gmax = nullptr;  // the chain's words; null: not used
  void *buf = nullptr;             // compact row w0
  long rows = 0;                   // nw (the whole chain), or the rows of a frequency block
  const OrbCanon *oc = nullptr;
  long w0 = 0;                     // the frequency of buf's first row
};
#ifdef __CUDACC__
__device__ __forceinline__ bool canon_says_yes(const unsigned *gmax) {
  return gmax_says_real(gmax) && hermitian_says_yes(gmax + 2) && transpose_says_yes(gmax + 2);
}
#endif
// Whether the r -> q transform of launch_lattice_fft_fmt can take a CompactChi
// on this mesh: three non-trivial axes, the last two in one plane pass.
bool compact_r_to_q_applies(const int dims[3], long n_target);

// Input / output stored as complex128 or (in_df / out_df, double-float
// arithmetic only, N_k > 1) as double-float pairs of the same 16 bytes.
// gmax (nullable): the rows are the 2 nw - 1 bosonic frequencies of a real
// bubble (launch_chi0_wr_from_grt_df with the same words); when the words say
// real, the negative frequencies are skipped and filled by symmetry,
// x(-w, q) = conj(x(w, -q)), by the last pass, which stores each value of a
// non-negative frequency a second time, conjugated, at its partner (the sign
// bits of the imaginary words flipped: exact). With in != out the skipped
// input rows are not read. fill_partners (without gmax): the same partner
// stores unconditionally, row j of the call (counted from `out`) going to
// row partner_c - j; rows with partner_c - j > j are then not stored, and the
// row with partner_c - j == j has no partner (a frequency block m0 .. m1 - 1
// of the non-negative rows, out at row nw - 1 + m0: partner_c = -2 m0).
// cc (with gmax, on a mesh where compact_r_to_q_applies): when the words say
// canon_says_yes, the passes read cc->buf instead of `in` (the first in place,
// the last writing every column and both signs of w to `out`); otherwise as
// above.
int launch_lattice_fft_fmt(bool forward, long n_w, const int dims[3], long n_target, const void *in, bool in_df,
                           void *out, bool out_df, double scale, cudaStream_t stream, const unsigned *gmax = nullptr,
                           bool fill_partners = false, long partner_c = 0, const CompactChi *cc = nullptr);
// The fused bubble + tau -> iw, writing chi0(iw, r) as double-float pairs when
// want_df and the double-float path runs (*wrote_df tells which). skip_neg:
// on a real bubble (gmax words), the negative frequencies are left unwritten
// for a following launch_lattice_fft_fmt with the same words, which fills them.
// With gmax and the transposition words (gmax[2], gmax[4]) saying yes, only the
// canonical columns of the rank-4 transposition pairs are transformed, each
// result stored at its column and its partner; with cc as well (skip_neg and
// want_df required), each result goes to the canonical orbital column of the
// pair in cc->buf instead, and chi0_wr is not written.
int launch_chi0_wr_from_grt_df(double beta, int n_tau, int nw, const int dims[3], int nb, const double2 *g,
                               const void *g_df, double2 *chi0_wr, cudaStream_t stream, bool want_df, bool *wrote_df,
                               const unsigned *gmax = nullptr, bool skip_neg = false,
                               const CompactChi *cc = nullptr);
// iv -> tau writing the double-float copy as well; gmax (nullable, zeroed by
// the caller) receives max |G| and max |Im G| for launch_chi0_wr_from_grt_df,
// which pairs real bubble columns when G is real.
// When hwords say G(iv, r) is Hermitian (G(tau, r) real), gt_df holds the real
// parts only, one dfl (8 bytes) per element, and with fit_rows_only the
// complex128 gt holds only the rows t <= 8 and t >= n_tau - 9 that the
// bubble's fit samples (the fused bubble reads nothing else of it).
// tp (nullable): the rank-2 transposition pairs of the columns; with hwords'
// transposition word saying yes, only the canonical columns are transformed and
// each stored at its column and its partner (G(tau, r) then meets
// G(tau, -r) = G(tau, r)^T bit for bit).
int launch_nu_to_tau_df(double beta, int n_iw, int n_tau, long C, const double2 *gw, const double2 *mom, double2 *gt,
                        void *gt_df, cudaStream_t stream, unsigned *gmax = nullptr, const unsigned *hwords = nullptr,
                        bool fit_rows_only = false, const TransposePairs *tp = nullptr);
// hwords (three words the caller zeroed) <- max |G(iv, r)|, max |G(iv) - conj(G(-iv))|
// over the 2 n_iw fermionic rows of C columns, and max |G_ab(iv, -r) - G_ba(iv, r)|
// when dims and nb give the column layout (C = N_r nb^2; nb = 0: the third word
// says no); launch_nu_to_tau_df with them pairs columns when G(iv, r) is
// Hermitian in iv, and transposition partners when it is transpose-symmetric.
int launch_hermitian_check(int n_iw, long C, const double2 *gw, unsigned *hwords, cudaStream_t stream,
                           const int *dims = nullptr, int nb = 0);
int launch_tau_to_w_adjoint(double beta, int n_tau, int nw, long C, const double2 *yg, double2 *xg,
                            cudaStream_t stream);
int launch_nu_to_tau_adjoint(double beta, int n_iw, int n_tau, long C, const double2 *yg, double2 *gg, bool fitted,
                             cudaStream_t stream);
// The fused bubble + tau -> w (launch_chi0_wr_from_grt_df) transposed: gg = G_grad(tau, r)
// [n_tau][N_r][nb^2] from yg = chi0_grad(w, r) [2nw-1][N_r][nb^4]; chi0_grad(tau, r) is never stored.
int launch_chi0_wr_from_grt_adjoint(double beta, int n_tau, int nw, const int dims[3], int nb, const double2 *g_tr,
                                    const double2 *yg, double2 *gg, cudaStream_t stream);
int launch_bubble_adjoint(int n_tau, const int dims[3], int nb, const double2 *g_tr, const double2 *chig,
                          double2 *gg, cudaStream_t stream);
int launch_dyson_adjoint(int n_iw, long n_k, int nb, const double2 *g, const double2 *gg, double2 *e_grad,
                         cudaStream_t stream);
int launch_rpa_adjoint(long n_points, int nb, const double2 *chi0, const double2 *U, const double2 *chi,
                       const double2 *chig, double2 *chi0g, double2 *Ug, cudaStream_t stream, unsigned *status);

// The RPA on a bosonic (w, q) mesh: conjugate point pairs solved once where
// U is real and chi0 is bit for bit conjugate-symmetric (rpa.cu).
int launch_rpa_wk(int nw, const int dims[3], int nb, const double2 *chi0, const double2 *U, double2 *chi,
                  cudaStream_t stream);
// Where the pair solves of the frequencies m = mh0 .. mh1-1 (and -m) put chi:
// frequency m >= 0 at pos + (m - mh0) row, frequency -m (m > 0) at
// neg + (m - mh0) neg_step (element offsets; row = N_k nb^4). The whole mesh in
// place: pos = neg = chi + (nw - 1) row, neg_step = -row, mh0 = 0, mh1 = nw.
struct PairOut {
  double2 *pos, *neg;
  long row, neg_step;
  int mh0, mh1;
};
int launch_rpa_wk_block(int nw, const int dims[3], int nb, const double2 *chi0, const double2 *U, PairOut out,
                        cudaStream_t stream);

// Autotuner (tune.cu): the wisdom value of `key` if one is recorded and is
// among the candidates; else, in measure mode and outside a stream capture,
// times launch(v) for every candidate on `s` and records the fastest; else the
// fallback.
int tune_mode();
std::string tune_key(const char *kernel, std::initializer_list<long> shape);
// The wisdom value of `key` among the candidates, else the fallback; never times anything.
int tune_lookup(const std::string &key, const std::vector<int> &candidates, int fallback, int *choice);
int tune_pick(const std::string &key, const std::vector<int> &candidates, int fallback, cudaStream_t s,
              const std::function<int(int)> &launch, int *choice);

}  // namespace tprf
