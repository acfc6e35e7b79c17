/*
 * tprf_gb300 — C ABI of the GB300-native imaginary-time bubble + RPA path.
 *
 * Every entry point replaces one function of TPRF (TRIQS/tprf 3.2); the
 * reference declaration each one stands in for is cited beside it
 * (paths relative to the TPRF source tree).
 *
 * Conventions shared by all entry points
 *  - Complex data is complex128, interleaved (re, im) doubles, passed as
 *    `double*`. Layout is TRIQS gf data order: mesh indices first, then the
 *    target indices, C order. Example: G(iv, k) is [2 n_iw, N_k, nb, nb].
 *  - Fermionic Matsubara meshes are full meshes n = -n_iw .. n_iw-1
 *    (2 n_iw points); bosonic meshes are m = -(nw-1) .. nw-1 (2 nw - 1
 *    points); imaginary time has n_tau points tau_i = i beta / (n_tau - 1).
 *  - k / r meshes are 3-dimensional `dims[3]` (unused dimensions 1), linear
 *    index (i1 * n2 + i2) * n3 + i3.
 *  - All pointers are DEVICE pointers owned by the caller; nothing is freed
 *    or retained. `stream` is a cudaStream_t (NULL = legacy default stream).
 *    Work is stream-ordered; a call returns after the launches are queued,
 *    except where a synchronous check is enabled (tprf_set_sync_checks).
 *  - Return value: TPRF_OK (0) or a negative status; no C++ exception ever
 *    crosses the ABI. tprf_last_error() gives a one-line reason (per thread).
 *  - The first call for a new mesh / FFT length builds a plan (twiddle and
 *    tail tables, uploaded synchronously, cached for the process); make that
 *    first call before capturing a stream into a CUDA graph.
 *  - FFT lengths may be any integer: factors 2, 3, 4, 5, 7, 8 use fixed
 *    butterflies, any other prime factor p a direct p-point stage (slower).
 */
#ifndef TPRF_GB300_H
#define TPRF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define TPRF_OK 0
#define TPRF_ERR_INVALID_ARGUMENT (-1)  /* bad shape, null pointer, nb out of range */
#define TPRF_ERR_UNSUPPORTED_SIZE (-2)  /* FFT tile does not fit one CTA (mesh dimension or time mesh too long) */
#define TPRF_ERR_MESH_TOO_SHORT (-3)    /* time mesh shorter than 2x the frequency mesh (fourier_matsubara.cpp:105-108,128-131) */
#define TPRF_ERR_TAIL_FIT (-4)          /* tail fit error above 1e-3 (fourier_matsubara.cpp:227-230) */
#define TPRF_ERR_NONFINITE (-5)         /* NaN / Inf produced or found */
#define TPRF_ERR_CUDA (-6)              /* a CUDA runtime call failed */
#define TPRF_ERR_ALLOC (-7)             /* device allocation failed or workspace too small */
#define TPRF_ERR_SINGULAR (-8)          /* exactly singular matrix in Dyson or RPA */
#define TPRF_ERR_RANGE (-9)             /* double-float chain: max |G(iv, r)| outside [1e-15, 1e15] (use TPRF_ARITH_FP64) */

const char *tprf_status_string(int status);
const char *tprf_last_error(void);
/* Library version, e.g. "0.1.0". */
const char *tprf_version(void);

/* When on (default), entry points that can detect data-dependent errors
 * (tail-fit error, singular matrices) synchronise `stream` once at the end
 * and report them. Switch off for CUDA-graph capture or pipelining; the
 * device-side error word is then read by tprf_check_device_status. */
void tprf_set_sync_checks(int on);
int tprf_check_device_status(void *stream);

/* Kernels this library has put on the GPU since the process started: one per
 * launch of one of its kernels, and the kernel count of one of its graphs
 * (tprf_batch_*) each time that graph is launched. Process-wide. No reference
 * counterpart. */
unsigned long long tprf_kernel_launches(void);

/* Bound of the device-side waits of the TMA-staged lattice pass on the tile
 * copies it has in flight, in nanoseconds of the GPU's global timer (default
 * 200 ms; 0 makes every such wait give up at once). A wait that runs out sets
 * the device error word (reported as "device wait timed out" by the call's
 * check or tprf_check_device_status); the block then waits up to 1 s for each
 * of its copies in flight to land and leaves, so the context stays usable.
 * Process-wide. No reference counterpart. */
int tprf_set_device_wait_limit_ns(long long ns);

/* Arithmetic of the path. Double-float means pairs of FP32 values (~48-bit
 * significand, FP32 exponent range) on the FP32 pipe, which on GB300 runs ~70x
 * faster than the FP64 pipe.
 * TPRF_ARITH_DF64 (default): double-float in the lattice FFTs, iv -> tau, the
 *   bubble + tau -> i omega, the Dyson inversion and the RPA solve of nb >= 3
 *   (the warp-group kernels; a point whose conditioning estimate, largest term
 *   over smallest pivot, exceeds 100 is re-solved in FP64); native FP64 in the
 *   tail fits, the fit_derivatives samples and the thread-per-point RPA of
 *   nb <= 2.
 * TPRF_ARITH_FP64: native FP64 in every kernel (the plain GPU path).
 * TPRF_ARITH_DF64_ALL: as DF64, with the nb <= 2 RPA in double-float as well.
 * Inputs and outputs are complex128 in every mode. Process-wide; no reference
 * counterpart (the reference has one CPU path). */
#define TPRF_ARITH_DF64 0
#define TPRF_ARITH_FP64 1
#define TPRF_ARITH_DF64_ALL 2
int tprf_set_arithmetic(int mode);
int tprf_get_arithmetic(void);

/* Autotuner of launch shapes. The reference plans its FFTs with FFTW_ESTIMATE
 * (c++/triqs_tprf/fourier/fourier_common.cpp:32-43): a fixed heuristic. Mode 0
 * (default) uses fixed heuristics here too; mode 1 ("measure", as FFTW_MEASURE)
 * times every candidate on the first call of each shape (the shortest of three
 * launches) and keeps the fastest, or the heuristic's choice when no candidate
 * beats it by more than 2 %: columns per CTA and the radix order of the FFT of
 * the iv -> tau and tau -> i omega kernels (fused bubble included), lanes per
 * point of the RPA group kernels (nb >= 3), threads per CTA of the Dyson
 * kernel, and the tile size of the TMA-staged lattice plane pass (0 = the
 * plain pass; in-place calls only read it from wisdom).
 * Candidates run on a prefix of the call's own columns or points, or on the
 * whole call (out-of-place kernels only), so results do not depend on the mode
 * beyond rounding (the TMA plane pass rounds as a decimation-in-frequency FFT). A tuning call waits for its stream;
 * tuning is skipped while the stream is being captured. The choices ("wisdom")
 * are process-wide, keyed by GPU, arithmetic mode, kernel and shape, and can be
 * saved to and loaded from a text file ("key value" per line). */
int tprf_set_autotune(int mode);
int tprf_get_autotune(void);
int tprf_autotune_entries(void);
void tprf_autotune_clear(void);
int tprf_autotune_save(const char *path);
int tprf_autotune_load(const char *path);

/* Device capability: sustained FP64 FMA throughput (TFLOP/s) of the current
 * GPU, best of three timed runs of a fixed-length FMA loop; synchronises
 * `stream`. A native FP64 form of the path would be bound by this pipe on
 * GB300; the benchmark reports FP64 fractions against it. No reference
 * counterpart.
 * scratch: device buffer of at least 2048 doubles per SM. */
int tprf_measure_fp64_tflops(double *tflops, void *scratch, size_t scratch_bytes, void *stream);

/* Host-only (no GPU): the tail-fit definition tprf_fourier_wr_to_tr applies
 * when moments == NULL. A least-squares fit of g(iv) ~ sum_{p<=P} c_p (iv)^-p
 * on the outer 20% of the fermionic mesh (at most 30 points a side, both
 * signs), the stand-in for TRIQS fit_tail called at
 * fourier/fourier_matsubara.cpp:226. Writes n_fit and n_mom = P + 1; when rows
 * and F are non-NULL and capacity >= n_fit * n_mom, also the data rows of the
 * fit points and F [n_mom][n_fit] complex, with moments c = F g[rows]. */
int tprf_tail_fit_matrix(double beta, int n_iw, int capacity, int *n_fit, int *n_mom, int *rows, double *F);
/* The same for either statistic (fermion != 0: n = n_max, data index n + n_max of
 * iv_n; fermion == 0: n = nw, data index m + nw - 1 of iw_m, fitting the positive
 * indices 1 .. nw-1 and their mirrors), as tprf_chi_tr_from_chi_wr applies it. */
int tprf_tail_fit_matrix_stat(double beta, int n, int fermion, int capacity, int *n_fit, int *n_mom,
                              int *rows, double *F);

/* Host-only: exact inverse of the 8x8 Vandermonde matrix V[m][j] = m^j
 * (m = 1..8), the matrix fourier_matsubara.cpp:56-71 approximates. */
void tprf_vandermonde_inverse8(double out[64]);
/* Host-only: rows 0 and 1 of that inverse as TPRF hard-codes them in
 * fit_derivatives (fourier_matsubara.cpp:56-71, up to ~5e-12 relative from
 * the exact rationals): out[0..7] row 0 (first derivative), out[8..15] row 1.
 * These are the constants the tau -> i omega kernels apply. */
void tprf_fit_derivative_rows(double out[16]);

/* ---- (a) Dyson equation -------------------------------------------------
 * G(iv_n, k) = [(iv_n + mu) I - e(k) - Sigma]^-1, per (v, k).
 * Replaces triqs_tprf::lattice_dyson_g0_wk(double mu, e_k_cvt, mesh::imfreq)
 *   (c++/triqs_tprf/lattice/gf.hpp:44, gf.cpp:42-58) when sigma == NULL, and
 * triqs_tprf::lattice_dyson_g_wk(double mu, e_k_cvt, g_w_cvt | g_wk_cvt)
 *   (gf.hpp:83,123, gf.cpp:91-132) otherwise.
 * e_k [n_k, nb, nb]; sigma_kind 0: none, 1: sigma_w [2 n_iw, nb, nb],
 * 2: sigma_wk [2 n_iw, n_k, nb, nb]. g_wk [2 n_iw, n_k, nb, nb]. nb <= 8. */
int tprf_lattice_dyson_g_wk(double beta, int n_iw, long n_k, int nb, double mu,
                            const double *e_k, const double *sigma, int sigma_kind,
                            double *g_wk, void *stream);

/* ---- (b) lattice FFTs ---------------------------------------------------
 * k -> r: FFTW_FORWARD over the k dims, divided by N_k, for each of n_w
 * mesh slices and n_target target elements.
 * Replaces triqs_tprf::fourier_wk_to_wr(g_wk_cvt) (gf.hpp:286, gf.cpp:209;
 * lattice/fourier.hpp:166-197; fourier/fourier_lattice.cpp:39-50).
 * in [n_w, N_k, n_target] -> out [n_w, N_r, n_target]; in == out allowed. */
int tprf_fourier_wk_to_wr(long n_w, const int dims[3], long n_target,
                          const double *g_wk, double *g_wr, void *stream);

/* r -> k: FFTW_BACKWARD, unscaled.
 * Replaces triqs_tprf::fourier_wr_to_wk (gf.cpp:214) and
 * triqs_tprf::chi_wk_from_chi_wr(chi_wr_cvt) (lattice/chi_imtime.hpp:141,
 * chi_imtime.cpp:289-292; lattice/fourier.hpp:200-231). */
int tprf_fourier_wr_to_wk(long n_w, const int dims[3], long n_target,
                          const double *g_wr, double *g_wk, void *stream);

/* Allocation-free lattice FFT: the same transforms as tprf_fourier_wk_to_wr
 * (forward != 0) and tprf_fourier_wr_to_wk (forward == 0), for callers that
 * cannot let a library allocate device memory (codes whose device memory all
 * belongs to their own pool allocator, hosts with a fixed device-memory
 * budget). No counterpart in the reference: it is an addition of this library.
 * Its FFT tables live in a static 1 MiB device array inside the library
 * image, 36 bytes per point of each distinct mesh length: tables beyond it
 * return TPRF_ERR_INVALID_ARGUMENT. A mesh length above 12 799 points (6 399
 * with a prime factor above 8) does not fit one CTA's shared memory and returns
 * TPRF_ERR_UNSUPPORTED_SIZE. Both checks come before any work is queued. The
 * first call on a device may load the library's device code there, so make it
 * before any stream capture. Calls share the array: calls overlapping on the
 * GPU race. */
int tprf_fourier_lattice_noalloc(int forward, long n_w, const int dims[3], long n_target,
                                 const double *in, double *out, void *stream);

/* iv -> tau, fermionic, per r and target element, with the three-pole
 * high-frequency tail model (fourier/fourier_matsubara.cpp:218-308).
 * Replaces triqs_tprf::fourier_wr_to_tr(g_wr_cvt, int nt = -1)
 *   (gf.hpp:306, gf.cpp:262; lattice/fourier.hpp:99-130).
 * n_tau = -1 selects 6 n_iw + 1. moments == NULL: moments m1..m3 come from
 * the least-squares tail fit (the reference's fit_tail call at
 * fourier_matsubara.cpp:226); otherwise moments [3, n_r, n_target] holds
 * m1, m2, m3. g_wr [2 n_iw, n_r, n_target] -> g_tr [n_tau, n_r, n_target]. */
int tprf_fourier_wr_to_tr(double beta, int n_iw, int n_tau, long n_r, long n_target,
                          const double *g_wr, const double *moments, double *g_tr,
                          void *stream);

/* ---- (c) bubble ----------------------------------------------------------
 * chi0_abcd(tau_i, r) = G_da(tau_i, r) G_bc(tau_{n_tau-1-i}, -r).
 * Replaces triqs_tprf::chi0_tr_from_grt_PH(g_tr_cvt)
 *   (lattice/chi_imtime.hpp:38, chi_imtime.cpp:88-136).
 * g_tr [n_tau, N_r, nb, nb] -> chi0_tr [n_tau, N_r, nb, nb, nb, nb]. */
int tprf_chi0_tr_from_grt_PH(int n_tau, const int dims[3], int nb,
                             const double *g_tr, double *chi0_tr, void *stream);

/* Bubble fused with the bosonic tau -> i omega transform per r (chi0(tau, r)
 * never materialised). Replaces triqs_tprf::chi0_wr_from_grt_PH(g_tr_cvt, int nw)
 *   (chi_imtime.hpp:40, chi_imtime.cpp:139-182).
 * -> chi0_wr [2 nw - 1, N_r, nb^4]. */
int tprf_chi0_wr_from_grt_PH(double beta, int n_tau, int nw, const int dims[3], int nb,
                             const double *g_tr, double *chi0_wr, void *stream);

/* Bubble + trapezoid integral over tau (static chi0).
 * Replaces triqs_tprf::chi0_w0r_from_grt_PH(g_tr_cvt) (chi_imtime.hpp:56,
 * chi_imtime.cpp:185-228). -> chi0_wr [1, N_r, nb^4]. */
int tprf_chi0_w0r_from_grt_PH(double beta, int n_tau, const int dims[3], int nb,
                              const double *g_tr, double *chi0_wr, void *stream);

/* Bosonic tau -> i omega with the fit_derivatives tail
 * (fourier_matsubara.cpp:42-97,123-184).
 * Replaces triqs_tprf::chi_wr_from_chi_tr(chi_tr_cvt, int nw)
 *   (chi_imtime.hpp:104, chi_imtime.cpp:279-282; lattice/fourier.hpp:133-163).
 * chi_tr [n_tau, n_r, n_target] -> chi_wr [2 nw - 1, n_r, n_target]. */
int tprf_chi_wr_from_chi_tr(double beta, int n_tau, int nw, long n_r, long n_target,
                            const double *chi_tr, double *chi_wr, void *stream);

/* ---- inverse transforms -------------------------------------------------------
 * Fermionic tau -> i nu with the fit_derivatives tail (fermion branch of
 * fourier_matsubara.cpp:123-184: input multiplied by exp(i pi tau / beta),
 * b = (0, 1, -1)).
 * Replaces triqs_tprf::fourier_tr_to_wr(g_tr_cvt, int nw) (gf.hpp:306,
 *   gf.cpp:257-260; lattice/fourier.hpp:133-163).
 * g_tr [n_tau, n_r, n_target] -> g_wr [2 n_iw, n_r, n_target] (n = -n_iw .. n_iw-1);
 * n_iw < 0: (n_tau - 1) / 6. Requires n_tau - 1 >= 2 n_iw. */
int tprf_fourier_tr_to_wr(double beta, int n_tau, int n_iw, long n_r, long n_target,
                          const double *g_tr, double *g_wr, void *stream);

/* Bosonic i omega -> tau with the tail fit on the bosonic mesh (boson branch of
 * fourier_matsubara.cpp:218-308: b = (-1/2, -1, 1), chi[L] = +(chi[0] + m1)).
 * Replaces triqs_tprf::chi_tr_from_chi_wr(chi_wr_cvt, int ntau)
 *   (chi_imtime.hpp:105, chi_imtime.cpp:284-287; lattice/fourier.hpp:99-130).
 * chi_wr [2 nw - 1, n_r, n_target] -> chi_tr [n_tau, n_r, n_target];
 * n_tau < 0: 6 nw + 1. moments: NULL (fit) or [3][n_r * n_target] m1, m2, m3. */
int tprf_chi_tr_from_chi_wr(double beta, int nw, int n_tau, long n_r, long n_target,
                            const double *chi_wr, const double *moments, double *chi_tr,
                            void *stream);

/* Trapezoid integral over tau.
 * Replaces triqs_tprf::chi_w0r_from_chi_tr(chi_tr_cvt) (chi_imtime.hpp:82,
 * chi_imtime.cpp:250-276). -> chi_wr [1, n_r, n_target]. */
int tprf_chi_w0r_from_chi_tr(double beta, int n_tau, long n_r, long n_target,
                             const double *chi_tr, double *chi_wr, void *stream);

/* ---- (d) RPA --------------------------------------------------------------
 * chi = [I - chi0 U]^-1 chi0 on PH-grouped (rows (a,b), columns (d,c))
 * nb^2 x nb^2 matrices, for each of n_points (omega, q) points.
 * Replaces triqs_tprf::solve_rpa_PH(chi_wk_vt, array_contiguous_view<dcomplex,4>)
 *   (lattice/rpa.hpp:43, rpa.cpp:29-68).
 * chi0 [n_points, nb, nb, nb, nb], U [nb, nb, nb, nb] -> chi (same as chi0).
 * nb <= 8. */
int tprf_solve_rpa_PH(long n_points, int nb, const double *chi0, const double *U,
                      double *chi, void *stream);
/* solve_rpa_PH on a (bosonic i omega, q) mesh: chi0 and chi are
 * [2 nw - 1][dims[0] dims[1] dims[2]][nb^4], frequencies -(nw-1) .. nw-1 and q
 * row-major over dims, as the reference's chi_wk. Same result as
 * tprf_solve_rpa_PH; knowing the mesh, it solves a point pair (w, q), (-w, -q)
 * once where U is real and chi0(-w, -q) is bit for bit conj(chi0(w, q)) (a
 * bubble of real hoppings from tprf_imtime_bubble_chi0_wk is), since the
 * elimination then gives the conjugate result bit for bit (up to the signs of
 * zeros). In place (chi == chi0) allowed. Reference: rpa.cpp:29-68 (solve_rpa_PH). */
int tprf_solve_rpa_PH_wk(int nw, const int dims[3], int nb, const double *chi0, const double *U, double *chi,
                         void *stream);

/* imtime_bubble_chi0_wk followed by solve_rpa_PH (lattice_utils.py:191-269,
 * rpa.cpp:29-68) with chi written to host memory (chi_host: pinned, shape of
 * chi_wk). chi0_wk is a device buffer of chi_wk's shape, used as scratch (it
 * ends holding chi0 for the frequencies the blocks transformed). The r -> q
 * transform, the RPA and the copies to the host run in blocks of block_freqs
 * bosonic frequencies with `slots` device buffers (1..32), so that the copy of
 * one block overlaps the solve of the next. With a slot for every block, a
 * call's solves never wait for its own copies, and with wait = 0 those copies
 * drain behind the next call's chain. Same chi as the two calls. With a
 * real bubble and a real U, chi(-w, q) = conj(chi(w, -q)) exactly, and only the
 * frequencies w >= 0 cross to the host: host threads fill the others there.
 * Stream-ordered: `stream` waits for the last copy, and with sync checks on
 * (tprf_set_sync_checks) the call returns when chi is on the host. No
 * reference counterpart as one call. */
size_t tprf_imtime_bubble_rpa_to_host_workspace_bytes(int n_iw, int n_tau, int nw, const int dims[3], int nb,
                                                      int block_freqs, int slots);
int tprf_imtime_bubble_rpa_to_host(double beta, int n_iw, int n_tau, int nw, const int dims[3], int nb,
                                   const double *g_wk, const double *moments, const double *U, double *chi0_wk,
                                   double *chi_host, int block_freqs, int slots, void *workspace,
                                   size_t workspace_bytes, void *stream);
/* The same call without the final wait: the copies of chi keep running on the
 * library's copy stream of the device after the compute on `stream` is done,
 * so that the next call's chain overlaps them (a pipeline over many inputs;
 * that call's solves wait for the device buffers they reuse). chi_host is
 * complete once `stream` gets past tprf_imtime_bubble_rpa_to_host_join(stream)
 * (a device-wide synchronisation alone does not wait for the host threads that
 * fill the negative frequencies). Do not reuse chi_host or chi0_wk before then. */
int tprf_imtime_bubble_rpa_to_host_async(double beta, int n_iw, int n_tau, int nw, const int dims[3], int nb,
                                         const double *g_wk, const double *moments, const double *U,
                                         double *chi0_wk, double *chi_host, int block_freqs, int slots,
                                         void *workspace, size_t workspace_bytes, void *stream);
/* `stream` waits for every copy the calls above have enqueued on this device
 * and for the host threads' fill of every such call. */
int tprf_imtime_bubble_rpa_to_host_join(void *stream);
/* Bytes the last of these calls on this device copied from the device to the host. */
size_t tprf_imtime_bubble_rpa_to_host_last_d2h_bytes(void);
/* Host-side record of the last of these calls on this device, for diagnosing
 * the end-to-end time: out[0] bytes copied to the host, out[1] summed duration
 * of its device-to-host copies (ms, CUDA events around each copy), out[2] span
 * from the start of the first copy to the end of the last (ms), out[3] span of
 * the host threads' fill of the negative frequencies (ms, 0 without a fill),
 * out[4] summed fill-job time (ms), out[5] distinct host CPUs the fill jobs ran
 * on, out[6] copies, out[7] fill threads of the pool, out[8] 1 when the call
 * took the real-bubble path (conjugate pairs), out[9] fraction of the
 * frequency blocks whose negative frequencies crossed the link (1 when the host
 * filled none). Writes min(n, 10) values. Waits for that call's copies and
 * fill to finish. No reference counterpart. */
int tprf_imtime_bubble_rpa_to_host_last_stats(double *out, int n);
/* Where the negative frequencies of a real chi come from when only some need to
 * cross the link (a real bubble and a real U): mode 1 fills all of them on the
 * host from the rows w >= 0 (half the link bytes, twice the host-memory traffic
 * of a copy), mode 0 copies every row over the link, mode -1 (default) splits the
 * frequency blocks between the two, moving the split on every completed call
 * toward the point where the link's and the host threads' measured times meet.
 * Per device, process-wide. The fill runs on one host thread per CPU the
 * process may use (at most 16; the environment variable TPRF_HOST_FILL_THREADS,
 * 1..64, read once, overrides the count). No reference counterpart. */
int tprf_set_host_fill(int mode);
/* A fixed split: the negative frequencies of a fraction f in [0, 1] of the
 * frequency blocks cross the link, the others are filled on the host (f = 1 is
 * mode 0, f = 0 mode 1). TPRF_ERR_INVALID_ARGUMENT outside [0, 1];
 * tprf_set_host_fill(-1) returns to the adaptive split. Per device,
 * process-wide. No reference counterpart. */
int tprf_set_host_fill_fraction(double f);

/* solve_rpa_PH with chi written to HOST memory, as the reference's C++ function
 * returns it (rpa.cpp:29-68 returns a host gf). The points are solved in chunks
 * of `chunk_points` into a device ring held in `workspace` (one slot per chunk of
 * tprf_solve_rpa_PH_to_host_workspace_bytes(chunk_points, nb, 1); up to 16 slots
 * are used), and each solved chunk is copied to chi_host on an internal copy
 * stream while the next one is solved. chi_host should be pinned (page-locked)
 * for the copies to overlap. Stream-ordered: `stream` waits for the last copy.
 * Calls are serialised by a process-wide lock while they enqueue. */
size_t tprf_solve_rpa_PH_to_host_workspace_bytes(long chunk_points, int nb, int slots);
int tprf_solve_rpa_PH_to_host(long n_points, int nb, const double *chi0, const double *U,
                              double *chi_host, long chunk_points, void *workspace,
                              size_t workspace_bytes, void *stream);

/* ---- whole chain ------------------------------------------------------------
 * g_wk -> chi0_wk as triqs_tprf.lattice_utils.imtime_bubble_chi0_wk
 * (python/triqs_tprf/lattice_utils.py:191-269): k->r, iv->tau, bubble, tau->iw
 * (nw > 1) or trapezoid (nw == 1), r->q. chi0(tau, r) is never stored.
 * Intermediate G(iv, r), G(tau, r) and a double-float copy of G(tau, r) (the
 * bubble's FFT input is formed from the copy; the tail-fit samples from the
 * complex128 values) live in the caller's workspace, whose size
 * tprf_imtime_bubble_workspace_bytes returns. chi0_wk [2nw-1, N_k, nb^4]. */
size_t tprf_imtime_bubble_workspace_bytes(int n_iw, int n_tau, const int dims[3], int nb);
int tprf_imtime_bubble_chi0_wk(double beta, int n_iw, int n_tau, int nw, const int dims[3],
                               int nb, const double *g_wk, const double *moments,
                               double *chi0_wk, void *workspace, size_t workspace_bytes,
                               void *stream);
/* The same, recording events[0..4] (cudaEvent_t, each may be NULL) on `stream`
 * before k->r and after k->r, iv->tau, the bubble + tau->iw and r->q: the
 * per-stage timing of the benchmark. No reference counterpart. */
int tprf_imtime_bubble_chi0_wk_timed(double beta, int n_iw, int n_tau, int nw, const int dims[3],
                                     int nb, const double *g_wk, const double *moments,
                                     double *chi0_wk, void *workspace, size_t workspace_bytes,
                                     void *const *events, void *stream);

/* ---- GW consumers of the chain ----------------------------------------------------
 * bubble_PI_wk (python/triqs_tprf/gw.py:56-91) is tprf_imtime_bubble_chi0_wk
 * with nw = n_iw.
 *
 * Dynamic GW self energy sigma_ab(tau, r) = - sum_cd W_acdb(tau, r) G_cd(tau, r).
 * Replaces triqs_tprf::gw_dynamic_sigma(chi_tr_cvt W_tr, g_tr_cvt g_tr)
 *   (gw.hpp:158, gw.cpp:66-84).
 * W_tr [n_tau, n_r, nb, nb, nb, nb], g_tr [n_tau, n_r, nb, nb] -> sigma_tr (as g_tr). */
int tprf_gw_dynamic_sigma(long n_tau, long n_r, int nb, const double *W_tr, const double *g_tr,
                          double *sigma_tr, void *stream);

/* Screened interaction W(iw, k) from the bubble PI(iw, k).
 * v_kind 0: static V [n_k, nb^4]; replaces
 *   triqs_tprf::dynamical_screened_interaction_W(chi_wk_cvt PI_wk, chi_k_cvt V_k)
 *   (dynamical_screened_interaction.hpp:44, .cpp:85-124):
 *   W = sum_ef V(a,b,e,f) D^-1(e,f,c,d), D = delta_ad delta_bc - sum_ef PI(a,b,e,f) V(e,f,c,d).
 * v_kind 1: dynamic V [n_w, n_k, nb^4]; replaces the chi_wk_cvt V_wk overload
 *   (.cpp:30-80): W = V [I - PI V]^-1 on PH-grouped matrices.
 * PI_wk, W_wk [n_w, n_k, nb, nb, nb, nb]; nb <= 8; FP64. */
int tprf_dynamical_screened_interaction_W(long n_w, long n_k, int nb, const double *PI_wk,
                                          const double *V, int v_kind, double *W_wk, void *stream);

/* chi_const(k) = the constant (0th) moment of the tail fit of chi(iw, k) on the
 * bosonic mesh (the fit of tprf_tail_fit_matrix_stat), chi_dyn = chi - chi_const.
 * Replaces triqs_tprf::split_into_dynamic_wk_and_constant_k(chi_wk_cvt)
 *   (lattice_utility.hpp:47, lattice_utility.cpp:57-85).
 * chi_wk, chi_dyn_wk [2 nw - 1, n_k, n_target], chi_const_k [n_k, n_target]. */
int tprf_split_into_dynamic_wk_and_constant_k(double beta, int nw, long n_k, long n_target,
                                              const double *chi_wk, double *chi_dyn_wk,
                                              double *chi_const_k, void *stream);

/* ---- analytic Lindhard bubble (validation) ------------------------------------------
 * chi00_abcd(iw, q) = 1/N_k sum_k sum_ij U_k(a,i) U_k^*(d,i) U_k+q(c,j) U_k+q^*(b,j)
 *   (f(e_ki) - f(e_k+q,j)) / (iw + e_k+q,j - e_ki), with the eigen-decomposition of
 *   e(k) - mu and the w = 0 degenerate limit beta / (4 cosh^2(beta e / 2)).
 * Replaces triqs_tprf::lindhard_chi00(e_k_cvt, mesh::imfreq, double mu)
 *   (lindhard_chi00.hpp:97, lindhard_chi00.cpp:34-100). Cost O(N_k^2 nb^6 nw).
 * e_k [n_k, nb, nb] (dims[0] dims[1] dims[2] = n_k) -> chi_wk [2 nw - 1, n_k, nb^4];
 * workspace: tprf_lindhard_chi00_workspace_bytes(n_k, nb) bytes of device memory. */
size_t tprf_lindhard_chi00_workspace_bytes(long n_k, int nb);
int tprf_lindhard_chi00(long n_k, const int dims[3], int nb, const double *e_k, double beta, double mu,
                        int nw, double *chi_wk, void *workspace, size_t workspace_bytes, void *stream);

/* ---- adjoints (differentiable path) ---------------------------------------------
 * Gradients for a real loss, in the conjugate-Wirtinger convention (for a
 * linear map y = M x, x_grad = M^H y_grad), used by the torch.autograd
 * function of the Python package. The reference has no derivatives; each
 * entry point is the transpose of the forward entry point named.
 *  - tprf_solve_rpa_PH_adjoint: transpose of tprf_solve_rpa_PH. Writes
 *    chi0_grad = A^-H chi_grad (I + U chi)^H per point (A = I - chi0 U,
 *    PH-grouped) and ADDS sum_points chi^H chi_grad chi^H to U_grad [nb^4]
 *    (zero it first). nb <= 3.
 *  - tprf_chi_wr_from_chi_tr_adjoint: transpose of tprf_chi_wr_from_chi_tr
 *    (FFT part and fit_derivatives tail terms).
 *  - tprf_chi0_tr_from_grt_PH_adjoint: transpose (in the bubble's first
 *    argument, by the product rule over both G factors) of
 *    tprf_chi0_tr_from_grt_PH: g_tr_grad [n_tau, N_r, nb, nb].
 *  - tprf_fourier_wr_to_tr_adjoint: transpose of tprf_fourier_wr_to_tr, with
 *    the moments from the tail fit (fitted = 1) or held fixed (fitted = 0).
 *  - tprf_lattice_dyson_g_wk_adjoint: e_k_grad[k] = sum_v G^H G_grad G^H.
 * The lattice FFTs are their own adjoints up to scaling: the transpose of
 * k -> r (1/N_k FFTW_FORWARD) is tprf_fourier_wr_to_wk / N_k, that of r -> k
 * is N_k tprf_fourier_wk_to_wr. */
int tprf_solve_rpa_PH_adjoint(long n_points, int nb, const double *chi0, const double *U, const double *chi,
                              const double *chi_grad, double *chi0_grad, double *U_grad, void *stream);
int tprf_chi_wr_from_chi_tr_adjoint(double beta, int n_tau, int nw, long n_r, long n_target,
                                    const double *chi_wr_grad, double *chi_tr_grad, void *stream);
int tprf_chi0_tr_from_grt_PH_adjoint(int n_tau, const int dims[3], int nb, const double *g_tr,
                                     const double *chi0_tr_grad, double *g_tr_grad, void *stream);
/* Transpose of tprf_chi0_wr_from_grt_PH (the bubble fused with tau -> i omega):
 * g_tr_grad [n_tau, N_r, nb, nb] from chi0_wr_grad [2 nw - 1, N_r, nb^4]. Each
 * bubble column's tau -> i omega transpose stays in shared memory and adds its
 * two product-rule terms to g_tr_grad, so chi0_grad(tau, r) is never stored
 * (the order of the additions, by atomics, varies at rounding level). */
int tprf_chi0_wr_from_grt_PH_adjoint(double beta, int n_tau, int nw, const int dims[3], int nb, const double *g_tr,
                                     const double *chi0_wr_grad, double *g_tr_grad, void *stream);
int tprf_fourier_wr_to_tr_adjoint(double beta, int n_iw, int n_tau, long n_r, long n_target,
                                  const double *g_tr_grad, int fitted, double *g_wr_grad, void *stream);
int tprf_lattice_dyson_g_wk_adjoint(int n_iw, long n_k, int nb, const double *g_wk, const double *g_wk_grad,
                                    double *e_k_grad, void *stream);

/* ---- batched instances --------------------------------------------------------
 * Many independent instances of the whole path (Dyson -> k->r -> iv->tau ->
 * bubble + tau->iw -> r->q -> RPA), each with its own beta, mu, meshes, nb and
 * vertex, run by one graph launch. The reference runs instances one call at
 * a time (a Python loop over lattice_dyson_g0_wk / imtime_bubble_chi0_wk /
 * solve_rpa_PH, python/triqs_tprf/lattice_utils.py:191-269, rpa.cpp:29-68);
 * this is the batched form of that loop. Per instance: e_k [N_k, nb, nb],
 * U [nb^4], chi [2 nw - 1, N_k, nb^4] (device pointers, caller owned);
 * n_tau = -1 selects 6 n_iw + 1; nw == 1 uses the trapezoid (static) branch. */
typedef struct {
  double beta, mu;
  int n_iw, n_tau, nw, nb;
  int dims[3];
  const double *e_k;
  const double *U;
  double *chi;
} tprf_instance;
typedef struct tprf_batch tprf_batch;

/* Workspace for tprf_batch_create with n_streams concurrent streams: each
 * stream reuses one slot sized for its largest instance. */
size_t tprf_batch_workspace_bytes(const tprf_instance *inst, int n, int n_streams);
/* Plans every instance, runs it once (eagerly, to build the plans), then
 * captures all instances, spread longest-first over n_streams streams, into
 * one CUDA graph. The instance array is copied; the device buffers it points
 * to and the workspace must stay valid until tprf_batch_destroy. */
int tprf_batch_create(const tprf_instance *inst, int n, int n_streams, void *workspace, size_t workspace_bytes,
                      tprf_batch **out);
/* One graph launch on `stream` computing chi for every instance. */
int tprf_batch_run(tprf_batch *batch, void *stream);
int tprf_batch_size(const tprf_batch *batch);
int tprf_batch_destroy(tprf_batch *batch);

/* ---- batched forward + gradient ---------------------------------------------------
 * The differentiable form of the batch: the forward graph also keeps each
 * instance's chi0 (in the caller's buffer) and a second graph runs every
 * instance's adjoint chain (RPA adjoint, r->q, tau->iw, G recomputed, bubble,
 * iv->tau, k->r, Dyson). Gradients follow the conjugate-Wirtinger convention of
 * torch: given chi_grad = dL/d conj(chi), the backward graph writes
 *   U_grad [nb^4]            dL/d conj(U)
 *   e_grad [N_k, nb, nb]     dL/d conj(e(k))                        (nullable)
 *   t_grad [N_k, nb, nb]     dL/d conj(t(R)) for every lattice vector R of the
 *                            periodic mesh, row-major R index like k, with
 *                            e(k) = sum_R t(R) e^{i k.R}: t_grad(R) =
 *                            sum_k e_grad(k) e^{-i k.R}             (nullable)
 * No reference counterpart (the reference has no gradients); the single-instance
 * adjoints above are the same maps. nw must be >= 2 (the trapezoid branch has no
 * adjoint here). All buffers are device memory and must outlive the batch. */
typedef struct {
  tprf_instance inst;
  double *chi0;            /* [2nw-1, N_k, nb^4], written by the forward graph */
  const double *chi_grad;  /* same shape as chi, read by the backward graph */
  double *U_grad;
  double *e_grad;
  double *t_grad;
} tprf_grad_instance;

size_t tprf_batch_grad_workspace_bytes(const tprf_grad_instance *inst, int n, int n_streams);
/* Plans, runs forward and backward once eagerly, then captures both graphs.
 * tprf_batch_run launches the forward graph of the returned batch. */
int tprf_batch_grad_create(const tprf_grad_instance *inst, int n, int n_streams, void *workspace,
                           size_t workspace_bytes, tprf_batch **out);
/* One graph launch computing every instance's gradients from its chi_grad. */
int tprf_batch_backward(tprf_batch *batch, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* TPRF_GB300_H */
