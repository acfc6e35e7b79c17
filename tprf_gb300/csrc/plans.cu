// Host-side context of tprf_gb300: status reporting, the per-device error
// word, and the plan caches (FFT twiddles, Matsubara tail tables, tail-fit
// matrices). Plans are built once per key, uploaded synchronously and kept
// for the life of the process.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

#include <cuda.h>

#include "internal.hpp"

namespace tprf {

namespace {
thread_local std::string g_last_error;
std::atomic<bool> g_sync_checks{true};
std::atomic<int> g_arith{kArithDF64};
std::mutex g_mutex;

using cd = std::complex<double>;

// Device allocations owned by the plan caches; released at process exit by
// the driver, never by us (a static destructor may run after the context).
template <class T>
int upload(const std::vector<T> &h, const T **out) {
  void *d = nullptr;
  size_t bytes = std::max<size_t>(1, h.size()) * sizeof(T);
  cudaError_t e = cudaMalloc(&d, bytes);
  if (e != cudaSuccess) return cuda_status(e, "cudaMalloc(plan table)");
  if (!h.empty()) {
    e = cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_status(e, "cudaMemcpy(plan table)");
  }
  *out = static_cast<const T *>(d);
  return TPRF_OK;
}

int current_device(int *dev) {
  cudaError_t e = cudaGetDevice(dev);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  return TPRF_OK;
}

double2 to_d2(cd z) { return make_double2(z.real(), z.imag()); }

float4 to_df(cd z) {
  const float rh = (float)z.real(), ih = (float)z.imag();
  return make_float4(rh, (float)(z.real() - (double)rh), ih, (float)(z.imag() - (double)ih));
}

std::vector<float4> to_df(const std::vector<double2> &v) {
  std::vector<float4> out(v.size());
  for (size_t i = 0; i < v.size(); ++i) out[i] = to_df(cd(v[i].x, v[i].y));
  return out;
}

// exp(sign 2 pi i k / L) for k < L, with the angle reduced exactly
std::vector<cd> unit_roots(int L, double sign) {
  std::vector<cd> w(L);
  for (int k = 0; k < L; ++k) {
    const double a = sign * 2.0 * M_PI * (double)k / (double)L;
    w[k] = cd(std::cos(a), std::sin(a));
  }
  return w;
}

}  // namespace

int current_context_key(unsigned long long *key) {
  using GetCurrent = CUresult (*)(CUcontext *);
  using GetId = CUresult (*)(CUcontext, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
  });
  int dev = 0;
  if (int st = current_device(&dev)) return st;
  unsigned long long id = 0;
  if (get_current && get_id) {
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) {
      cudaError_t e = cudaFree(nullptr);  // the runtime creates the device's context on first use
      if (e != cudaSuccess) return cuda_status(e, "cudaFree(nullptr)");
      if (get_current(&ctx) != CUDA_SUCCESS) ctx = nullptr;
    }
    if (ctx == nullptr || get_id(ctx, &id) != CUDA_SUCCESS) id = 0;
  }
  *key = id != 0 ? id : ((1ull << 63) | (unsigned long long)dev);
  return TPRF_OK;
}

int set_error(int status, const std::string &msg) {
  g_last_error = msg;
  return status;
}

int cuda_status(cudaError_t e, const char *what) {
  return set_error(TPRF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bool sync_checks_enabled() { return g_sync_checks.load(); }

std::atomic<unsigned long long> g_kernel_launches{0};
thread_local bool t_tallying = false;
thread_local unsigned long long t_tally = 0;
void count_launch() {
  if (t_tallying)
    ++t_tally;
  else
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
}
void count_graph_launch(unsigned long long kernels) { g_kernel_launches.fetch_add(kernels, std::memory_order_relaxed); }
void begin_capture_tally() {
  t_tallying = true;
  t_tally = 0;
}
unsigned long long end_capture_tally() {
  t_tallying = false;
  return t_tally;
}

int arith_mode() { return g_arith.load(); }

std::atomic<unsigned long long> g_wait_limit_ns{200000000ull};  // 200 ms
unsigned long long device_wait_limit_ns() { return g_wait_limit_ns.load(); }

unsigned *device_status_word() {
  static std::map<unsigned long long, unsigned *> words;
  unsigned long long dev = 0;
  if (current_context_key(&dev) != TPRF_OK) return nullptr;
  std::lock_guard<std::mutex> lock(g_mutex);
  auto it = words.find(dev);
  if (it != words.end()) return it->second;
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, sizeof(unsigned));
  if (e != cudaSuccess) {
    cuda_status(e, "cudaMalloc(status word)");
    return nullptr;
  }
  e = cudaMemset(p, 0, sizeof(unsigned));
  if (e != cudaSuccess) {
    cuda_status(e, "cudaMemset(status word)");
    return nullptr;
  }
  words[dev] = static_cast<unsigned *>(p);
  return static_cast<unsigned *>(p);
}

int read_and_clear_status(cudaStream_t stream, unsigned *flags) {
  unsigned *w = device_status_word();
  if (!w) return TPRF_ERR_CUDA;
  TPRF_CUDA(cudaMemcpyAsync(flags, w, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
  TPRF_CUDA(cudaMemsetAsync(w, 0, sizeof(unsigned), stream));
  TPRF_CUDA(cudaStreamSynchronize(stream));
  return TPRF_OK;
}

int status_from_flags(unsigned f, const char *what) {
  if (f & kDevErrRange)
    return set_error(TPRF_ERR_RANGE, std::string(what) + ": max |G| outside [1e-15, 1e15], the double-float range "
                                                         "of the chain; run it with TPRF_ARITH_FP64");
  if (f & kDevErrTailFit)
    return set_error(TPRF_ERR_TAIL_FIT, std::string(what) + ": high frequency moments have an error greater than 1e-3");
  if (f & kDevErrSingular) return set_error(TPRF_ERR_SINGULAR, std::string(what) + ": singular matrix");
  if (f & kDevErrNonFinite) return set_error(TPRF_ERR_NONFINITE, std::string(what) + ": non-finite value");
  if (f & kDevErrTimeout) return set_error(TPRF_ERR_CUDA, std::string(what) + ": device wait timed out");
  return TPRF_OK;
}

int finish_with_checks(cudaStream_t stream, const char *what) {
  TPRF_LAUNCH_CHECK(what);
  if (!sync_checks_enabled()) return TPRF_OK;
  unsigned f = 0;
  int st = read_and_clear_status(stream, &f);
  if (st != TPRF_OK) return st;
  return status_from_flags(f, what);
}

int max_smem_optin() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v > 0 ? v : 48 * 1024;
}

int num_sms() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
  return v > 0 ? v : 1;
}

// ---------------------------------------------------------------------------
// FFT plans

static bool factorize(int n, int *radix, int *nst) {
  int m = n, s = 0;
  while (m % 8 == 0 && s < kMaxStages) { radix[s++] = 8; m /= 8; }
  if (m % 4 == 0 && s < kMaxStages) { radix[s++] = 4; m /= 4; }
  if (m % 2 == 0 && s < kMaxStages) { radix[s++] = 2; m /= 2; }
  for (int r : {3, 5, 7})
    while (m % r == 0 && s < kMaxStages) { radix[s++] = r; m /= r; }
  // remaining prime factors: generic radix stages
  for (int r = 11; (long)r * r <= m && s < kMaxStages; r += 2)
    while (m % r == 0 && s < kMaxStages) { radix[s++] = r; m /= r; }
  if (m > 1 && s < kMaxStages) { radix[s++] = m; m = 1; }
  *nst = s;
  return m == 1;
}

// Radix orders the autotuner chooses among (the same factors in another order,
// which changes the stage count and which radix the last stage has):
//   0: 8s, one 4, one 2, then 3s, 5s, 7s, larger primes (factorize);
//   1: 4s and at most one 2 instead of 8s, then the odd factors;
//   2: the odd factors first, then 8s, one 4, one 2;
//   3: the leftover 2 or 4 of the power of two first, then 8s, then the odd factors.
static bool factorize_variant(int n, int v, int *radix, int *nst) {
  if (v == 0) return factorize(n, radix, nst);
  int m = n, p2 = 0;
  while (m % 2 == 0) {
    m /= 2;
    ++p2;
  }
  int odd[kMaxStages], no = 0, mo = m;
  for (int r : {3, 5, 7})
    while (mo % r == 0 && no < kMaxStages) { odd[no++] = r; mo /= r; }
  for (int r = 11; (long)r * r <= mo && no < kMaxStages; r += 2)
    while (mo % r == 0 && no < kMaxStages) { odd[no++] = r; mo /= r; }
  if (mo > 1 && no < kMaxStages) { odd[no++] = mo; mo = 1; }
  int pw[kMaxStages], np = 0;  // the power-of-two stages of this variant
  if (v == 1) {
    for (int e = p2; e >= 2; e -= 2) pw[np++] = 4;
    if (p2 % 2) pw[np++] = 2;
  } else if (v == 2) {
    int e = p2;
    for (; e >= 3; e -= 3) pw[np++] = 8;
    if (e == 2) pw[np++] = 4;
    if (e == 1) pw[np++] = 2;
  } else {
    if (p2 % 3 == 1) pw[np++] = 2;
    if (p2 % 3 == 2) pw[np++] = 4;
    for (int e = p2 - p2 % 3; e >= 3; e -= 3) pw[np++] = 8;
  }
  if (np + no > kMaxStages || mo != 1) return false;
  int s = 0;
  if (v == 2) {
    for (int i = 0; i < no; ++i) radix[s++] = odd[i];
    for (int i = 0; i < np; ++i) radix[s++] = pw[i];
  } else {
    for (int i = 0; i < np; ++i) radix[s++] = pw[i];
    for (int i = 0; i < no; ++i) radix[s++] = odd[i];
  }
  *nst = s;
  return true;
}

std::vector<int> fft_variants(int n) {
  std::vector<int> out;
  std::vector<std::vector<int>> seen;
  for (int v = 0; v < kFftVariants; ++v) {
    int radix[kMaxStages], nst = 0;
    if (!factorize_variant(n, v, radix, &nst)) continue;
    std::vector<int> seq(radix, radix + nst);
    bool dup = false;
    for (const auto &x : seen) dup = dup || x == seq;
    if (dup) continue;
    seen.push_back(seq);
    out.push_back(v);
  }
  return out;
}

int get_fft(int n, FftDesc *out) { return get_fft_variant(n, 0, out); }

int get_fft_variant(int n, int variant, FftDesc *out) {
  if (n < 1) return set_error(TPRF_ERR_INVALID_ARGUMENT, "FFT length must be >= 1");
  unsigned long long dev = 0;  // the context: plans die with it
  int st = current_context_key(&dev);
  if (st) return st;
  static std::map<std::tuple<unsigned long long, int, int>, FftDesc> cache;
  std::lock_guard<std::mutex> lock(g_mutex);
  auto key = std::make_tuple(dev, n, variant);
  auto it = cache.find(key);
  if (it != cache.end()) {
    *out = it->second;
    return TPRF_OK;
  }
  FftDesc d{};
  d.n = n;
  if (!factorize_variant(n, variant, d.radix, &d.nst))
    return set_error(TPRF_ERR_UNSUPPORTED_SIZE, "FFT length " + std::to_string(n) + " has too many factors");
  std::vector<double2> tw(n);
  for (int t = 0; t < n; ++t) {
    const double a = -2.0 * M_PI * (double)t / (double)n;
    tw[t] = make_double2(std::cos(a), std::sin(a));
  }
  std::vector<float4> twf(n);
  for (int t = 0; t < n; ++t) {
    const float rh = (float)tw[t].x, ih = (float)tw[t].y;
    twf[t] = make_float4(rh, (float)(tw[t].x - (double)rh), ih, (float)(tw[t].y - (double)ih));
  }
  // digit reversal for the in-place decimation-in-time stages: position
  // p = p_0 + R_0 p_1 + R_0 R_1 p_2 + ... holds natural index
  // sigma(p) = sum_k p_k n / (R_0 ... R_k); rev is its inverse.
  std::vector<int> rev(n);
  for (int p = 0; p < n; ++p) {
    long q = p, prod = 1, sig = 0;
    for (int s = 0; s < d.nst; ++s) {
      const int R = d.radix[s];
      const long dg = q % R;
      q /= R;
      prod *= R;
      sig += dg * (n / prod);
    }
    rev[sig] = p;
  }
  d.has_generic = 0;
  for (int s = 0; s < d.nst; ++s)
    if (d.radix[s] > 8 || d.radix[s] == 6) d.has_generic = 1;
  st = upload(tw, &d.tw);
  if (st) return st;
  st = upload(twf, &d.twf);
  if (st) return st;
  st = upload(rev, &d.rev);
  if (st) return st;
  cache[key] = d;
  *out = d;
  return TPRF_OK;
}

// ---------------------------------------------------------------------------
// Tail fit: a linear least-squares fit of g(iw) ~ sum_{p<=P} c_p (iw)^-p on
// the outer 20% of the mesh's positive frequency indices (at most 30 points a
// side, both signs), frequencies normalised by omega_max; the order P is the
// largest with omega_max^P <= 1e16, at most 9. This restates the method of
// TRIQS's fit_tail (called at fourier_matsubara.cpp:226); the TRIQS code
// itself is not part of the reference tree. A fermionic mesh (n = n_freq)
// holds iv_n for n = -n .. n-1 and fits the indices 0 .. n-1; a bosonic one
// (n = nw) holds iw_m for m = -(nw-1) .. nw-1 and fits the indices 1 .. nw-1.

static void tail_fit_points(int n, bool fermion, std::vector<int> *rows) {
  const int i_min = fermion ? 0 : 1, i_max = n - 1;
  const int count = i_max - i_min + 1;
  int n_pts = std::max(1, std::min((2 * count + 5) / 10, 30));
  int n_hi = i_max;
  int n_lo = std::min(n_hi, i_min + (8 * count + 5) / 10);
  std::vector<int> pos;
  if (n_pts == 1) {
    pos.push_back(n_hi);
  } else {
    const int span = n_hi - n_lo;
    for (int j = 0; j < n_pts; ++j) pos.push_back(n_lo + (2 * j * span + (n_pts - 1)) / (2 * (n_pts - 1)));
  }
  rows->clear();
  if (fermion) {
    for (int i = (int)pos.size() - 1; i >= 0; --i) rows->push_back(-pos[i] - 1 + n);
    for (int p : pos) rows->push_back(p + n);
  } else {
    for (int i = (int)pos.size() - 1; i >= 0; --i) rows->push_back(-pos[i] + n - 1);
    for (int p : pos) rows->push_back(p + n - 1);
  }
}

static double mesh_omega_max(double beta, int n, bool fermion) {
  return fermion ? (2.0 * n - 1.0) * M_PI / beta : 2.0 * (n - 1) * M_PI / beta;
}

// the Matsubara frequency of data index i of a mesh
static cd mesh_freq(double beta, int n, bool fermion, int i) {
  return fermion ? cd(0.0, (2.0 * (i - n) + 1.0) * M_PI / beta) : cd(0.0, 2.0 * (i - (n - 1)) * M_PI / beta);
}

static int tail_order(double omega_max, int n_eq) {
  int order = 9;
  if (omega_max > 1.0) order = (int)std::floor(16.0 * std::log(10.0) / std::log(omega_max));
  order = std::min(order, 9);
  order = std::min(order, n_eq - 1);
  return std::max(order, 0);
}

// Pseudo-inverse of a full-column-rank m x n complex matrix (row-major) by
// Householder QR: pinv = R^-1 Q^H. Returns false if rank deficient.
static bool pinv_householder(std::vector<cd> A, int m, int n, std::vector<cd> *pinv) {
  std::vector<cd> QH(m * m, cd(0));
  for (int i = 0; i < m; ++i) QH[i * m + i] = 1.0;
  std::vector<cd> v(m);
  for (int k = 0; k < n; ++k) {
    double nrm2 = 0;
    for (int i = k; i < m; ++i) nrm2 += std::norm(A[i * n + k]);
    const double nrm = std::sqrt(nrm2);
    if (nrm == 0.0) return false;
    const cd akk = A[k * n + k];
    const cd phase = (std::abs(akk) > 0) ? akk / std::abs(akk) : cd(1.0);
    const cd alpha = -phase * nrm;
    double vn2 = 0;
    for (int i = k; i < m; ++i) {
      v[i] = A[i * n + k] - (i == k ? alpha : cd(0));
      vn2 += std::norm(v[i]);
    }
    if (vn2 == 0.0) continue;
    for (int j = k; j < n; ++j) {
      cd s = 0;
      for (int i = k; i < m; ++i) s += std::conj(v[i]) * A[i * n + j];
      s *= 2.0 / vn2;
      for (int i = k; i < m; ++i) A[i * n + j] -= v[i] * s;
    }
    for (int j = 0; j < m; ++j) {
      cd s = 0;
      for (int i = k; i < m; ++i) s += std::conj(v[i]) * QH[i * m + j];
      s *= 2.0 / vn2;
      for (int i = k; i < m; ++i) QH[i * m + j] -= v[i] * s;
    }
  }
  pinv->assign(n * m, cd(0));
  for (int j = 0; j < m; ++j) {
    for (int i = n - 1; i >= 0; --i) {
      cd s = QH[i * m + j];
      for (int l = i + 1; l < n; ++l) s -= A[i * n + l] * (*pinv)[l * m + j];
      if (A[i * n + i] == cd(0)) return false;
      (*pinv)[i * m + j] = s / A[i * n + i];
    }
  }
  return true;
}

static double one_fermion(double b, double tau, double beta) {
  return -(b >= 0 ? std::exp(-b * tau) / (1 + std::exp(-beta * b))
                  : std::exp(b * (beta - tau)) / (1 + std::exp(beta * b)));
}

static double one_boson(double b, double tau, double beta) {
  return (b >= 0 ? std::exp(-b * tau) / (std::exp(-beta * b) - 1)
                 : std::exp(b * (beta - tau)) / (1 - std::exp(b * beta)));
}

// Host-side definition of the tail fit for a mesh (beta, n, statistic): the
// data rows of the fit points, F (moments = F g[rows], [n_mom][n_fit]) and G
// (model value at fit point i = sum_p c_p G[i][p], G = (iw_i)^-p).
int build_tail_fit(double beta, int n, bool fermion, std::vector<int> *rows, std::vector<double2> *F,
                   std::vector<double2> *G, int *n_mom_out) {
  tail_fit_points(n, fermion, rows);
  const int n_fit = (int)rows->size();
  const double omega_max = mesh_omega_max(beta, n, fermion);
  const int P = tail_order(omega_max, n_fit);
  const int n_mom = P + 1;
  std::vector<cd> A(n_fit * n_mom);
  G->assign(n_fit * n_mom, make_double2(0, 0));
  for (int i = 0; i < n_fit; ++i) {
    const cd iw = mesh_freq(beta, n, fermion, (*rows)[i]);
    if (std::abs(iw) == 0.0) return set_error(TPRF_ERR_TAIL_FIT, "tail fit: bosonic mesh too short");
    const cd z = omega_max / iw;
    cd zp = 1.0, wp = 1.0;
    for (int q = 0; q < n_mom; ++q) {
      A[i * n_mom + q] = zp;
      (*G)[i * n_mom + q] = to_d2(wp);
      zp *= z;
      wp /= iw;
    }
  }
  std::vector<cd> pinv;
  if (!pinv_householder(A, n_fit, n_mom, &pinv))
    return set_error(TPRF_ERR_TAIL_FIT, "tail fit design matrix is rank deficient");
  F->assign(n_mom * n_fit, make_double2(0, 0));
  double scale = 1.0;
  for (int q = 0; q < n_mom; ++q) {
    for (int i = 0; i < n_fit; ++i) (*F)[q * n_fit + i] = to_d2(scale * pinv[q * n_fit + i]);
    scale *= omega_max;
  }
  *n_mom_out = n_mom;
  return TPRF_OK;
}

int get_nu_tau_plan(double beta, int n_iw, int n_tau, const NuTauPlan **out) {
  return get_nu_tau_plan_stat(beta, n_iw, n_tau, true, out);
}

// Matsubara -> tau for either statistic (fourier_matsubara.cpp:218-308): n is
// the fermionic n_max or the bosonic nw.
int get_nu_tau_plan_stat(double beta, int n, int n_tau, bool fermion, const NuTauPlan **out) {
  unsigned long long dev = 0;  // the context: plans die with it
  int st = current_context_key(&dev);
  if (st) return st;
  static std::map<std::tuple<unsigned long long, uint64_t, int, int, int>, std::unique_ptr<NuTauPlan>> cache;
  uint64_t bbits;
  std::memcpy(&bbits, &beta, 8);
  auto key = std::make_tuple(dev, bbits, n, n_tau, fermion ? 1 : 0);
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    auto it = cache.find(key);
    if (it != cache.end()) {
      *out = it->second.get();
      return TPRF_OK;
    }
  }
  auto p = std::make_unique<NuTauPlan>();
  p->beta = beta;
  p->n_iw = n;
  p->n_tau = n_tau;
  p->L = n_tau - 1;
  p->fermion = fermion ? 1 : 0;
  p->n_in = fermion ? 2 * n : 2 * n - 1;
  p->in0 = fermion ? -n : -(n - 1);
  const int L = p->L, nnu = p->n_in;
  st = get_fft(L, &p->fft);
  if (st) return st;
  const double bf[3] = {0.0, 1.0, -1.0}, bb[3] = {-0.5, -1.0, 1.0};
  const double *bj = fermion ? bf : bb;
  std::vector<double2> den(3 * nnu);
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < nnu; ++i) den[j * nnu + i] = to_d2(1.0 / (mesh_freq(beta, n, fermion, i) - bj[j]));
  std::vector<double2> phase(L);
  std::vector<double> ftail(3 * L);
  const double dtau = beta / (double)(n_tau - 1);
  for (int t = 0; t < L; ++t) {
    const double tau = (double)t * dtau;
    phase[t] = fermion ? to_d2(std::exp(cd(0.0, -M_PI * tau / beta))) : make_double2(1.0, 0.0);
    for (int j = 0; j < 3; ++j) ftail[j * L + t] = fermion ? one_fermion(bj[j], tau, beta) : one_boson(bj[j], tau, beta);
  }
  // tail fit
  std::vector<int> rows;
  std::vector<double2> F, G;
  int n_mom = 0;
  st = build_tail_fit(beta, n, fermion, &rows, &F, &G, &n_mom);
  if (st) return st;
  const int n_fit = (int)rows.size();
  p->n_fit = n_fit;
  p->n_mom = n_mom;
  // folded tail tables: FFT_FORWARD of each pole column, placed at rows (m+L)%L
  const std::vector<cd> wr = unit_roots(L, -1.0);
  std::vector<double2> P(L), Q(3 * L);
  for (int t = 0; t < L; ++t) {
    const cd Pt = cd(phase[t].x, phase[t].y) / beta;
    P[t] = to_d2(Pt);
    for (int j = 0; j < 3; ++j) {
      cd acc = 0.0;
      for (int i = 0; i < nnu; ++i) {
        const long row = ((long)(i + p->in0) + L) % L;
        acc += cd(den[j * nnu + i].x, den[j * nnu + i].y) * wr[(row * t) % L];
      }
      Q[j * L + t] = to_d2(ftail[j * L + t] - Pt * acc);
    }
  }
  if ((st = upload(den, &p->den)) || (st = upload(phase, &p->phase)) || (st = upload(ftail, &p->ftail)) ||
      (st = upload(rows, &p->fit_row)) || (st = upload(F, &p->fitF)) || (st = upload(G, &p->fitG)) ||
      (st = upload(P, &p->P)) || (st = upload(Q, &p->Q)) || (st = upload(to_df(P), &p->Pf)) ||
      (st = upload(to_df(Q), &p->Qf)) || (st = upload(to_df(F), &p->fitFf)) || (st = upload(to_df(G), &p->fitGf)))
    return st;
  std::lock_guard<std::mutex> lock(g_mutex);
  auto &slot = cache[key];
  if (!slot) slot = std::move(p);
  *out = slot.get();
  return TPRF_OK;
}

int get_tau_w_plan(double beta, int n_tau, int nw, const TauWPlan **out) {
  return get_tau_w_plan_stat(beta, n_tau, nw, false, out);
}

// tau -> Matsubara for either statistic (fourier_matsubara.cpp:123-184): n is
// the bosonic nw (outputs m = -(nw-1) .. nw-1) or the fermionic n_max
// (outputs n = -n_max .. n_max-1).
int get_tau_w_plan_stat(double beta, int n_tau, int n, bool fermion, const TauWPlan **out) {
  unsigned long long dev = 0;  // the context: plans die with it
  int st = current_context_key(&dev);
  if (st) return st;
  static std::map<std::tuple<unsigned long long, uint64_t, int, int, int>, std::unique_ptr<TauWPlan>> cache;
  uint64_t bbits;
  std::memcpy(&bbits, &beta, 8);
  auto key = std::make_tuple(dev, bbits, n_tau, n, fermion ? 1 : 0);
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    auto it = cache.find(key);
    if (it != cache.end()) {
      *out = it->second.get();
      return TPRF_OK;
    }
  }
  auto p = std::make_unique<TauWPlan>();
  p->beta = beta;
  p->n_tau = n_tau;
  p->nw = n;
  p->L = n_tau - 1;
  p->fermion = fermion ? 1 : 0;
  p->n_out = fermion ? 2 * n : 2 * n - 1;
  p->out0 = fermion ? -n : -(n - 1);
  const int L = p->L, nwt = p->n_out;
  st = get_fft(L, &p->fft);
  if (st) return st;
  const double bf[3] = {0.0, 1.0, -1.0}, bb[3] = {-0.5, -1.0, 1.0};
  const double *bj = fermion ? bf : bb;
  // the input phase exp(i pi tau / beta) of the fermionic transform, and the
  // one-pole tau functions with that phase applied
  std::vector<double2> ph(L);
  std::vector<cd> tailt(3 * L);
  const double dtau = beta / (double)(n_tau - 1);
  for (int t = 0; t < L; ++t) {
    const double tau = (double)t * dtau;
    const cd e = fermion ? std::exp(cd(0.0, M_PI * tau / beta)) : cd(1.0);
    ph[t] = to_d2(e);
    for (int j = 0; j < 3; ++j)
      tailt[j * L + t] = e * (fermion ? one_fermion(bj[j], tau, beta) : one_boson(bj[j], tau, beta));
  }
  std::vector<double2> den(3 * nwt);
  for (int j = 0; j < 3; ++j)
    for (int m = 0; m < nwt; ++m) den[j * nwt + m] = to_d2(1.0 / (mesh_freq(beta, n, fermion, m) - bj[j]));
  // folded tail tables: FFT_BACKWARD of each one-pole tau function, at the output rows
  const std::vector<cd> wb = unit_roots(L, +1.0);
  const double fact = beta / (double)L;
  std::vector<double2> K(3 * nwt);
  for (int j = 0; j < 3; ++j)
    for (int m = 0; m < nwt; ++m) {
      const long k = ((long)(m + p->out0) + L) % L;
      cd acc = 0.0;
      for (int t = 0; t < L; ++t) acc += tailt[j * L + t] * wb[(k * t) % L];
      K[j * nwt + m] = to_d2(cd(den[j * nwt + m].x, den[j * nwt + m].y) - fact * acc);
    }
  std::vector<double> btail(3 * L);
  for (int i = 0; i < 3 * L; ++i) btail[i] = std::real(tailt[i] / cd(ph[i % L].x, ph[i % L].y));
  if ((st = upload(btail, &p->btail)) || (st = upload(den, &p->den)) || (st = upload(K, &p->K)) ||
      (st = upload(to_df(K), &p->Kf)) || (st = upload(ph, &p->ph)))
    return st;
  std::lock_guard<std::mutex> lock(g_mutex);
  auto &slot = cache[key];
  if (!slot) slot = std::move(p);
  *out = slot.get();
  return TPRF_OK;
}

int get_tail_fit_plan(double beta, int n, bool fermion, const TailFitPlan **out) {
  unsigned long long dev = 0;  // the context: plans die with it
  int st = current_context_key(&dev);
  if (st) return st;
  static std::map<std::tuple<unsigned long long, uint64_t, int, int>, std::unique_ptr<TailFitPlan>> cache;
  uint64_t bbits;
  std::memcpy(&bbits, &beta, 8);
  auto key = std::make_tuple(dev, bbits, n, fermion ? 1 : 0);
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    auto it = cache.find(key);
    if (it != cache.end()) {
      *out = it->second.get();
      return TPRF_OK;
    }
  }
  std::vector<int> rows;
  std::vector<double2> F, G;
  int n_mom = 0;
  if ((st = build_tail_fit(beta, n, fermion, &rows, &F, &G, &n_mom))) return st;
  auto p = std::make_unique<TailFitPlan>();
  p->n_fit = (int)rows.size();
  p->n_mom = n_mom;
  if ((st = upload(rows, &p->rows)) || (st = upload(F, &p->F))) return st;
  std::lock_guard<std::mutex> lock(g_mutex);
  auto &slot = cache[key];
  if (!slot) slot = std::move(p);
  *out = slot.get();
  return TPRF_OK;
}

int get_orb_canon(int nb, const OrbCanon **out) {
  if (nb < 1 || nb > 8) return set_error(TPRF_ERR_INVALID_ARGUMENT, "orbital canon: bad nb");
  unsigned long long dev = 0;  // the context: tables die with it
  int st = current_context_key(&dev);
  if (st) return st;
  static std::map<std::tuple<unsigned long long, int>, std::unique_ptr<OrbCanon>> cache;
  auto key = std::make_tuple(dev, nb);
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    auto it = cache.find(key);
    if (it != cache.end()) {
      *out = it->second.get();
      return TPRF_OK;
    }
  }
  const int E = nb * nb * nb * nb;
  std::vector<int> ocan, orev, ocomp((size_t)E, -1);
  for (int o = 0; o < E; ++o) {
    // dcba of o = abcd: the base-nb digits in reverse order
    int x = o, r = 0;
    for (int i = 0; i < 4; ++i) {
      r = r * nb + x % nb;
      x /= nb;
    }
    if (o <= r) {
      ocomp[(size_t)o] = (int)ocan.size();
      ocan.push_back(o);
      orev.push_back(r);
    }
  }
  auto p = std::make_unique<OrbCanon>();
  p->nc = (int)ocan.size();
  if ((st = upload(ocan, &p->ocan)) || (st = upload(orev, &p->orev)) || (st = upload(ocomp, &p->ocomp))) return st;
  std::lock_guard<std::mutex> lock(g_mutex);
  auto &slot = cache[key];
  if (!slot) slot = std::move(p);
  *out = slot.get();
  return TPRF_OK;
}

int get_k_pair_order(int d1, int d2, const int **out) {
  if (d1 < 1 || d2 < 1) return set_error(TPRF_ERR_INVALID_ARGUMENT, "k pair order: bad mesh");
  unsigned long long dev = 0;  // the context: tables die with it
  int st = current_context_key(&dev);
  if (st) return st;
  static std::map<std::tuple<unsigned long long, int, int>, const int *> cache;
  auto key = std::make_tuple(dev, d1, d2);
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    auto it = cache.find(key);
    if (it != cache.end()) {
      *out = it->second;
      return TPRF_OK;
    }
  }
  std::vector<int> order;
  order.reserve((size_t)d1 * d2);
  for (int k1 = 0; k1 < d1; ++k1)
    for (int k2 = 0; k2 < d2; ++k2) {
      const int k = k1 * d2 + k2, mk = ((d1 - k1) % d1) * d2 + (d2 - k2) % d2;
      if (k < mk) {
        order.push_back(k);
        order.push_back(mk);
      } else if (k == mk) {
        order.push_back(k);
      }
    }
  const int *p = nullptr;
  if ((st = upload(order, &p))) return st;
  std::lock_guard<std::mutex> lock(g_mutex);
  auto &slot = cache[key];
  if (!slot) slot = p;
  *out = slot;
  return TPRF_OK;
}

int get_transpose_pairs(const int dims[3], int nb, int rank, const TransposePairs **out) {
  unsigned long long dev = 0;  // the context: plans die with it
  int st = current_context_key(&dev);
  if (st) return st;
  static std::map<std::tuple<unsigned long long, int, int, int, int, int>, std::unique_ptr<TransposePairs>> cache;
  auto key = std::make_tuple(dev, dims[0], dims[1], dims[2], nb, rank);
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    auto it = cache.find(key);
    if (it != cache.end()) {
      *out = it->second.get();
      return TPRF_OK;
    }
  }
  if (nb < 1 || (rank != 2 && rank != 4)) return set_error(TPRF_ERR_INVALID_ARGUMENT, "transpose pairs: bad shape");
  const long nr = (long)dims[0] * dims[1] * dims[2];
  long E = 1;
  for (int i = 0; i < rank; ++i) E *= nb;
  if (nr * E > 0x7fffffffL) return set_error(TPRF_ERR_INVALID_ARGUMENT, "transpose pairs: too many columns");
  std::vector<int> rev((size_t)E);  // element with its indices reversed
  for (long e = 0; e < E; ++e) {
    long x = e, r = 0;
    for (int i = 0; i < rank; ++i) {
      r = r * nb + x % nb;
      x /= nb;
    }
    rev[(size_t)e] = (int)r;
  }
  std::vector<int2> pairs;
  pairs.reserve((size_t)(nr * E / 2 + E));
  for (long r = 0; r < nr; ++r) {
    const long i2 = r % dims[2], i1 = (r / dims[2]) % dims[1], i0 = r / ((long)dims[2] * dims[1]);
    const long mr = (((dims[0] - i0) % dims[0]) * dims[1] + (dims[1] - i1) % dims[1]) * dims[2] + (dims[2] - i2) % dims[2];
    for (long e = 0; e < E; ++e) {
      const long c = r * E + e, t = mr * E + rev[(size_t)e];
      if (c <= t) pairs.push_back(make_int2((int)c, (int)t));
    }
  }
  auto p = std::make_unique<TransposePairs>();
  p->n_can = (long)pairs.size();
  if ((st = upload(pairs, &p->pairs))) return st;
  std::lock_guard<std::mutex> lock(g_mutex);
  auto &slot = cache[key];
  if (!slot) slot = std::move(p);
  *out = slot.get();
  return TPRF_OK;
}

// Rows 0 and 1 of the inverse of the Vandermonde matrix V[m][j] = m^j (m = 1..8)
// exactly as TPRF hard-codes them in fit_derivatives
// (c++/triqs_tprf/fourier/fourier_matsubara.cpp:56-71). They differ from the
// exact rationals (vandermonde_inverse8) by up to ~5e-12 relative; using the
// same constants keeps the tau -> i omega moments m2, m3 the reference's. Rows
// 2..7 of the table never enter the moments.
void fit_derivative_rows(double r0[8], double r1[8]) {
  static const double row0[8] = {8.000000000008853,  -28.000000000055913, 56.000000000151815, -70.00000000021936,
                                 56.00000000020795,  -28.000000000115904, 8.00000000003683,   -1.0000000000049232};
  static const double row1[8] = {-13.742857142879107, 62.10000000013776,   -133.5333333337073, 172.75000000055635,
                                 -141.00000000052023, 71.43333333362274,   -20.600000000091182, 2.592857142869304};
  for (int m = 0; m < 8; ++m) {
    r0[m] = row0[m];
    r1[m] = row1[m];
  }
}

void vandermonde_inverse8(double out[64]) {
  // Column m of the inverse holds the coefficients of the Lagrange basis
  // polynomial through nodes 1..8 that is 1 at node m+1: integer polynomial
  // prod_{k != m+1}(x - k) divided by the integer prod_{k != m+1}(m+1 - k).
  for (int col = 0; col < 8; ++col) {
    const long long node = col + 1;
    long long poly[9] = {1, 0, 0, 0, 0, 0, 0, 0, 0};
    int deg = 0;
    long long den = 1;
    for (long long k = 1; k <= 8; ++k) {
      if (k == node) continue;
      for (int i = deg + 1; i >= 1; --i) poly[i] = poly[i - 1] - k * poly[i];
      poly[0] = -k * poly[0];
      ++deg;
      den *= (node - k);
    }
    for (int j = 0; j < 8; ++j) out[j * 8 + col] = (double)poly[j] / (double)den;
  }
}

}  // namespace tprf

// ---------------------------------------------------------------------------
// C ABI: status helpers

extern "C" const char *tprf_status_string(int status) {
  switch (status) {
    case TPRF_OK: return "ok";
    case TPRF_ERR_INVALID_ARGUMENT: return "invalid argument";
    case TPRF_ERR_UNSUPPORTED_SIZE: return "unsupported FFT length";
    case TPRF_ERR_MESH_TOO_SHORT: return "time mesh too short";
    case TPRF_ERR_TAIL_FIT: return "tail fit error";
    case TPRF_ERR_NONFINITE: return "non-finite value";
    case TPRF_ERR_CUDA: return "CUDA error";
    case TPRF_ERR_ALLOC: return "allocation failed or workspace too small";
    case TPRF_ERR_SINGULAR: return "singular matrix";
    case TPRF_ERR_RANGE: return "values outside the double-float range";
    default: return "unknown status";
  }
}

extern "C" const char *tprf_last_error(void) { return tprf::g_last_error.c_str(); }

extern "C" const char *tprf_version(void) { return "0.1.0"; }

extern "C" void tprf_set_sync_checks(int on) { tprf::g_sync_checks.store(on != 0); }

extern "C" unsigned long long tprf_kernel_launches(void) { return tprf::g_kernel_launches.load(); }

extern "C" int tprf_set_arithmetic(int mode) {
  if (mode != TPRF_ARITH_DF64 && mode != TPRF_ARITH_FP64 && mode != TPRF_ARITH_DF64_ALL)
    return tprf::set_error(TPRF_ERR_INVALID_ARGUMENT, "set_arithmetic: unknown mode");
  tprf::g_arith.store(mode);
  return TPRF_OK;
}

extern "C" int tprf_get_arithmetic(void) { return tprf::g_arith.load(); }

extern "C" int tprf_set_device_wait_limit_ns(long long ns) {
  if (ns < 0) return tprf::set_error(TPRF_ERR_INVALID_ARGUMENT, "set_device_wait_limit_ns: negative limit");
  tprf::g_wait_limit_ns.store((unsigned long long)ns);
  return TPRF_OK;
}

extern "C" int tprf_check_device_status(void *stream) {
  unsigned f = 0;
  int st = tprf::read_and_clear_status(static_cast<cudaStream_t>(stream), &f);
  if (st != TPRF_OK) return st;
  return tprf::status_from_flags(f, "device status");
}

extern "C" int tprf_tail_fit_matrix(double beta, int n_iw, int capacity, int *n_fit, int *n_mom, int *rows,
                                    double *F) {
  return ::tprf_tail_fit_matrix_stat(beta, n_iw, 1, capacity, n_fit, n_mom, rows, F);
}

extern "C" int tprf_tail_fit_matrix_stat(double beta, int n, int fermion, int capacity, int *n_fit, int *n_mom,
                                         int *rows, double *F) {
  if (!(beta > 0.0) || n < 1 || !n_fit || !n_mom)
    return tprf::set_error(TPRF_ERR_INVALID_ARGUMENT, "tail_fit_matrix: bad mesh or null pointer");
  std::vector<int> r;
  std::vector<double2> f, g;
  int nm = 0;
  int st = tprf::build_tail_fit(beta, n, fermion != 0, &r, &f, &g, &nm);
  if (st) return st;
  *n_fit = (int)r.size();
  *n_mom = nm;
  if (rows && F) {
    if (capacity < (int)f.size()) return tprf::set_error(TPRF_ERR_INVALID_ARGUMENT, "tail_fit_matrix: capacity");
    for (size_t i = 0; i < r.size(); ++i) rows[i] = r[i];
    for (size_t i = 0; i < f.size(); ++i) {
      F[2 * i] = f[i].x;
      F[2 * i + 1] = f[i].y;
    }
  }
  return TPRF_OK;
}

extern "C" void tprf_vandermonde_inverse8(double out[64]) { tprf::vandermonde_inverse8(out); }
extern "C" void tprf_fit_derivative_rows(double out[16]) { tprf::fit_derivative_rows(out, out + 8); }
