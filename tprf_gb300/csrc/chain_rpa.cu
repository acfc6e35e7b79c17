// The bubble chain and the RPA in one call, with chi streamed to host memory:
// imtime_bubble_chi0_wk (lattice_utils.py:191-269) followed by solve_rpa_PH
// (rpa.cpp:29-68) as a TPRF user chains them, for callers that want chi on the
// host. Copying chi to the host (21.7 GB for the 3-orbital 32^3 case at about
// 193 GB/s on GB300) takes longer than the RPA itself, so the r -> q transform,
// the RPA and the copies run block by block over the bosonic frequencies: the
// copy of one block overlaps the transform and solve of the next, and the copy
// starts as soon as the first block is solved rather than after all of chi0.
//
// On a real bubble (the chain's real-input words) a block holds the
// frequencies m = m0 .. m1-1 >= 0: r -> q on those rows, the rows -m filled by
// symmetry, chi0(-w, q) = conj(chi0(w, -q)), and the conjugate-pair solve,
// which writes both signs. Otherwise a block is a range of rows of the whole
// mesh, transformed and solved point by point.
#include <pthread.h>
#include <sched.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"

namespace tprf {
int bubble_to_wr(double beta, int n_iw, int n_tau, int nw, const int dims[3], int nb, const double *g_wk,
                 const double *moments, double2 *out, void *workspace, size_t workspace_bytes, void *const *events,
                 cudaStream_t s, bool *chi_df, unsigned **gmax_out, CompactChi *cc);
int launch_rpa(long n_points, int nb, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream);

namespace {

constexpr int kMaxSlots = 32;

// Host threads that fill the negative frequencies of chi in host memory from
// the non-negative ones already copied there, chi(-w, q) = conj(chi(w, -q)),
// when the device solve gives exactly that (a real bubble and a real U: the
// conjugate-pair solve stores the conjugate of the same values): half the
// bytes cross the device-to-host link, which bounds the call. Jobs are
// submitted by host functions on the copy stream once a block's copy has
// landed. The copy stream does not wait for them: the next call's copies
// follow at once (holding the copy stream until each call's fill ended left
// the link idle for the fill's tail; on the 3-orbital 32^3 workload a pipelined
// step went from 127.6 to 112.3 ms with this and the word-wise fill). A stream
// joined to the copies (the waiting call, tprf_imtime_bubble_rpa_to_host_join)
// runs a host function that waits until the pool is idle, so it passes only
// when chi is complete. No CUDA calls here.
class HostPool {
 public:
  static HostPool &get() {
    static HostPool *p = new HostPool();  // never destroyed: its threads sleep until exit
    return *p;
  }
  int threads() const { return (int)n_; }
  void submit(std::function<void()> f) {
    {
      std::lock_guard<std::mutex> l(mu_);
      q_.push_back(std::move(f));
      ++outstanding_;
    }
    cv_.notify_one();
  }
  void wait_idle() {
    std::unique_lock<std::mutex> l(mu_);
    idle_.wait(l, [&] { return outstanding_ == 0; });
  }

 private:
  HostPool() {
    // one thread per CPU this process may run on, at most 16 (on the 16-core
    // GB300 host, 16 threads filled faster than 15 or 12 with the enqueuing
    // thread beside them); TPRF_HOST_FILL_THREADS (1..64) overrides the count
    unsigned cpus = 0;
    cpu_set_t set;
    CPU_ZERO(&set);
    if (sched_getaffinity(0, sizeof(set), &set) == 0) cpus = (unsigned)CPU_COUNT(&set);
    if (cpus == 0) cpus = std::thread::hardware_concurrency();
    n_ = std::max(1u, std::min(cpus, 16u));
    if (const char *env = std::getenv("TPRF_HOST_FILL_THREADS")) {
      const long v = std::strtol(env, nullptr, 10);
      if (v >= 1 && v <= 64) n_ = (unsigned)v;
    }
    for (unsigned i = 0; i < n_; ++i) {
      std::thread t([this] { run(); });
      pthread_setname_np(t.native_handle(), "tprf-host-fill");  // visible in /proc/<pid>/task/*/comm
      t.detach();
    }
  }
  void run() {
    for (;;) {
      std::function<void()> f;
      {
        std::unique_lock<std::mutex> l(mu_);
        cv_.wait(l, [&] { return !q_.empty(); });
        f = std::move(q_.front());
        q_.pop_front();
      }
      f();
      std::lock_guard<std::mutex> l(mu_);
      if (--outstanding_ == 0) idle_.notify_all();
    }
  }
  unsigned n_ = 1;
  std::mutex mu_;
  std::condition_variable cv_, idle_;
  std::deque<std::function<void()>> q_;
  long outstanding_ = 0;
};

using Clock = std::chrono::steady_clock;

// Host-side record of one call's fill of the negative frequencies: the span
// from the first job's start to the last job's end, the summed job times and
// the host CPUs the jobs ran on (sched_getcpu), read by
// tprf_imtime_bubble_rpa_to_host_last_stats.
struct FillStats {
  std::mutex mu;
  std::atomic<bool> complete{false};  // set once the call's last fill job has ended
  // jobs submitted and not yet ended, and whether the call's last submission has
  // happened (the copy stream's mark_fill_submitted): complete when both say done
  std::atomic<long> pending{0};
  std::atomic<bool> all_submitted{false};
  void job_done() {
    if (pending.fetch_sub(1) == 1 && all_submitted.load()) complete = true;
  }
  void mark_submitted() {
    all_submitted = true;
    if (pending.load() == 0) complete = true;
  }
  bool any = false;
  Clock::time_point first, last;
  double job_ms = 0.0;
  std::vector<int> cpus;
  void add(Clock::time_point t0, Clock::time_point t1, int cpu) {
    std::lock_guard<std::mutex> l(mu);
    if (!any || t0 < first) first = t0;
    if (!any || t1 > last) last = t1;
    any = true;
    job_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
    if (cpu >= 0 && std::find(cpus.begin(), cpus.end(), cpu) == cpus.end()) cpus.push_back(cpu);
  }
  double span_ms() {
    std::lock_guard<std::mutex> l(mu);
    return any ? std::chrono::duration<double, std::milli>(last - first).count() : 0.0;
  }
};

// rows -m for m in [m_lo, m_hi) of host chi [2 nw - 1][N_k][n_target] from rows
// m, split over the pool's threads
struct HostMirror {
  double2 *host;
  int nw, m_lo, m_hi, d0, d1, d2;
  long n_target;
  std::shared_ptr<FillStats> stats;
};

// The conjugate is the source with the sign bit of every imaginary part flipped:
// the block as 64-bit words, eight loads before the eight stores (a host
// measurement filled 6 to 12 % faster than element by element).
void host_mirror_range(const HostMirror &j, long b0, long b1) {
  const long nk = (long)j.d0 * j.d1 * j.d2;
  const long n = 2 * j.n_target;  // 64-bit words per block
  for (long b = b0; b < b1; ++b) {
    const int m = j.m_lo + (int)(b / nk);
    const long k = b - (long)(m - j.m_lo) * nk;
    const int k2 = (int)(k % j.d2), k1 = (int)((k / j.d2) % j.d1), k0 = (int)(k / ((long)j.d2 * j.d1));
    const long mk = ((long)((j.d0 - k0) % j.d0) * j.d1 + (j.d1 - k1) % j.d1) * j.d2 + (j.d2 - k2) % j.d2;
    const uint64_t *src = reinterpret_cast<const uint64_t *>(j.host + ((long)(j.nw - 1 + m) * nk + mk) * j.n_target);
    uint64_t *dst = reinterpret_cast<uint64_t *>(j.host + ((long)(j.nw - 1 - m) * nk + k) * j.n_target);
    long e = 0;
    for (; e + 8 <= n; e += 8) {
      uint64_t v[8];
      for (int u = 0; u < 8; ++u) v[u] = src[e + u];
      for (int u = 0; u < 8; ++u) dst[e + u] = v[u] ^ ((uint64_t)(u & 1) << 63);
    }
    for (; e < n; ++e) dst[e] = src[e] ^ ((uint64_t)(e & 1) << 63);
  }
}

void CUDART_CB submit_host_mirror(void *data) {
  const HostMirror *j = static_cast<const HostMirror *>(data);
  HostPool &pool = HostPool::get();
  const long blocks = (long)(j->m_hi - j->m_lo) * j->d0 * j->d1 * j->d2;
  const long parts = std::min<long>(blocks, pool.threads());
  j->stats->pending += parts;
  for (long i = 0; i < parts; ++i) {
    const long b0 = blocks * i / parts, b1 = blocks * (i + 1) / parts;
    const HostMirror copy = *j;
    pool.submit([copy, b0, b1] {
      const Clock::time_point t0 = Clock::now();
      host_mirror_range(copy, b0, b1);
      copy.stats->add(t0, Clock::now(), sched_getcpu());
      copy.stats->job_done();
    });
  }
  delete j;
}

// the copy stream's last host function of a call: every fill job of the call has
// been submitted (host functions of one stream run in order). It does not wait
// for them, so the next call's copies follow at once; join_fills waits.
void CUDART_CB mark_fill_submitted(void *data) {
  auto *sp = static_cast<std::shared_ptr<FillStats> *>(data);
  (*sp)->mark_submitted();
  delete sp;
}

// on the caller's stream, after it has waited for the copy stream: every fill
// job submitted so far has ended (the host's part of chi is in place)
void CUDART_CB join_fills(void *) { HostPool::get().wait_idle(); }

// One call's copies and host fill: timing events around every copy (grown on
// demand), the bytes that crossed the link and that the host filled, and the
// fill record.
constexpr int kRecords = 4;
struct CallRecord {
  std::vector<cudaEvent_t> copy_begin, copy_end;
  int copies = 0;
  size_t d2h = 0, filled = 0;
  std::shared_ptr<FillStats> fill;
  bool real = false, mirror = false, fold_pending = false;
  double frac = 1.0;
};

// One copy stream and its events per device, created on first use. copied[i]
// marks the last copy out of ring slot i (of this call or an earlier one: a
// call that does not wait for its copies leaves them running while the next
// call computes, and that call's solves wait for the slot they reuse).
struct CopyCtx {
  bool ready = false;
  cudaStream_t copy = nullptr;
  cudaEvent_t computed[kMaxSlots], copied[kMaxSlots], done;
  bool pending[kMaxSlots] = {};
  // the records of the last kRecords calls (a call that does not wait for its
  // copies is still in flight when the next ones start; its rates are folded
  // into the split by whichever later call finds it complete)
  CallRecord rec[kRecords];
  long calls = 0;  // calls enqueued so far; the last one's record is rec[(calls - 1) % kRecords]
  // Split of the negative frequencies of a real chi between the link and the host
  // threads: block k copies its rows -m over the link (both signs solved on the
  // device) when floor((k + 1) f + 1/2) > floor(k f + 1/2), so a fraction f of the
  // blocks does, spread evenly; the other blocks' rows -m are filled on the host.
  // Both draw on host memory bandwidth (a DMA write of a row against a read, a
  // write and a write-allocate read of the fill), so the best f balances the
  // link's busy time against the fill's. Adaptive mode measures both on each
  // completed call and moves f by a quarter of their relative imbalance (kept
  // in [0.1, 0.8], so both stay measured).
  // -1 adaptive, 0 every row over the link, 1 every row -m filled on the host,
  // 2 a fixed f (tprf_set_host_fill_fraction)
  int host_fill_mode = -1;
  double dma_frac = 0.4;    // current f of the adaptive mode
  double fixed_frac = 1.0;  // f of mode 2
  std::mutex mu;        // one call at a time enqueues on this device's copy stream
  CallRecord &last() { return rec[(calls + kRecords - 1) % kRecords]; }
};

// the i-th pair of timing events of a call's record (created on first use)
int copy_events(CallRecord *r, int i, cudaEvent_t *b, cudaEvent_t *e) {
  while ((int)r->copy_begin.size() <= i) {
    cudaEvent_t x, y;
    TPRF_CUDA(cudaEventCreate(&x));
    TPRF_CUDA(cudaEventCreate(&y));
    r->copy_begin.push_back(x);
    r->copy_end.push_back(y);
  }
  *b = r->copy_begin[i];
  *e = r->copy_end[i];
  return TPRF_OK;
}

// Adaptive split: fold a call's rates into dma_frac once its copies and fill
// have finished (checked without waiting). fold_split_rates folds every
// recorded call that has, oldest first; a record reused before its call was
// found complete is dropped.
void fold_record(CopyCtx *c, CallRecord *r) {
  if (!r->fold_pending || r->copies == 0 || !r->fill) return;
  if (cudaEventQuery(r->copy_end[r->copies - 1]) != cudaSuccess) {
    cudaGetLastError();  // a not-ready query is not an error of the next call
    return;
  }
  if (!r->fill->complete.load()) return;
  r->fold_pending = false;
  double copy_ms = 0.0;
  for (int i = 0; i < r->copies; ++i) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r->copy_begin[i], r->copy_end[i]) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    copy_ms += ms;
  }
  double fill_busy_ms;
  {
    std::lock_guard<std::mutex> l(r->fill->mu);
    fill_busy_ms = r->fill->job_ms / std::max(1, HostPool::get().threads());
  }
  if (copy_ms <= 0.0 || fill_busy_ms <= 0.0 || r->filled == 0) return;
  // move f by a quarter of the relative imbalance of the two busy times, as
  // measured with each other's contention for host memory (a balance point
  // computed from the rates would assume they do not depend on f)
  const double step = 0.25 * (fill_busy_ms - copy_ms) / (fill_busy_ms + copy_ms);
  c->dma_frac = std::min(0.8, std::max(0.1, c->dma_frac + step));
}
void fold_split_rates(CopyCtx *c) {
  for (long k = std::max(0L, c->calls - kRecords); k < c->calls; ++k) fold_record(c, &c->rec[k % kRecords]);
}
std::mutex g_copy_mu;
std::map<unsigned long long, CopyCtx> g_copy;  // per context (its streams and events die with it)

int copy_ctx(CopyCtx **out) {
  unsigned long long dev = 0;
  if (int st = current_context_key(&dev)) return st;
  std::lock_guard<std::mutex> lock(g_copy_mu);
  CopyCtx &c = g_copy[dev];
  if (!c.ready) {
    TPRF_CUDA(cudaStreamCreateWithFlags(&c.copy, cudaStreamNonBlocking));
    for (int i = 0; i < kMaxSlots; ++i) {
      TPRF_CUDA(cudaEventCreateWithFlags(&c.computed[i], cudaEventDisableTiming));
      TPRF_CUDA(cudaEventCreateWithFlags(&c.copied[i], cudaEventDisableTiming));
    }
    TPRF_CUDA(cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming));
    c.ready = true;
  }
  *out = &c;
  return TPRF_OK;
}

size_t slot_bytes(int block_freqs, long row) { return (2 * (size_t)block_freqs * row * sizeof(double2) + 255) & ~size_t(255); }

}  // namespace
}  // namespace tprf

using namespace tprf;

extern "C" size_t tprf_imtime_bubble_rpa_to_host_workspace_bytes(int n_iw, int n_tau, int nw, const int dims[3], int nb,
                                                                 int block_freqs, int slots) {
  if (!dims || nb < 1 || block_freqs < 1 || slots < 1) return 0;
  if (n_tau < 0) n_tau = default_n_tau(n_iw);
  const long row = (long)dims[0] * dims[1] * dims[2] * nb * nb * nb * nb;
  return tprf_imtime_bubble_workspace_bytes(n_iw, n_tau, dims, nb) + (size_t)slots * slot_bytes(block_freqs, row) + 256;
}

namespace {
// join: `stream` waits for the last copy (chi is on the host once the stream
// gets there); otherwise the copies run on past the call, behind its compute.
int bubble_rpa_to_host(double beta, int n_iw, int n_tau, int nw, const int dims[3], int nb, const double *g_wk,
                       const double *moments, const double *U, double *chi0_wk, double *chi_host, int block_freqs,
                       int slots, void *workspace, size_t workspace_bytes, void *stream, bool join) {
  if (!dims || !g_wk || !U || !chi0_wk || !chi_host || !workspace || nb < 1 || nb > 8 || nw < 1 || n_iw < 1 ||
      block_freqs < 1 || slots < 1 || slots > kMaxSlots)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "imtime_bubble_rpa_to_host: bad shape, slots or null pointer");
  if (n_tau < 0) n_tau = default_n_tau(n_iw);
  if (workspace_bytes < tprf_imtime_bubble_rpa_to_host_workspace_bytes(n_iw, n_tau, nw, dims, nb, block_freqs, slots))
    return set_error(TPRF_ERR_ALLOC, "imtime_bubble_rpa_to_host: workspace smaller than its workspace-bytes query");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long nk = (long)dims[0] * dims[1] * dims[2], nb4 = (long)nb * nb * nb * nb, row = nk * nb4;
  const size_t chain_bytes = tprf_imtime_bubble_workspace_bytes(n_iw, n_tau, dims, nb);
  double2 *chi0 = reinterpret_cast<double2 *>(chi0_wk);
  double2 *host = reinterpret_cast<double2 *>(chi_host);
  const double2 *Ud = reinterpret_cast<const double2 *>(U);
  bool chi_df = false;
  unsigned *gmax = nullptr;
  CompactChi cc;  // the canonical orbital columns of a transpose-symmetric real bubble, where they apply
  int st = bubble_to_wr(beta, n_iw, n_tau, nw, dims, nb, g_wk, moments, chi0, workspace, chain_bytes, nullptr, s,
                        &chi_df, &gmax, &cc);
  if (st) return st;
  // the plan depends on whether the bubble was real: read its two words (and
  // U: with U real as well the host fills the negative frequencies)
  bool real = false, u_real = false;
  if (chi_df && nw >= 2) {
    unsigned w[2];
    std::vector<double2> uh((size_t)nb * nb * nb * nb);
    TPRF_CUDA(cudaMemcpyAsync(w, gmax, sizeof(w), cudaMemcpyDeviceToHost, s));
    TPRF_CUDA(cudaMemcpyAsync(uh.data(), Ud, uh.size() * sizeof(double2), cudaMemcpyDeviceToHost, s));
    TPRF_CUDA(cudaStreamSynchronize(s));
    float a, b;
    memcpy(&a, &w[0], 4);
    memcpy(&b, &w[1], 4);
    real = real_input_ratio(a, b);
    u_real = std::all_of(uh.begin(), uh.end(), [](const double2 &v) { return v.y == 0.0; });
  }
  const bool host_mirror = real && u_real;
  size_t d2h = 0;
  const uintptr_t ring0 = (reinterpret_cast<uintptr_t>(workspace) + chain_bytes + 255) & ~uintptr_t(255);
  const size_t sb = slot_bytes(block_freqs, row);
  CopyCtx *c = nullptr;
  if ((st = copy_ctx(&c))) return st;
  std::lock_guard<std::mutex> lock(c->mu);
  fold_split_rates(c);
  const double frac = !host_mirror               ? 1.0
                      : c->host_fill_mode == 0 ? 1.0
                      : c->host_fill_mode == 1 ? 0.0
                      : c->host_fill_mode == 2 ? c->fixed_frac
                                               : c->dma_frac;
  size_t filled = 0;
  TPRF_CUDA(cudaEventRecord(c->done, s));  // the copy stream starts after the chain
  TPRF_CUDA(cudaStreamWaitEvent(c->copy, c->done, 0));
  const int n_w = 2 * nw - 1;
  const int n_blocks = real ? (nw + block_freqs - 1) / block_freqs : (n_w + block_freqs - 1) / block_freqs;
  auto fill = std::make_shared<FillStats>();
  int n_copies = 0;
  CallRecord *rec = &c->rec[c->calls % kRecords];
  rec->fold_pending = false;  // a record still unfolded here is dropped
  // one device-to-host copy on the copy stream, between this call's timing events
  auto d2h_copy = [&](double2 *dst, const double2 *src, size_t bytes) -> int {
    cudaEvent_t b, e;
    if (int r = copy_events(rec, n_copies++, &b, &e)) return r;
    TPRF_CUDA(cudaEventRecord(b, c->copy));
    TPRF_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->copy));
    TPRF_CUDA(cudaEventRecord(e, c->copy));
    d2h += bytes;
    return TPRF_OK;
  };
  for (int k = 0; k < n_blocks; ++k) {
    const int slot = k % slots;
    double2 *pos = reinterpret_cast<double2 *>(ring0 + (size_t)slot * sb);
    double2 *neg = pos + (long)block_freqs * row;
    if (c->pending[slot]) TPRF_CUDA(cudaStreamWaitEvent(s, c->copied[slot], 0));
    if (real) {
      const int m0 = k * block_freqs, m1 = std::min(nw, m0 + block_freqs), m_lo = std::max(m0, 1);
      double2 *rows = chi0 + (long)(nw - 1 + m0) * row;
      // the r -> q pass also stores chi0(-m, -q) = conj(chi0(m, q)) for m in
      // [max(m0, 1), m1): row j of the block (m = m0 + j) at row -2 m0 - j from
      // `rows`; from the block's compact rows when the bubble wrote them
      CompactChi cb;
      if (cc.gmax && chi_df) {
        cb = cc;
        cb.buf = static_cast<char *>(cc.buf) + (size_t)m0 * nk * cc.oc->nc * sizeof(double2);
        cb.rows = m1 - m0;
        cb.w0 = m0;
      }
      if ((st = launch_lattice_fft_fmt(false, m1 - m0, dims, nb4, rows, chi_df, rows, false, 1.0, s, nullptr, true,
                                       -2L * m0, cb.gmax ? &cb : nullptr)))
        return st;
      // frequency m at pos row m - m0; frequency -m (m >= m_lo) at neg row m1 - 1 - m
      const PairOut out{pos, neg + (long)(m1 - 1 - m0) * row, row, -row, m0, m1};
      if ((st = launch_rpa_wk_block(nw, dims, nb, chi0, Ud, out, s))) return st;
      TPRF_CUDA(cudaEventRecord(c->computed[slot], s));
      TPRF_CUDA(cudaStreamWaitEvent(c->copy, c->computed[slot], 0));
      if ((st = d2h_copy(host + (long)(nw - 1 + m0) * row, pos, (size_t)(m1 - m0) * row * sizeof(double2))))
        return st;
      const bool by_link = std::floor((k + 1) * frac + 0.5) > std::floor(k * frac + 0.5);
      if (m_lo < m1 && host_mirror && !by_link) {
        // the partners' rows -m read rows m at every q: all in this block
        filled += (size_t)(m1 - m_lo) * row * sizeof(double2);
        TPRF_CUDA(cudaLaunchHostFunc(
            c->copy, submit_host_mirror, new HostMirror{host, nw, m_lo, m1, dims[0], dims[1], dims[2], nb4, fill}));
      } else if (m_lo < m1) {
        if ((st = d2h_copy(host + (long)(nw - m1) * row, neg, (size_t)(m1 - m_lo) * row * sizeof(double2))))
          return st;
      }
    } else {
      const int r0 = k * block_freqs, r1 = std::min(n_w, r0 + block_freqs);
      double2 *rows = chi0 + (long)r0 * row;
      if ((st = launch_lattice_fft_fmt(false, r1 - r0, dims, nb4, rows, chi_df, rows, false, 1.0, s))) return st;
      if ((st = launch_rpa((long)(r1 - r0) * nk, nb, rows, Ud, pos, s))) return st;
      TPRF_CUDA(cudaEventRecord(c->computed[slot], s));
      TPRF_CUDA(cudaStreamWaitEvent(c->copy, c->computed[slot], 0));
      if ((st = d2h_copy(host + (long)r0 * row, pos, (size_t)(r1 - r0) * row * sizeof(double2)))) return st;
    }
    TPRF_CUDA(cudaEventRecord(c->copied[slot], c->copy));
    c->pending[slot] = true;
  }
  if (host_mirror)
    TPRF_CUDA(cudaLaunchHostFunc(c->copy, mark_fill_submitted, new std::shared_ptr<FillStats>(fill)));
  rec->d2h = d2h;
  rec->copies = n_copies;
  rec->fill = fill;
  rec->real = real;
  rec->mirror = host_mirror;
  rec->frac = frac;
  rec->filled = filled;
  rec->fold_pending = host_mirror && filled > 0;
  ++c->calls;
  TPRF_CUDA(cudaEventRecord(c->done, c->copy));
  if (join) {
    TPRF_CUDA(cudaStreamWaitEvent(s, c->done, 0));
    if (host_mirror) TPRF_CUDA(cudaLaunchHostFunc(s, join_fills, nullptr));
  }
  return finish_with_checks(s, "imtime_bubble_rpa_to_host");
}
}  // namespace

extern "C" int tprf_imtime_bubble_rpa_to_host(double beta, int n_iw, int n_tau, int nw, const int dims[3], int nb,
                                              const double *g_wk, const double *moments, const double *U,
                                              double *chi0_wk, double *chi_host, int block_freqs, int slots,
                                              void *workspace, size_t workspace_bytes, void *stream) {
  return bubble_rpa_to_host(beta, n_iw, n_tau, nw, dims, nb, g_wk, moments, U, chi0_wk, chi_host, block_freqs, slots,
                            workspace, workspace_bytes, stream, true);
}

extern "C" int tprf_imtime_bubble_rpa_to_host_async(double beta, int n_iw, int n_tau, int nw, const int dims[3],
                                                    int nb, const double *g_wk, const double *moments,
                                                    const double *U, double *chi0_wk, double *chi_host,
                                                    int block_freqs, int slots, void *workspace,
                                                    size_t workspace_bytes, void *stream) {
  return bubble_rpa_to_host(beta, n_iw, n_tau, nw, dims, nb, g_wk, moments, U, chi0_wk, chi_host, block_freqs, slots,
                            workspace, workspace_bytes, stream, false);
}

extern "C" size_t tprf_imtime_bubble_rpa_to_host_last_d2h_bytes(void) {
  CopyCtx *c = nullptr;
  if (copy_ctx(&c)) return 0;
  std::lock_guard<std::mutex> lock(c->mu);
  return c->calls > 0 ? c->last().d2h : 0;
}

extern "C" int tprf_imtime_bubble_rpa_to_host_last_stats(double *out, int n) {
  if (!out || n < 1) return set_error(TPRF_ERR_INVALID_ARGUMENT, "imtime_bubble_rpa_to_host_last_stats: no output");
  CopyCtx *c = nullptr;
  if (int st = copy_ctx(&c)) return st;
  std::lock_guard<std::mutex> lock(c->mu);
  double v[10] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, (double)HostPool::get().threads(), 0.0, 1.0};
  if (c->calls == 0) {
    for (int i = 0; i < n && i < 10; ++i) out[i] = v[i];
    return TPRF_OK;
  }
  CallRecord *r = &c->last();
  v[0] = (double)r->d2h;
  v[8] = r->real ? 1.0 : 0.0;
  v[9] = r->mirror ? r->frac : 1.0;
  if (r->copies > 0) {
    TPRF_CUDA(cudaEventSynchronize(r->copy_end[r->copies - 1]));
    float ms = 0.f;
    for (int i = 0; i < r->copies; ++i) {
      TPRF_CUDA(cudaEventElapsedTime(&ms, r->copy_begin[i], r->copy_end[i]));
      v[1] += ms;
    }
    TPRF_CUDA(cudaEventElapsedTime(&ms, r->copy_begin[0], r->copy_end[r->copies - 1]));
    v[2] = ms;
  }
  if (r->fill && r->mirror) {
    // the copy stream's last host function sets the flag after the fill jobs (the
    // copies above have finished, so it runs next); bounded wait
    const Clock::time_point t0 = Clock::now();
    while (!r->fill->complete.load()) {
      if (Clock::now() - t0 > std::chrono::seconds(60))
        return set_error(TPRF_ERR_CUDA, "imtime_bubble_rpa_to_host_last_stats: host fill did not finish in 60 s");
      std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
    v[3] = r->fill->span_ms();
    std::lock_guard<std::mutex> l(r->fill->mu);
    v[4] = r->fill->job_ms;
    v[5] = (double)r->fill->cpus.size();
  }
  v[6] = (double)r->copies;
  for (int i = 0; i < n && i < 10; ++i) out[i] = v[i];
  return TPRF_OK;
}

extern "C" int tprf_set_host_fill(int mode) {
  if (mode < -1 || mode > 1) return set_error(TPRF_ERR_INVALID_ARGUMENT, "set_host_fill: mode must be -1, 0 or 1");
  CopyCtx *c = nullptr;
  if (int st = copy_ctx(&c)) return st;
  std::lock_guard<std::mutex> lock(c->mu);
  c->host_fill_mode = mode;
  return TPRF_OK;
}

extern "C" int tprf_set_host_fill_fraction(double f) {
  if (!(f >= 0.0 && f <= 1.0))
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "set_host_fill_fraction: the fraction must lie in [0, 1]");
  CopyCtx *c = nullptr;
  if (int st = copy_ctx(&c)) return st;
  std::lock_guard<std::mutex> lock(c->mu);
  c->host_fill_mode = 2;
  c->fixed_frac = f;
  return TPRF_OK;
}

extern "C" int tprf_imtime_bubble_rpa_to_host_join(void *stream) {
  CopyCtx *c = nullptr;
  if (int st = copy_ctx(&c)) return st;
  std::lock_guard<std::mutex> lock(c->mu);
  TPRF_CUDA(cudaEventRecord(c->done, c->copy));
  TPRF_CUDA(cudaStreamWaitEvent(static_cast<cudaStream_t>(stream), c->done, 0));
  TPRF_CUDA(cudaLaunchHostFunc(static_cast<cudaStream_t>(stream), join_fills, nullptr));
  return TPRF_OK;
}
