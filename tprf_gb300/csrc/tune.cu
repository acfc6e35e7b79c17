// Autotuner of launch shapes, kept as "wisdom" (a table from a shape key to the
// chosen value), after FFTW's planner: the reference plans its FFTs with
// FFTW_ESTIMATE (c++/triqs_tprf/fourier/fourier_common.cpp:32-43), a fixed
// heuristic; here the default is likewise a fixed heuristic, and measure mode
// (tprf_set_autotune(1)) times every candidate shape on the first call of each
// shape key and keeps the fastest for the rest of the process.
//
// What is tuned: the columns per CTA of the Matsubara FFT kernels (iv -> tau,
// the fused bubble + tau -> iw, tau -> iw) and the lanes per point and warps
// per CTA of the RPA group kernel. Every candidate runs on the call's own
// buffers, restricted to a prefix of its columns or points: these kernels are
// out of place and deterministic, so the prefix is recomputed with the same
// values and the call's result does not depend on the tuning. Tuning waits for
// the calling stream (a planning cost paid once per shape) and is skipped while
// the stream is being captured into a graph; the batched path plans with an
// eager run before its capture, so its graphs use tuned shapes.
#include <algorithm>
#include <atomic>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>

#include "internal.hpp"

namespace tprf {
namespace {

std::mutex g_tune_mu;
std::map<std::string, int> g_wisdom;
std::atomic<int> g_tune_mode{0};

// Milliseconds per launch of one candidate: one untimed launch, then the
// shortest of three timed launches (the minimum ranks candidates a few percent
// apart more reliably than a mean of short launches).
int time_candidate(const std::function<int(int)> &launch, int value, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1,
                   float *ms) {
  int st = launch(value);
  if (st) return st;
  *ms = 3.0e38f;
  for (int rep = 0; rep < 3; ++rep) {
    TPRF_CUDA(cudaEventRecord(e0, s));
    if ((st = launch(value))) return st;
    TPRF_CUDA(cudaEventRecord(e1, s));
    TPRF_CUDA(cudaEventSynchronize(e1));
    float t = 0.f;
    TPRF_CUDA(cudaEventElapsedTime(&t, e0, e1));
    *ms = std::min(*ms, t);
  }
  return TPRF_OK;
}

}  // namespace

int tune_mode() { return g_tune_mode.load(); }

std::string tune_key(const char *kernel, std::initializer_list<long> shape) {
  int dev = 0, sms = 0, major = 0, minor = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  std::ostringstream k;
  k << "sm" << major << minor << "x" << sms << "/" << kernel << "/" << arith_mode();
  for (long v : shape) k << "/" << v;
  return k.str();
}

int tune_lookup(const std::string &key, const std::vector<int> &candidates, int fallback, int *choice) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_wisdom.find(key);
  const bool hit =
      it != g_wisdom.end() && std::find(candidates.begin(), candidates.end(), it->second) != candidates.end();
  *choice = hit ? it->second : fallback;
  return TPRF_OK;
}

int tune_pick(const std::string &key, const std::vector<int> &candidates, int fallback, cudaStream_t s,
              const std::function<int(int)> &launch, int *choice) {
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_wisdom.find(key);
    if (it != g_wisdom.end() && std::find(candidates.begin(), candidates.end(), it->second) != candidates.end()) {
      *choice = it->second;
      return TPRF_OK;
    }
  }
  *choice = fallback;
  if (g_tune_mode.load() == 0 || candidates.size() < 2) return TPRF_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  TPRF_CUDA(cudaStreamIsCapturing(s, &cs));
  if (cs != cudaStreamCaptureStatusNone) return TPRF_OK;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  TPRF_CUDA(cudaEventCreate(&e0));
  cudaError_t ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) {
    cudaEventDestroy(e0);
    return cuda_status(ce, "autotune: event");
  }
  float best = 3.0e38f, fallback_ms = 3.0e38f;
  int best_v = fallback, st = TPRF_OK;
  for (int v : candidates) {
    float ms = 0.f;
    st = time_candidate(launch, v, s, e0, e1, &ms);
    if (st) break;
    if (v == fallback) fallback_ms = ms;
    if (ms < best) {
      best = ms;
      best_v = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  // the heuristic's choice stands unless another candidate is more than 2 %
  // faster: closer than that, the trials' noise decides
  if (fallback_ms <= 1.02f * best) best_v = fallback;
  *choice = best_v;
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_wisdom[key] = best_v;
  return TPRF_OK;
}

}  // namespace tprf

extern "C" int tprf_set_autotune(int mode) {
  if (mode != 0 && mode != 1) return tprf::set_error(TPRF_ERR_INVALID_ARGUMENT, "set_autotune: mode must be 0 or 1");
  tprf::g_tune_mode.store(mode);
  return TPRF_OK;
}

extern "C" int tprf_get_autotune(void) { return tprf::g_tune_mode.load(); }

extern "C" int tprf_autotune_entries(void) {
  std::lock_guard<std::mutex> lock(tprf::g_tune_mu);
  return (int)tprf::g_wisdom.size();
}

extern "C" void tprf_autotune_clear(void) {
  std::lock_guard<std::mutex> lock(tprf::g_tune_mu);
  tprf::g_wisdom.clear();
}

// One "key value" pair per line; keys hold no whitespace.
extern "C" int tprf_autotune_save(const char *path) {
  if (!path) return tprf::set_error(TPRF_ERR_INVALID_ARGUMENT, "autotune_save: null path");
  std::ofstream f(path);
  if (!f) return tprf::set_error(TPRF_ERR_INVALID_ARGUMENT, std::string("autotune_save: cannot write ") + path);
  std::lock_guard<std::mutex> lock(tprf::g_tune_mu);
  f << "# tprf_gb300 autotune wisdom v1\n";
  for (const auto &kv : tprf::g_wisdom) f << kv.first << " " << kv.second << "\n";
  return f.good() ? TPRF_OK : tprf::set_error(TPRF_ERR_INVALID_ARGUMENT, "autotune_save: write failed");
}

extern "C" int tprf_autotune_load(const char *path) {
  if (!path) return tprf::set_error(TPRF_ERR_INVALID_ARGUMENT, "autotune_load: null path");
  std::ifstream f(path);
  if (!f) return tprf::set_error(TPRF_ERR_INVALID_ARGUMENT, std::string("autotune_load: cannot read ") + path);
  std::map<std::string, int> read;
  std::string line;
  int n = 0;
  while (std::getline(f, line)) {
    ++n;
    if (line.empty() || line[0] == '#') continue;
    std::istringstream ls(line);
    std::string key, extra;
    long v = 0;
    if (!(ls >> key >> v) || (ls >> extra) || v < 0 || v > (1 << 20))
      return tprf::set_error(TPRF_ERR_INVALID_ARGUMENT,
                             "autotune_load: malformed line " + std::to_string(n) + " of " + path);
    read[key] = (int)v;
  }
  std::lock_guard<std::mutex> lock(tprf::g_tune_mu);
  for (const auto &kv : read) tprf::g_wisdom[kv.first] = kv.second;
  return TPRF_OK;
}
