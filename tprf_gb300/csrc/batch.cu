// Batched execution of many independent instances (different mu, beta, U,
// k meshes and frequency counts) of the whole path, Dyson -> k->r -> iv->tau
// -> bubble + tau->iw -> r->q -> RPA, in one launch.
//
// The reference computes one instance per call (its functions are called in
// a Python loop). Here tprf_batch_create plans every instance once (FFT and
// Matsubara tables, launch shapes), assigns the instances to K streams
// longest-first so the streams finish together, lays out one workspace per
// stream that its instances reuse in turn, and captures all of it into one
// CUDA graph; tprf_batch_run is then a single graph launch, so hundreds of
// small instances run concurrently without per-kernel host overhead.
#include <algorithm>
#include <cmath>
#include <memory>
#include <numeric>
#include <vector>

#include "common.cuh"

namespace tprf {
int launch_dyson(double beta, int n_iw, long n_k, int nb, double mu, const double2 *e_k, const double2 *sigma,
                 int sigma_kind, double2 *g, cudaStream_t stream);
int launch_lattice_fft(bool forward, long n_w, const int dims[3], long n_target, const double2 *in, double2 *out,
                       cudaStream_t stream);
int launch_nu_to_tau(double beta, int n_iw, int n_tau, long C, const double2 *gw, const double2 *mom, double2 *gt,
                     cudaStream_t stream);
int launch_chi0_wr_from_grt(double beta, int n_tau, int nw, const int dims[3], int nb, const double2 *g,
                            double2 *chi0_wr, cudaStream_t stream);
int launch_chi0_w0r_from_grt(double beta, int n_tau, const int dims[3], int nb, const double2 *g, double2 *chi0_wr,
                             cudaStream_t stream);
int launch_nu_to_tau_df(double beta, int n_iw, int n_tau, long C, const double2 *gw, const double2 *mom, double2 *gt,
                        void *gt_df, cudaStream_t stream);
int launch_chi0_wr_from_grt_df(double beta, int n_tau, int nw, const int dims[3], int nb, const double2 *g,
                               const void *g_df, double2 *chi0_wr, cudaStream_t stream);
int launch_rpa(long n_points, int nb, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream);
}  // namespace tprf

using namespace tprf;

struct tprf_batch {
  std::vector<tprf_instance> inst;
  std::vector<int> stream_of;        // instance -> stream slot
  std::vector<size_t> slot_offset;   // stream slot -> offset in the workspace
  int n_streams = 0;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

long inst_nk(const tprf_instance &a) { return (long)a.dims[0] * a.dims[1] * a.dims[2]; }
int inst_ntau(const tprf_instance &a) { return a.n_tau < 0 ? default_n_tau(a.n_iw) : a.n_tau; }

// Scratch of one instance: G(iv, k), G(iv, r), G(tau, r) and chi0(w, q).
size_t inst_scratch(const tprf_instance &a) {
  const size_t nk = inst_nk(a), nb2 = (size_t)a.nb * a.nb, nb4 = nb2 * nb2;
  const size_t g = 2ull * a.n_iw * nk * nb2, gt = (size_t)inst_ntau(a) * nk * nb2;
  const size_t c = (size_t)(2 * a.nw - 1) * nk * nb4;
  auto al = [](size_t n) { return (n * sizeof(double2) + 255) & ~size_t(255); };
  return 2 * al(g) + 2 * al(gt) + al(c);  // G(iv, k), G(iv, r), G(tau, r) and its double-float copy, chi0
}

// Relative cost used to balance the streams: FFT work plus the RPA solves.
double inst_cost(const tprf_instance &a) {
  const double nk = (double)inst_nk(a), nb2 = (double)a.nb * a.nb;
  const double L = inst_ntau(a) - 1;
  return nk * nb2 * nb2 * L * std::log2(std::max(2.0, L)) + (2.0 * a.nw - 1) * nk * nb2 * nb2 * nb2;
}

int check_instance(const tprf_instance &a, int i) {
  auto bad = [i](const char *what) {
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "batch instance " + std::to_string(i) + ": " + what);
  };
  if (!(a.beta > 0.0) || a.n_iw < 1 || a.nw < 1 || a.nb < 1 || a.nb > 5) return bad("bad mesh or nb (1..5)");
  for (int d = 0; d < 3; ++d)
    if (a.dims[d] < 1) return bad("mesh dims must be >= 1");
  if (!a.e_k || !a.U || !a.chi) return bad("null e_k, U or chi");
  const int nt = inst_ntau(a);
  if (nt - 1 < 2 * a.n_iw) return set_error(TPRF_ERR_MESH_TOO_SHORT, "batch: time mesh shorter than 2 n_iw");
  if (a.nw > 1 && nt - 1 < 2 * a.nw) return set_error(TPRF_ERR_MESH_TOO_SHORT, "batch: time mesh shorter than 2 nw");
  return TPRF_OK;
}

// The whole chain of one instance on one stream, into the slot's scratch.
int enqueue_instance(const tprf_instance &a, unsigned char *scratch, cudaStream_t s) {
  const long nk = inst_nk(a), nb2 = (long)a.nb * a.nb, nb4 = nb2 * nb2;
  const int nt = inst_ntau(a);
  auto al = [](size_t n) { return (n * sizeof(double2) + 255) & ~size_t(255); };
  const size_t g = 2ull * a.n_iw * nk * nb2, gt = (size_t)nt * nk * nb2;
  double2 *g_wk = reinterpret_cast<double2 *>(scratch);
  double2 *g_wr = reinterpret_cast<double2 *>(scratch + al(g));
  double2 *g_tr = reinterpret_cast<double2 *>(scratch + 2 * al(g));
  void *g_tr_df = scratch + 2 * al(g) + al(gt);
  double2 *chi0 = reinterpret_cast<double2 *>(scratch + 2 * al(g) + 2 * al(gt));
  int st = launch_dyson(a.beta, a.n_iw, nk, a.nb, a.mu, reinterpret_cast<const double2 *>(a.e_k), nullptr, 0, g_wk, s);
  if (st) return st;
  if ((st = launch_lattice_fft(true, 2L * a.n_iw, a.dims, nb2, g_wk, g_wr, s))) return st;
  if ((st = launch_nu_to_tau_df(a.beta, a.n_iw, nt, nk * nb2, g_wr, nullptr, g_tr, g_tr_df, s))) return st;
  if (a.nw == 1)
    st = launch_chi0_w0r_from_grt(a.beta, nt, a.dims, a.nb, g_tr, chi0, s);
  else
    st = launch_chi0_wr_from_grt_df(a.beta, nt, a.nw, a.dims, a.nb, g_tr, g_tr_df, chi0, s);
  if (st) return st;
  if ((st = launch_lattice_fft(false, 2L * a.nw - 1, a.dims, nb4, chi0, chi0, s))) return st;
  return launch_rpa((2L * a.nw - 1) * nk, a.nb, chi0, reinterpret_cast<const double2 *>(a.U),
                    reinterpret_cast<double2 *>(a.chi), s);
}

void destroy_parts(tprf_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto e : b->events) cudaEventDestroy(e);
  for (auto s : b->streams) cudaStreamDestroy(s);
}

}  // namespace

extern "C" size_t tprf_batch_workspace_bytes(const tprf_instance *inst, int n, int n_streams) {
  if (!inst || n < 1 || n_streams < 1) return 0;
  // same greedy assignment as tprf_batch_create: every stream slot holds the
  // largest scratch among its instances
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return inst_cost(inst[x]) > inst_cost(inst[y]); });
  const int K = std::min(n_streams, n);
  std::vector<double> load(K, 0.0);
  std::vector<size_t> slot(K, 0);
  for (int i : order) {
    const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    load[k] += inst_cost(inst[i]);
    slot[k] = std::max(slot[k], inst_scratch(inst[i]));
  }
  size_t total = 256;
  for (size_t x : slot) total += (x + 255) & ~size_t(255);
  return total;
}

extern "C" int tprf_batch_create(const tprf_instance *inst, int n, int n_streams, void *workspace,
                                 size_t workspace_bytes, tprf_batch **out) {
  if (!inst || n < 1 || n_streams < 1 || !workspace || !out)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "batch_create: bad arguments");
  for (int i = 0; i < n; ++i) {
    int st = check_instance(inst[i], i);
    if (st) return st;
  }
  if (workspace_bytes < tprf_batch_workspace_bytes(inst, n, n_streams))
    return set_error(TPRF_ERR_ALLOC, "batch_create: workspace smaller than tprf_batch_workspace_bytes");
  auto b = std::make_unique<tprf_batch>();
  b->inst.assign(inst, inst + n);
  // longest-processing-time assignment to streams
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return inst_cost(inst[x]) > inst_cost(inst[y]); });
  const int K = std::min(n_streams, n);
  b->n_streams = K;
  b->stream_of.assign(n, 0);
  std::vector<double> load(K, 0.0);
  std::vector<size_t> slot(K, 0);
  std::vector<std::vector<int>> per(K);
  for (int i : order) {
    const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    load[k] += inst_cost(inst[i]);
    slot[k] = std::max(slot[k], inst_scratch(inst[i]));
    b->stream_of[i] = k;
    per[k].push_back(i);
  }
  const uintptr_t base = (reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255);
  size_t off = 0;
  b->slot_offset.assign(K, 0);
  for (int k = 0; k < K; ++k) {
    b->slot_offset[k] = off;
    off += (slot[k] + 255) & ~size_t(255);
  }
  // Plans and the device error word are built before capture (they upload
  // tables synchronously): run every instance once, eagerly, on one stream.
  cudaStream_t s0 = nullptr;
  TPRF_CUDA(cudaStreamCreateWithFlags(&s0, cudaStreamNonBlocking));
  b->streams.push_back(s0);
  if (!device_status_word()) {
    destroy_parts(b.get());
    return TPRF_ERR_CUDA;
  }
  for (int i = 0; i < n; ++i) {
    int st = enqueue_instance(b->inst[i], reinterpret_cast<unsigned char *>(base + b->slot_offset[b->stream_of[i]]), s0);
    if (st) {
      destroy_parts(b.get());
      return st;
    }
  }
  cudaError_t e = cudaStreamSynchronize(s0);
  if (e != cudaSuccess) {
    destroy_parts(b.get());
    return cuda_status(e, "batch_create: first run");
  }
  // capture: fork K streams from s0, one chain of instances each, join
  for (int k = 1; k < K; ++k) {
    cudaStream_t s;
    TPRF_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    b->streams.push_back(s);
  }
  b->events.resize(K + 1);
  for (auto &ev : b->events) TPRF_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  TPRF_CUDA(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
  int st = TPRF_OK;
  cudaEventRecord(b->events[K], s0);
  for (int k = 1; k < K; ++k) cudaStreamWaitEvent(b->streams[k], b->events[K], 0);
  for (int k = 0; k < K && st == TPRF_OK; ++k)
    for (int i : per[k]) {
      st = enqueue_instance(b->inst[i], reinterpret_cast<unsigned char *>(base + b->slot_offset[k]), b->streams[k]);
      if (st) break;
    }
  for (int k = 1; k < K; ++k) {
    cudaEventRecord(b->events[k], b->streams[k]);
    cudaStreamWaitEvent(s0, b->events[k], 0);
  }
  e = cudaStreamEndCapture(s0, &b->graph);
  if (st == TPRF_OK && e != cudaSuccess) st = cuda_status(e, "batch_create: capture");
  if (st == TPRF_OK) {
    e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e != cudaSuccess) st = cuda_status(e, "batch_create: graph instantiate");
  }
  if (st) {
    destroy_parts(b.get());
    return st;
  }
  *out = b.release();
  return TPRF_OK;
}

extern "C" int tprf_batch_run(tprf_batch *b, void *stream) {
  if (!b || !b->exec) return set_error(TPRF_ERR_INVALID_ARGUMENT, "batch_run: not a batch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  TPRF_CUDA(cudaGraphLaunch(b->exec, s));
  return finish_with_checks(s, "batch_run");
}

extern "C" int tprf_batch_size(const tprf_batch *b) { return b ? (int)b->inst.size() : 0; }

extern "C" int tprf_batch_destroy(tprf_batch *b) {
  if (!b) return TPRF_OK;
  destroy_parts(b);
  delete b;
  return TPRF_OK;
}
