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
// tprf_batch_grad_create adds a second graph with every instance's adjoint
// chain (gradients with respect to U, e(k) and the hoppings t(R)).
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
int launch_rpa(long n_points, int nb, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream);
}  // namespace tprf

using namespace tprf;

struct tprf_batch {
  std::vector<tprf_instance> inst;
  std::vector<tprf_grad_instance> grad;  // empty unless made by tprf_batch_grad_create
  std::vector<int> stream_of;            // instance -> stream slot
  std::vector<size_t> slot_offset;       // stream slot -> offset in the workspace
  int n_streams = 0;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;
  cudaGraph_t graph = nullptr, graph_bwd = nullptr;
  cudaGraphExec_t exec = nullptr, exec_bwd = nullptr;
  unsigned long long kernels = 0, kernels_bwd = 0;  // kernel launches captured into each graph
};

namespace {

long inst_nk(const tprf_instance &a) { return (long)a.dims[0] * a.dims[1] * a.dims[2]; }
int inst_ntau(const tprf_instance &a) { return a.n_tau < 0 ? default_n_tau(a.n_iw) : a.n_tau; }
size_t al16(size_t n) { return (n * sizeof(double2) + 255) & ~size_t(255); }

// Scratch layout of one instance (element counts; every part 256-byte aligned):
//   256 B | G(iv, k) | G(iv, r) | G(tau, r) | double-float G(tau, r) | chi0(w, q) | chi0(tau, r) gradient
// The forward pass uses the first five (chi0 only when the caller does not keep
// it); the backward pass reuses them for the gradients of the same shapes.
struct Layout {
  size_t g, gt, c;
  Layout(const tprf_instance &a) {
    const size_t nk = inst_nk(a), nb2 = (size_t)a.nb * a.nb, nb4 = nb2 * nb2;
    g = 2ull * a.n_iw * nk * nb2;
    gt = (size_t)inst_ntau(a) * nk * nb2;
    c = (size_t)(2 * a.nw - 1) * nk * nb4;
  }
  // 256 bytes first: the max |G|, max |Im G| words of the real-pair test
  static constexpr size_t kHdr = 256;
  size_t off_gwk() const { return kHdr; }
  size_t off_gwr() const { return kHdr + al16(g); }
  size_t off_gtr() const { return kHdr + 2 * al16(g); }
  size_t off_gdf() const { return kHdr + 2 * al16(g) + al16(gt); }
  size_t off_c() const { return kHdr + 2 * al16(g) + 2 * al16(gt); }
  size_t off_gk() const { return off_c() + al16(c); }  // backward: G_grad(iv, k)
  size_t forward_bytes() const { return off_c() + al16(c); }
  size_t grad_bytes() const { return off_gk() + al16(g); }
};

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

int check_grad_instance(const tprf_grad_instance &g, int i) {
  int st = check_instance(g.inst, i);
  if (st) return st;
  if (!g.chi0 || !g.chi_grad || !g.U_grad)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "batch instance " + std::to_string(i) + ": null chi0, chi_grad or U_grad");
  if (g.inst.nw < 2)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "batch instance " + std::to_string(i) + ": the gradient needs nw >= 2");
  return TPRF_OK;
}

// Longest-processing-time assignment of the instances to K stream slots; each
// slot is sized for the largest scratch among its instances.
struct Assignment {
  std::vector<int> stream_of;
  std::vector<std::vector<int>> per;
  std::vector<size_t> slot;
};
Assignment assign(const tprf_instance *inst, int n, int n_streams, bool grad) {
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return inst_cost(inst[x]) > inst_cost(inst[y]); });
  const int K = std::min(n_streams, n);
  Assignment A;
  A.stream_of.assign(n, 0);
  A.per.assign(K, {});
  A.slot.assign(K, 0);
  std::vector<double> load(K, 0.0);
  for (int i : order) {
    const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    load[k] += inst_cost(inst[i]) * (grad ? 3.0 : 1.0);
    const Layout L(inst[i]);
    A.slot[k] = std::max(A.slot[k], grad ? L.grad_bytes() : L.forward_bytes());
    A.stream_of[i] = k;
    A.per[k].push_back(i);
  }
  return A;
}

size_t workspace_total(const Assignment &A) {
  size_t total = 256;
  for (size_t x : A.slot) total += (x + 255) & ~size_t(255);
  return total;
}

// The whole chain of one instance on one stream, into the slot's scratch;
// chi0 goes to chi0_out when given (kept for the backward pass).
int enqueue_instance(const tprf_instance &a, unsigned char *scratch, cudaStream_t s, double2 *chi0_out = nullptr) {
  const long nk = inst_nk(a), nb2 = (long)a.nb * a.nb, nb4 = nb2 * nb2;
  const int nt = inst_ntau(a);
  const Layout L(a);
  unsigned *gmax = reinterpret_cast<unsigned *>(scratch);
  double2 *g_wk = reinterpret_cast<double2 *>(scratch + L.off_gwk());
  double2 *g_wr = reinterpret_cast<double2 *>(scratch + L.off_gwr());
  double2 *g_tr = reinterpret_cast<double2 *>(scratch + L.off_gtr());
  void *g_tr_df = scratch + L.off_gdf();
  double2 *chi0 = chi0_out ? chi0_out : reinterpret_cast<double2 *>(scratch + L.off_c());
  int st = launch_dyson(a.beta, a.n_iw, nk, a.nb, a.mu, reinterpret_cast<const double2 *>(a.e_k), nullptr, 0, g_wk, s);
  if (st) return st;
  if ((st = launch_lattice_fft(true, 2L * a.n_iw, a.dims, nb2, g_wk, g_wr, s))) return st;
  // real-input, Hermitian and transposition tests
  TPRF_CUDA(cudaMemsetAsync(gmax, 0, 8 * sizeof(unsigned), s));
  if ((st = launch_hermitian_check(a.n_iw, nk * nb2, g_wr, gmax + 2, s, a.dims, a.nb))) return st;
  const TransposePairs *tp2 = nullptr;
  if ((st = get_transpose_pairs(a.dims, a.nb, 2, &tp2))) return st;
  if ((st = launch_nu_to_tau_df(a.beta, a.n_iw, nt, nk * nb2, g_wr, nullptr, g_tr, g_tr_df, s, gmax, gmax + 2,
                                a.nw > 1, tp2)))
    return st;
  bool chi_df = false;  // chi0(w, r) handed to r -> q as double-float pairs (as the single-instance chain)
  if (a.nw == 1)
    st = launch_chi0_w0r_from_grt(a.beta, nt, a.dims, a.nb, g_tr, chi0, s);
  else
    st = launch_chi0_wr_from_grt_df(a.beta, nt, a.nw, a.dims, a.nb, g_tr, g_tr_df, chi0, s, nk > 1, &chi_df, gmax,
                                    nk > 1);
  if (st) return st;
  if ((st = launch_lattice_fft_fmt(false, 2L * a.nw - 1, a.dims, nb4, chi0, chi_df, chi0, false, 1.0, s,
                                   chi_df ? gmax : nullptr)))
    return st;
  return launch_rpa_wk(a.nw, a.dims, a.nb, chi0, reinterpret_cast<const double2 *>(a.U),
                       reinterpret_cast<double2 *>(a.chi), s);
}

// The adjoint chain of one instance (the transposes of enqueue_instance's
// stages in reverse order, G recomputed). The r->q transform is unscaled
// FFTW_BACKWARD, so its transpose is the unscaled forward transform; k->r is
// (1/N_k) FFTW_FORWARD, whose transpose is (1/N_k) FFTW_BACKWARD.
int enqueue_backward(const tprf_grad_instance &gi, unsigned char *scratch, cudaStream_t s, unsigned *status) {
  const tprf_instance &a = gi.inst;
  const long nk = inst_nk(a), nb2 = (long)a.nb * a.nb, nb4 = nb2 * nb2;
  const int nt = inst_ntau(a), nwt = 2 * a.nw - 1;
  const Layout L(a);
  auto at = [&](size_t off) { return reinterpret_cast<double2 *>(scratch + off); };
  double2 *g_wk = at(L.off_gwk()), *g_wr = at(L.off_gwr()), *g_tr = at(L.off_gtr());
  double2 *g_tr_grad = at(L.off_gdf());  // the double-float slot is not needed here
  double2 *chi0_grad = at(L.off_c());
  double2 *g_wr_grad = g_wr;  // G(iv, r) is dead once G(tau, r) is recomputed
  double2 *g_wk_grad = at(L.off_gk());
  double2 *e_grad = gi.e_grad ? reinterpret_cast<double2 *>(gi.e_grad) : chi0_grad;
  double2 *U_grad = reinterpret_cast<double2 *>(gi.U_grad);
  auto cd = [](const double *p) { return reinterpret_cast<const double2 *>(p); };
  TPRF_CUDA(cudaMemsetAsync(U_grad, 0, nb4 * sizeof(double2), s));
  int st = launch_rpa_adjoint((long)nwt * nk, a.nb, cd(gi.chi0), cd(a.U), cd(a.chi), cd(gi.chi_grad), chi0_grad,
                                   U_grad, s, status);
  if (st) return st;
  if ((st = launch_lattice_fft_scaled(true, nwt, a.dims, nb4, chi0_grad, chi0_grad, 1.0, s))) return st;
  if ((st = launch_dyson(a.beta, a.n_iw, nk, a.nb, a.mu, cd(a.e_k), nullptr, 0, g_wk, s))) return st;
  if ((st = launch_lattice_fft(true, 2L * a.n_iw, a.dims, nb2, g_wk, g_wr, s))) return st;
  if ((st = launch_nu_to_tau(a.beta, a.n_iw, nt, nk * nb2, g_wr, nullptr, g_tr, s))) return st;
  // tau -> iw and the bubble transposed together: chi0_grad(tau, r) is never stored
  if ((st = launch_chi0_wr_from_grt_adjoint(a.beta, nt, a.nw, a.dims, a.nb, g_tr, chi0_grad, g_tr_grad, s))) return st;
  if ((st = launch_nu_to_tau_adjoint(a.beta, a.n_iw, nt, nk * nb2, g_tr_grad, g_wr_grad, true, s))) return st;
  if ((st = launch_lattice_fft_scaled(false, 2L * a.n_iw, a.dims, nb2, g_wr_grad, g_wk_grad, 1.0 / (double)nk, s)))
    return st;
  if ((st = launch_dyson_adjoint(a.n_iw, nk, a.nb, g_wk, g_wk_grad, e_grad, s))) return st;
  if (gi.t_grad)
    st = launch_lattice_fft_scaled(true, 1, a.dims, nb2, e_grad, reinterpret_cast<double2 *>(gi.t_grad), 1.0, s);
  return st;
}

void destroy_parts(tprf_batch *b) {
  if (b->exec_bwd) cudaGraphExecDestroy(b->exec_bwd);
  if (b->graph_bwd) cudaGraphDestroy(b->graph_bwd);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto e : b->events) cudaEventDestroy(e);
  for (auto s : b->streams) cudaStreamDestroy(s);
}

// Captures `body(i, scratch, stream)` for every instance, each on its slot's
// stream, forked from and joined into streams[0], into one graph.
template <class Body>
int capture(tprf_batch *b, const std::vector<std::vector<int>> &per, uintptr_t base, Body body, cudaGraph_t *graph,
            cudaGraphExec_t *exec, unsigned long long *kernels) {
  const int K = b->n_streams;
  cudaStream_t s0 = b->streams[0];
  TPRF_CUDA(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
  begin_capture_tally();
  int st = TPRF_OK;
  cudaEventRecord(b->events[K], s0);
  for (int k = 1; k < K; ++k) cudaStreamWaitEvent(b->streams[k], b->events[K], 0);
  for (int k = 0; k < K && st == TPRF_OK; ++k)
    for (int i : per[k]) {
      st = body(i, reinterpret_cast<unsigned char *>(base + b->slot_offset[k]), b->streams[k]);
      if (st) break;
    }
  for (int k = 1; k < K; ++k) {
    cudaEventRecord(b->events[k], b->streams[k]);
    cudaStreamWaitEvent(s0, b->events[k], 0);
  }
  cudaError_t e = cudaStreamEndCapture(s0, graph);
  *kernels = end_capture_tally();
  if (st == TPRF_OK && e != cudaSuccess) st = cuda_status(e, "batch_create: capture");
  if (st == TPRF_OK) {
    e = cudaGraphInstantiate(exec, *graph, 0);
    if (e != cudaSuccess) st = cuda_status(e, "batch_create: graph instantiate");
  }
  return st;
}

// Shared by tprf_batch_create and tprf_batch_grad_create (grad != nullptr).
int create_batch(const tprf_instance *inst, const tprf_grad_instance *grad, int n, int n_streams, void *workspace,
                 size_t workspace_bytes, tprf_batch **out) {
  const Assignment A = assign(inst, n, n_streams, grad != nullptr);
  if (workspace_bytes < workspace_total(A))
    return set_error(TPRF_ERR_ALLOC, "batch_create: workspace smaller than the workspace-bytes query");
  auto b = std::make_unique<tprf_batch>();
  b->inst.assign(inst, inst + n);
  if (grad) b->grad.assign(grad, grad + n);
  const int K = (int)A.per.size();
  b->n_streams = K;
  b->stream_of = A.stream_of;
  const uintptr_t base = (reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255);
  size_t off = 0;
  b->slot_offset.assign(K, 0);
  for (int k = 0; k < K; ++k) {
    b->slot_offset[k] = off;
    off += (A.slot[k] + 255) & ~size_t(255);
  }
  auto fail = [&](int st) {
    destroy_parts(b.get());
    return st;
  };
  for (int k = 0; k < K; ++k) {
    cudaStream_t s;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(cuda_status(e, "batch_create: stream"));
    b->streams.push_back(s);
  }
  b->events.resize(K + 1, nullptr);
  for (auto &ev : b->events) {
    cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return fail(cuda_status(e, "batch_create: event"));
  }
  unsigned *status = device_status_word();
  if (!status) return fail(TPRF_ERR_CUDA);
  auto fwd = [&](int i, unsigned char *scratch, cudaStream_t s) {
    return enqueue_instance(b->inst[i], scratch, s, grad ? reinterpret_cast<double2 *>(b->grad[i].chi0) : nullptr);
  };
  auto bwd = [&](int i, unsigned char *scratch, cudaStream_t s) {
    return enqueue_backward(b->grad[i], scratch, s, status);
  };
  // Plans upload their tables synchronously, so every instance runs once,
  // eagerly, on one stream before the capture (the backward pass reads whatever
  // chi_grad holds; its outputs are overwritten by every later run).
  cudaStream_t s0 = b->streams[0];
  for (int i = 0; i < n; ++i) {
    unsigned char *scratch = reinterpret_cast<unsigned char *>(base + b->slot_offset[A.stream_of[i]]);
    int st = fwd(i, scratch, s0);
    if (!st && grad) st = bwd(i, scratch, s0);
    if (st) return fail(st);
  }
  cudaError_t e = cudaStreamSynchronize(s0);
  if (e != cudaSuccess) return fail(cuda_status(e, "batch_create: first run"));
  int st = capture(b.get(), A.per, base, fwd, &b->graph, &b->exec, &b->kernels);
  if (!st && grad) st = capture(b.get(), A.per, base, bwd, &b->graph_bwd, &b->exec_bwd, &b->kernels_bwd);
  if (st) return fail(st);
  *out = b.release();
  return TPRF_OK;
}

}  // namespace

extern "C" size_t tprf_batch_workspace_bytes(const tprf_instance *inst, int n, int n_streams) {
  if (!inst || n < 1 || n_streams < 1) return 0;
  return workspace_total(assign(inst, n, n_streams, false));
}

extern "C" size_t tprf_batch_grad_workspace_bytes(const tprf_grad_instance *inst, int n, int n_streams) {
  if (!inst || n < 1 || n_streams < 1) return 0;
  std::vector<tprf_instance> base(n);
  for (int i = 0; i < n; ++i) base[i] = inst[i].inst;
  return workspace_total(assign(base.data(), n, n_streams, true));
}

extern "C" int tprf_batch_create(const tprf_instance *inst, int n, int n_streams, void *workspace,
                                 size_t workspace_bytes, tprf_batch **out) {
  if (!inst || n < 1 || n_streams < 1 || !workspace || !out)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "batch_create: bad arguments");
  for (int i = 0; i < n; ++i) {
    int st = check_instance(inst[i], i);
    if (st) return st;
  }
  return create_batch(inst, nullptr, n, n_streams, workspace, workspace_bytes, out);
}

extern "C" int tprf_batch_grad_create(const tprf_grad_instance *inst, int n, int n_streams, void *workspace,
                                      size_t workspace_bytes, tprf_batch **out) {
  if (!inst || n < 1 || n_streams < 1 || !workspace || !out)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "batch_grad_create: bad arguments");
  std::vector<tprf_instance> base(n);
  for (int i = 0; i < n; ++i) {
    int st = check_grad_instance(inst[i], i);
    if (st) return st;
    base[i] = inst[i].inst;
  }
  return create_batch(base.data(), inst, n, n_streams, workspace, workspace_bytes, out);
}

extern "C" int tprf_batch_backward(tprf_batch *b, void *stream) {
  if (!b || !b->exec_bwd) return set_error(TPRF_ERR_INVALID_ARGUMENT, "batch_backward: not a gradient batch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  TPRF_CUDA(cudaGraphLaunch(b->exec_bwd, s));
  count_graph_launch(b->kernels_bwd);
  return finish_with_checks(s, "batch_backward");
}

extern "C" int tprf_batch_run(tprf_batch *b, void *stream) {
  if (!b || !b->exec) return set_error(TPRF_ERR_INVALID_ARGUMENT, "batch_run: not a batch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  TPRF_CUDA(cudaGraphLaunch(b->exec, s));
  count_graph_launch(b->kernels);
  return finish_with_checks(s, "batch_run");
}

extern "C" int tprf_batch_size(const tprf_batch *b) { return b ? (int)b->inst.size() : 0; }

extern "C" int tprf_batch_destroy(tprf_batch *b) {
  if (!b) return TPRF_OK;
  destroy_parts(b);
  delete b;
  return TPRF_OK;
}
