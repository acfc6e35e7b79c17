// C++ host layer with TPRF's signatures (include/triqs_tprf_gb300/triqs_tprf.hpp)
// over the C ABI (include/tprf_gb300.h). Every function checks its arguments on
// the host (the checks the reference makes with TRIQS_RUNTIME_ERROR, plus the
// mesh and target-shape contracts its types enforce), copies the inputs to
// device memory, calls one C-ABI entry point on the legacy default stream (the
// entry points synchronise and report data-dependent errors with their default
// synchronous checks) and copies the output back into a new gf.
#include "triqs_tprf_gb300/triqs_tprf.hpp"

#include <cuda_runtime_api.h>

#include <cmath>
#include <cstring>
#include <sstream>

#include "tprf_gb300.h"

namespace triqs_tprf {

dcomplex mesh::imfreq::index_to_value(long n) const {
  const double s = statistic_ == Fermion ? 1.0 : 0.0;
  return dcomplex(0.0, M_PI * (2.0 * (double)n + s) / beta_);
}

std::array<double, 3> mesh::brzone::index_to_value(long linear) const {
  const std::array<long, 3> i = index(linear);
  std::array<double, 3> k{};
  for (int d = 0; d < 3; ++d) k[d] = 2.0 * M_PI * (double)i[d] / (double)dims()[d];
  return k;
}

namespace {

[[noreturn]] void fail(const char *what, const std::string &why) { throw runtime_error(std::string(what) + ": " + why); }

void check(int status, const char *what) {
  if (status == TPRF_OK) return;
  const char *msg = tprf_last_error();
  fail(what, (msg && *msg) ? msg : tprf_status_string(status));
}

void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) fail(what, std::string("CUDA: ") + cudaGetErrorString(e));
}

// Device copy of a block of complex128 values, freed on scope exit.
class device_block {
 public:
  device_block(long elements, const char *what) : bytes_((size_t)std::max(elements, 1L) * sizeof(dcomplex)) {
    cuda_check(cudaMalloc(&ptr_, bytes_), what);
  }
  device_block(const dcomplex *host, long elements, const char *what) : device_block(elements, what) {
    if (elements > 0) cuda_check(cudaMemcpy(ptr_, host, (size_t)elements * sizeof(dcomplex), cudaMemcpyHostToDevice), what);
  }
  ~device_block() {
    if (ptr_) cudaFree(ptr_);
  }
  device_block(const device_block &) = delete;
  device_block &operator=(const device_block &) = delete;
  double *get() const { return static_cast<double *>(ptr_); }
  void *raw() const { return ptr_; }
  size_t bytes() const { return bytes_; }
  void to_host(dcomplex *host, long elements, const char *what) const {
    if (elements > 0) cuda_check(cudaMemcpy(host, ptr_, (size_t)elements * sizeof(dcomplex), cudaMemcpyDeviceToHost), what);
  }

 private:
  size_t bytes_;
  void *ptr_ = nullptr;
};

std::array<int, 3> int_dims(const mesh::periodic_mesh &m) {
  const auto &d = m.dims();
  for (long x : d)
    if (x < 1 || x > (1L << 30)) throw runtime_error("periodic mesh: dimension out of range");
  return {(int)d[0], (int)d[1], (int)d[2]};
}

// square matrix target [nb, nb], 1 <= nb <= 8
int matrix_nb(const std::vector<long> &t, const char *what) {
  if (t.size() != 2 || t[0] != t[1] || t[0] < 1 || t[0] > 8)
    fail(what, "target must be a square nb x nb matrix with 1 <= nb <= 8");
  return (int)t[0];
}

// rank-4 target [nb, nb, nb, nb], 1 <= nb <= 8
int tensor_nb(const std::vector<long> &t, const char *what) {
  if (t.size() != 4 || t[0] < 1 || t[0] > 8 || t[1] != t[0] || t[2] != t[0] || t[3] != t[0])
    fail(what, "target must be a rank-4 tensor nb x nb x nb x nb with 1 <= nb <= 8");
  return (int)t[0];
}

void need_fermion(const mesh::imfreq &m, const char *what) {
  if (m.statistic() != Fermion || m.n_iw() < 1) fail(what, "needs a fermionic Matsubara mesh with n_iw >= 1");
}
void need_boson(const mesh::imfreq &m, const char *what) {
  if (m.statistic() != Boson || m.n_iw() < 1) fail(what, "needs a bosonic Matsubara mesh with n_iw >= 1");
}

// the time mesh must hold at least twice the frequency mesh (fourier_matsubara.cpp:105-108, 128-131)
void need_long_enough(long n_tau, long n_freq_points, const char *what) {
  if (n_tau - 1 < n_freq_points) {
    std::ostringstream os;
    os << "too few time points: n_tau - 1 = " << n_tau - 1 << " < " << n_freq_points
       << " (the time mesh must be at least twice as long as the frequency mesh)";
    fail(what, os.str());
  }
}

template <typename G>
long n_elements(const G &g) {
  return g.data().size();
}

}  // namespace

// ---- Dyson (c++/triqs_tprf/lattice/gf.cpp:42-58, 91-132)

namespace {
g_wk_t dyson(double mu, const e_k_cvt &e_k, const mesh::imfreq &wmesh, const dcomplex *sigma, long sigma_elems,
             int kind, const char *what) {
  need_fermion(wmesh, what);
  const int nb = matrix_nb(e_k.target_shape(), what);
  const long nk = e_k.mesh().size();
  g_wk_t g({wmesh, e_k.mesh()}, {nb, nb});
  device_block d_ek(e_k.data().data(), n_elements(e_k), what);
  device_block d_sig(sigma, sigma ? sigma_elems : 0, what);
  device_block d_g(n_elements(g), what);
  check(tprf_lattice_dyson_g_wk(wmesh.beta(), (int)wmesh.n_iw(), nk, nb, mu, d_ek.get(), sigma ? d_sig.get() : nullptr,
                                kind, d_g.get(), nullptr),
        what);
  d_g.to_host(g.data().data(), n_elements(g), what);
  return g;
}
}  // namespace

g_wk_t lattice_dyson_g0_wk(double mu, e_k_cvt e_k, mesh::imfreq mesh) {
  return dyson(mu, e_k, mesh, nullptr, 0, 0, "lattice_dyson_g0_wk");
}

g_wk_t lattice_dyson_g_wk(double mu, e_k_cvt e_k, g_w_cvt sigma_w) {
  const char *what = "lattice_dyson_g_wk";
  const int nb = matrix_nb(e_k.target_shape(), what);
  if (sigma_w.target_shape() != std::vector<long>{nb, nb}) fail(what, "sigma_w and e_k have different targets");
  return dyson(mu, e_k, sigma_w.mesh(), sigma_w.data().data(), n_elements(sigma_w), 1, what);
}

g_wk_t lattice_dyson_g_wk(double mu, e_k_cvt e_k, g_wk_cvt sigma_wk) {
  const char *what = "lattice_dyson_g_wk";
  const int nb = matrix_nb(e_k.target_shape(), what);
  if (sigma_wk.target_shape() != std::vector<long>{nb, nb}) fail(what, "sigma_wk and e_k have different targets");
  if (!(std::get<1>(sigma_wk.mesh()) == e_k.mesh())) fail(what, "sigma_wk and e_k have different k meshes");
  return dyson(mu, e_k, std::get<0>(sigma_wk.mesh()), sigma_wk.data().data(), n_elements(sigma_wk), 2, what);
}

// ---- k <-> r (lattice/fourier.hpp:166-231, fourier/fourier_lattice.cpp:28-59)

namespace {
template <typename Out, typename In, typename NewP>
Out lattice_fft(const In &in, const NewP &new_p, bool forward, const char *what) {
  const auto &wm = std::get<0>(in.mesh());
  const auto d = int_dims(std::get<1>(in.mesh()));
  Out out({wm, new_p}, in.target_shape());
  long nt = 1;
  for (long s : in.target_shape()) nt *= s;
  device_block d_in(in.data().data(), n_elements(in), what);
  device_block d_out(n_elements(out), what);
  check(forward ? tprf_fourier_wk_to_wr(wm.size(), d.data(), nt, d_in.get(), d_out.get(), nullptr)
                : tprf_fourier_wr_to_wk(wm.size(), d.data(), nt, d_in.get(), d_out.get(), nullptr),
        what);
  d_out.to_host(out.data().data(), n_elements(out), what);
  return out;
}
}  // namespace

g_wr_t fourier_wk_to_wr(g_wk_cvt g_wk) {
  return lattice_fft<g_wr_t>(g_wk, mesh::cyclat(std::get<1>(g_wk.mesh()).dims()), true, "fourier_wk_to_wr");
}
g_wk_t fourier_wr_to_wk(g_wr_cvt g_wr) {
  return lattice_fft<g_wk_t>(g_wr, mesh::brzone(std::get<1>(g_wr.mesh()).dims()), false, "fourier_wr_to_wk");
}
chi_wk_t chi_wk_from_chi_wr(chi_wr_cvt chi_wr) {
  tensor_nb(chi_wr.target_shape(), "chi_wk_from_chi_wr");
  return lattice_fft<chi_wk_t>(chi_wr, mesh::brzone(std::get<1>(chi_wr.mesh()).dims()), false, "chi_wk_from_chi_wr");
}
chi_wr_t chi_wr_from_chi_wk(chi_wk_cvt chi_wk) {
  tensor_nb(chi_wk.target_shape(), "chi_wr_from_chi_wk");
  return lattice_fft<chi_wr_t>(chi_wk, mesh::cyclat(std::get<1>(chi_wk.mesh()).dims()), true, "chi_wr_from_chi_wk");
}

// ---- Matsubara transforms (lattice/fourier.hpp:99-163, fourier/fourier_matsubara.cpp)

g_tr_t fourier_wr_to_tr(g_wr_cvt g_wr, int nt) {
  const char *what = "fourier_wr_to_tr";
  const auto &wm = std::get<0>(g_wr.mesh());
  const auto &rm = std::get<1>(g_wr.mesh());
  need_fermion(wm, what);
  const int nb = matrix_nb(g_wr.target_shape(), what);
  const long n_tau = nt < 0 ? 6 * wm.n_iw() + 1 : nt;
  need_long_enough(n_tau, wm.size(), what);
  g_tr_t out({mesh::imtime(wm.beta(), Fermion, n_tau), rm}, {nb, nb});
  device_block d_in(g_wr.data().data(), n_elements(g_wr), what);
  device_block d_out(n_elements(out), what);
  check(tprf_fourier_wr_to_tr(wm.beta(), (int)wm.n_iw(), (int)n_tau, rm.size(), (long)nb * nb, d_in.get(), nullptr,
                              d_out.get(), nullptr),
        what);
  d_out.to_host(out.data().data(), n_elements(out), what);
  return out;
}

g_wr_t fourier_tr_to_wr(g_tr_cvt g_tr, int nw) {
  const char *what = "fourier_tr_to_wr";
  const auto &tm = std::get<0>(g_tr.mesh());
  const auto &rm = std::get<1>(g_tr.mesh());
  if (tm.statistic() != Fermion) fail(what, "needs a fermionic time mesh");
  const int nb = matrix_nb(g_tr.target_shape(), what);
  const long n_iw = nw < 0 ? (tm.size() - 1) / 6 : nw;
  if (n_iw < 1) fail(what, "needs at least one frequency");
  need_long_enough(tm.size(), 2 * n_iw, what);
  g_wr_t out({mesh::imfreq(tm.beta(), Fermion, n_iw), rm}, {nb, nb});
  device_block d_in(g_tr.data().data(), n_elements(g_tr), what);
  device_block d_out(n_elements(out), what);
  check(tprf_fourier_tr_to_wr(tm.beta(), (int)tm.size(), (int)n_iw, rm.size(), (long)nb * nb, d_in.get(), d_out.get(),
                              nullptr),
        what);
  d_out.to_host(out.data().data(), n_elements(out), what);
  return out;
}

chi_wr_t chi_wr_from_chi_tr(chi_tr_cvt chi_tr, int nw) {
  const char *what = "chi_wr_from_chi_tr";
  const auto &tm = std::get<0>(chi_tr.mesh());
  const auto &rm = std::get<1>(chi_tr.mesh());
  if (tm.statistic() != Boson) fail(what, "needs a bosonic time mesh");
  const int nb = tensor_nb(chi_tr.target_shape(), what);
  if (nw < 1) fail(what, "nw must be >= 1");
  need_long_enough(tm.size(), 2L * nw, what);
  chi_wr_t out({mesh::imfreq(tm.beta(), Boson, nw), rm}, chi_tr.target_shape());
  device_block d_in(chi_tr.data().data(), n_elements(chi_tr), what);
  device_block d_out(n_elements(out), what);
  check(tprf_chi_wr_from_chi_tr(tm.beta(), (int)tm.size(), nw, rm.size(), (long)nb * nb * nb * nb, d_in.get(),
                                d_out.get(), nullptr),
        what);
  d_out.to_host(out.data().data(), n_elements(out), what);
  return out;
}

chi_wr_t chi_w0r_from_chi_tr(chi_tr_cvt chi_tr) {
  const char *what = "chi_w0r_from_chi_tr";
  const auto &tm = std::get<0>(chi_tr.mesh());
  const auto &rm = std::get<1>(chi_tr.mesh());
  if (tm.statistic() != Boson) fail(what, "needs a bosonic time mesh");
  const int nb = tensor_nb(chi_tr.target_shape(), what);
  chi_wr_t out({mesh::imfreq(tm.beta(), Boson, 1), rm}, chi_tr.target_shape());
  device_block d_in(chi_tr.data().data(), n_elements(chi_tr), what);
  device_block d_out(n_elements(out), what);
  check(tprf_chi_w0r_from_chi_tr(tm.beta(), (int)tm.size(), rm.size(), (long)nb * nb * nb * nb, d_in.get(),
                                 d_out.get(), nullptr),
        what);
  d_out.to_host(out.data().data(), n_elements(out), what);
  return out;
}

chi_tr_t chi_tr_from_chi_wr(chi_wr_cvt chi_wr, int ntau) {
  const char *what = "chi_tr_from_chi_wr";
  const auto &wm = std::get<0>(chi_wr.mesh());
  const auto &rm = std::get<1>(chi_wr.mesh());
  need_boson(wm, what);
  const int nb = tensor_nb(chi_wr.target_shape(), what);
  const long n_tau = ntau < 0 ? 6 * wm.n_iw() + 1 : ntau;
  need_long_enough(n_tau, 2 * wm.n_iw(), what);
  chi_tr_t out({mesh::imtime(wm.beta(), Boson, n_tau), rm}, chi_wr.target_shape());
  device_block d_in(chi_wr.data().data(), n_elements(chi_wr), what);
  device_block d_out(n_elements(out), what);
  check(tprf_chi_tr_from_chi_wr(wm.beta(), (int)wm.n_iw(), (int)n_tau, rm.size(), (long)nb * nb * nb * nb, d_in.get(),
                                nullptr, d_out.get(), nullptr),
        what);
  d_out.to_host(out.data().data(), n_elements(out), what);
  return out;
}

// ---- bubble (lattice/chi_imtime.cpp:88-228)

namespace {
// G(tau, r) on a fermionic time mesh with a square target: (nb, dims)
int bubble_input(const g_tr_cvt &g_tr, std::array<int, 3> &d, const char *what) {
  const auto &tm = std::get<0>(g_tr.mesh());
  if (tm.statistic() != Fermion) fail(what, "needs G(tau, r) on a fermionic time mesh");
  if (tm.size() < 2) fail(what, "needs at least two time points");
  d = int_dims(std::get<1>(g_tr.mesh()));
  return matrix_nb(g_tr.target_shape(), what);
}
}  // namespace

chi_tr_t chi0_tr_from_grt_PH(g_tr_cvt g_tr) {
  const char *what = "chi0_tr_from_grt_PH";
  std::array<int, 3> d{};
  const int nb = bubble_input(g_tr, d, what);
  const auto &tm = std::get<0>(g_tr.mesh());
  chi_tr_t out({mesh::imtime(tm.beta(), Boson, tm.size()), std::get<1>(g_tr.mesh())}, {nb, nb, nb, nb});
  device_block d_in(g_tr.data().data(), n_elements(g_tr), what);
  device_block d_out(n_elements(out), what);
  check(tprf_chi0_tr_from_grt_PH((int)tm.size(), d.data(), nb, d_in.get(), d_out.get(), nullptr), what);
  d_out.to_host(out.data().data(), n_elements(out), what);
  return out;
}

chi_wr_t chi0_wr_from_grt_PH(g_tr_cvt g_tr, int nw) {
  const char *what = "chi0_wr_from_grt_PH";
  std::array<int, 3> d{};
  const int nb = bubble_input(g_tr, d, what);
  const auto &tm = std::get<0>(g_tr.mesh());
  if (nw < 1) fail(what, "nw must be >= 1");
  need_long_enough(tm.size(), 2L * nw, what);
  chi_wr_t out({mesh::imfreq(tm.beta(), Boson, nw), std::get<1>(g_tr.mesh())}, {nb, nb, nb, nb});
  device_block d_in(g_tr.data().data(), n_elements(g_tr), what);
  device_block d_out(n_elements(out), what);
  check(tprf_chi0_wr_from_grt_PH(tm.beta(), (int)tm.size(), nw, d.data(), nb, d_in.get(), d_out.get(), nullptr), what);
  d_out.to_host(out.data().data(), n_elements(out), what);
  return out;
}

chi_wr_t chi0_w0r_from_grt_PH(g_tr_cvt g_tr) {
  const char *what = "chi0_w0r_from_grt_PH";
  std::array<int, 3> d{};
  const int nb = bubble_input(g_tr, d, what);
  const auto &tm = std::get<0>(g_tr.mesh());
  chi_wr_t out({mesh::imfreq(tm.beta(), Boson, 1), std::get<1>(g_tr.mesh())}, {nb, nb, nb, nb});
  device_block d_in(g_tr.data().data(), n_elements(g_tr), what);
  device_block d_out(n_elements(out), what);
  check(tprf_chi0_w0r_from_grt_PH(tm.beta(), (int)tm.size(), d.data(), nb, d_in.get(), d_out.get(), nullptr), what);
  d_out.to_host(out.data().data(), n_elements(out), what);
  return out;
}

// ---- RPA (lattice/rpa.cpp:29-68)

chi_wk_t solve_rpa_PH(chi_wk_vt chi0, array_contiguous_view<dcomplex, 4> U) {
  const char *what = "solve_rpa_PH";
  const auto &wm = std::get<0>(chi0.mesh());
  need_boson(wm, what);
  const int nb = tensor_nb(chi0.target_shape(), what);
  for (long s : U.shape())
    if (s != nb) fail(what, "U must have the shape nb x nb x nb x nb of chi0's target");
  const auto d = int_dims(std::get<1>(chi0.mesh()));
  chi_wk_t out({wm, std::get<1>(chi0.mesh())}, chi0.target_shape());
  device_block d_chi0(chi0.data().data(), n_elements(chi0), what);
  device_block d_U(U.data(), U.size(), what);
  device_block d_out(n_elements(out), what);
  check(tprf_solve_rpa_PH_wk((int)wm.n_iw(), d.data(), nb, d_chi0.get(), d_U.get(), d_out.get(), nullptr), what);
  d_out.to_host(out.data().data(), n_elements(out), what);
  return out;
}

// ---- analytic Lindhard bubble (lattice/lindhard_chi00.cpp:34-100)

chi_wk_t lindhard_chi00(e_k_cvt e_k, mesh::imfreq mesh, double mu) {
  const char *what = "lindhard_chi00";
  need_boson(mesh, what);
  const int nb = matrix_nb(e_k.target_shape(), what);
  const long nk = e_k.mesh().size();
  const auto d = int_dims(e_k.mesh());
  chi_wk_t out({mesh, e_k.mesh()}, {nb, nb, nb, nb});
  device_block d_ek(e_k.data().data(), n_elements(e_k), what);
  device_block d_out(n_elements(out), what);
  const size_t ws_bytes = tprf_lindhard_chi00_workspace_bytes(nk, nb);
  device_block ws((long)((ws_bytes + sizeof(dcomplex) - 1) / sizeof(dcomplex)), what);
  check(tprf_lindhard_chi00(nk, d.data(), nb, d_ek.get(), mesh.beta(), mu, (int)mesh.n_iw(), d_out.get(), ws.raw(),
                            ws.bytes(), nullptr),
        what);
  d_out.to_host(out.data().data(), n_elements(out), what);
  return out;
}

// ---- the chain (python/triqs_tprf/lattice_utils.py:191-269)

chi_wk_t imtime_bubble_chi0_wk(g_wk_cvt g_wk, int nw) {
  const char *what = "imtime_bubble_chi0_wk";
  const auto &wm = std::get<0>(g_wk.mesh());
  need_fermion(wm, what);
  const int nb = matrix_nb(g_wk.target_shape(), what);
  if (nw < 1) fail(what, "nw must be >= 1");
  const long n_tau = 6 * wm.n_iw() + 1;
  need_long_enough(n_tau, 2L * nw, what);
  const auto d = int_dims(std::get<1>(g_wk.mesh()));
  chi_wk_t out({mesh::imfreq(wm.beta(), Boson, nw), std::get<1>(g_wk.mesh())}, {nb, nb, nb, nb});
  device_block d_g(g_wk.data().data(), n_elements(g_wk), what);
  device_block d_out(n_elements(out), what);
  const size_t ws_bytes = tprf_imtime_bubble_workspace_bytes((int)wm.n_iw(), (int)n_tau, d.data(), nb);
  device_block ws((long)((ws_bytes + sizeof(dcomplex) - 1) / sizeof(dcomplex)), what);
  check(tprf_imtime_bubble_chi0_wk(wm.beta(), (int)wm.n_iw(), (int)n_tau, nw, d.data(), nb, d_g.get(), nullptr,
                                   d_out.get(), ws.raw(), ws.bytes(), nullptr),
        what);
  d_out.to_host(out.data().data(), n_elements(out), what);
  return out;
}

}  // namespace triqs_tprf
