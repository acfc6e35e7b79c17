/*
 * triqs_tprf_gb300/triqs_tprf.hpp — C++ host layer with the signatures of TPRF's
 * C++ functions on this path, implemented over the C ABI of tprf_gb300.h.
 *
 * A C++ caller of TPRF (TRIQS/tprf 3.2) keeps its calls:
 *   g_wk_t   lattice_dyson_g0_wk(double mu, e_k_cvt e_k, mesh::imfreq mesh);   lattice/gf.hpp:44
 *   g_wk_t   lattice_dyson_g_wk(double mu, e_k_cvt e_k, g_w_cvt sigma_w);      lattice/gf.hpp:83
 *   g_wk_t   lattice_dyson_g_wk(double mu, e_k_cvt e_k, g_wk_cvt sigma_wk);    lattice/gf.hpp:123
 *   g_wr_t   fourier_wk_to_wr(g_wk_cvt g_wk);                                  lattice/gf.hpp:276
 *   g_wk_t   fourier_wr_to_wk(g_wr_cvt g_wr);                                  lattice/gf.hpp:286
 *   g_tr_t   fourier_wr_to_tr(g_wr_cvt g_wr, int nt = -1);                     lattice/gf.hpp:296
 *   g_wr_t   fourier_tr_to_wr(g_tr_cvt g_tr, int nw = -1);                     lattice/gf.hpp:306
 *   chi_tr_t chi0_tr_from_grt_PH(g_tr_cvt g_tr);                               lattice/chi_imtime.hpp:38
 *   chi_wr_t chi0_wr_from_grt_PH(g_tr_cvt g_tr, int nw);                       lattice/chi_imtime.hpp:40
 *   chi_wr_t chi0_w0r_from_grt_PH(g_tr_cvt g_tr);                              lattice/chi_imtime.hpp:54
 *   chi_wr_t chi_w0r_from_chi_tr(chi_tr_cvt chi_tr);                           lattice/chi_imtime.hpp:70
 *   chi_wr_t chi_wr_from_chi_tr(chi_tr_cvt chi_tr, int nw);                    lattice/chi_imtime.hpp:87
 *   chi_tr_t chi_tr_from_chi_wr(chi_wr_cvt chi_wr, int ntau = -1);             lattice/chi_imtime.hpp:105
 *   chi_wk_t chi_wk_from_chi_wr(chi_wr_cvt chi_wr);                            lattice/chi_imtime.hpp:123
 *   chi_wr_t chi_wr_from_chi_wk(chi_wk_cvt chi_wk);                            lattice/chi_imtime.hpp:141
 *   chi_wk_t solve_rpa_PH(chi_wk_vt chi0, array_contiguous_view<dcomplex, 4> U);  lattice/rpa.hpp:43
 *   chi_wk_t lindhard_chi00(e_k_cvt e_k, mesh::imfreq mesh, double mu);        lattice/lindhard_chi00.hpp:97
 * plus imtime_bubble_chi0_wk(g_wk, nw), the chain the reference writes in
 * Python (python/triqs_tprf/lattice_utils.py:191-269).
 *
 * The containers are small stand-ins for the TRIQS ones the reference's
 * type aliases name (c++/triqs_tprf/types.hpp:109-213): meshes imfreq, imtime,
 * brzone, cyclat and prod<...>, and gf<Mesh, Target> owning its data in host
 * memory in TRIQS data order (mesh indices first, then the target indices, C
 * order, std::complex<double>), with const views (..._cvt) and views (..._vt).
 * As in the reference, inputs are views and every output is a new gf returned
 * by value. Each call copies its inputs to device memory, runs the CUDA path
 * through the C ABI on the legacy default stream and copies the result back;
 * errors throw triqs_tprf::runtime_error (where TPRF throws
 * TRIQS_RUNTIME_ERROR) carrying tprf_last_error(). Argument checks run on the
 * host before any device work.
 *
 * Link: -ltprf_gb300_cxx -ltprf_gb300 -lcudart.
 */
#ifndef TRIQS_TPRF_GB300_HPP
#define TRIQS_TPRF_GB300_HPP

#include <array>
#include <complex>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

namespace triqs_tprf {

using dcomplex = std::complex<double>;

/* Thrown where the reference raises TRIQS_RUNTIME_ERROR. */
struct runtime_error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

enum statistic_enum { Boson = 0, Fermion = 1 };

namespace mesh {

/* Matsubara frequencies: fermionic i nu_n = i (2n + 1) pi / beta, n = -n_iw .. n_iw - 1
 * (2 n_iw points); bosonic i omega_m = i 2 m pi / beta, m = -(n_iw - 1) .. n_iw - 1
 * (2 n_iw - 1 points). n_iw is the number of non-negative frequencies. */
class imfreq {
 public:
  imfreq() = default;
  imfreq(double beta, statistic_enum statistic, long n_iw) : beta_(beta), statistic_(statistic), n_iw_(n_iw) {}
  double beta() const { return beta_; }
  statistic_enum statistic() const { return statistic_; }
  long n_iw() const { return n_iw_; }
  long size() const { return statistic_ == Fermion ? 2 * n_iw_ : 2 * n_iw_ - 1; }
  long first_index() const { return statistic_ == Fermion ? -n_iw_ : -(n_iw_ - 1); }
  long last_index() const { return n_iw_ - 1; }
  dcomplex index_to_value(long n) const;
  bool operator==(const imfreq &o) const {
    return beta_ == o.beta_ && statistic_ == o.statistic_ && n_iw_ == o.n_iw_;
  }

 private:
  double beta_ = 1.0;
  statistic_enum statistic_ = Fermion;
  long n_iw_ = 0;
};

/* Imaginary time tau_i = i beta / (n_tau - 1), i = 0 .. n_tau - 1. */
class imtime {
 public:
  imtime() = default;
  imtime(double beta, statistic_enum statistic, long n_tau) : beta_(beta), statistic_(statistic), n_tau_(n_tau) {}
  double beta() const { return beta_; }
  statistic_enum statistic() const { return statistic_; }
  long size() const { return n_tau_; }
  double index_to_value(long i) const { return n_tau_ > 1 ? beta_ * (double)i / (double)(n_tau_ - 1) : 0.0; }
  bool operator==(const imtime &o) const {
    return beta_ == o.beta_ && statistic_ == o.statistic_ && n_tau_ == o.n_tau_;
  }

 private:
  double beta_ = 1.0;
  statistic_enum statistic_ = Fermion;
  long n_tau_ = 0;
};

/* Periodic mesh of dims[0] x dims[1] x dims[2] points (unused dimensions 1),
 * linear index (i0 dims[1] + i1) dims[2] + i2. brzone: k_d = 2 pi i_d / dims[d]
 * in reciprocal-lattice units; cyclat: lattice vectors R = (i0, i1, i2). */
class periodic_mesh {
 public:
  periodic_mesh() = default;
  explicit periodic_mesh(std::array<long, 3> dims) : dims_(dims) {}
  const std::array<long, 3> &dims() const { return dims_; }
  long size() const { return dims_[0] * dims_[1] * dims_[2]; }
  long linear_index(long i0, long i1, long i2) const { return (i0 * dims_[1] + i1) * dims_[2] + i2; }
  std::array<long, 3> index(long linear) const {
    return {linear / (dims_[1] * dims_[2]), (linear / dims_[2]) % dims_[1], linear % dims_[2]};
  }
  bool operator==(const periodic_mesh &o) const { return dims_ == o.dims_; }

 private:
  std::array<long, 3> dims_{{1, 1, 1}};
};

class brzone : public periodic_mesh {
 public:
  using periodic_mesh::periodic_mesh;
  std::array<double, 3> index_to_value(long linear) const;
};

class cyclat : public periodic_mesh {
 public:
  using periodic_mesh::periodic_mesh;
};

/* Product mesh; std::get<0>(m), std::get<1>(m) give the components. */
template <typename M0, typename M1>
struct prod : std::tuple<M0, M1> {
  prod() = default;
  prod(M0 m0, M1 m1) : std::tuple<M0, M1>(std::move(m0), std::move(m1)) {}
  long size() const { return std::get<0>(*this).size() * std::get<1>(*this).size(); }
};

}  // namespace mesh

struct matrix_valued {
  static constexpr int rank = 2;
};
template <int R>
struct tensor_valued {
  static constexpr int rank = R;
};

/* Non-owning C-order view of a block of elements with a shape. */
template <typename T>
class array_view {
 public:
  array_view() = default;
  array_view(T *data, std::vector<long> shape) : data_(data), shape_(std::move(shape)) {}
  T *data() const { return data_; }
  const std::vector<long> &shape() const { return shape_; }
  long size() const {
    long n = 1;
    for (long s : shape_) n *= s;
    return n;
  }
  template <typename... I>
  T &operator()(I... idx) const {
    const long i[] = {static_cast<long>(idx)...};
    if (sizeof...(I) != shape_.size()) throw runtime_error("array_view: wrong number of indices");
    long off = 0;
    for (size_t d = 0; d < shape_.size(); ++d) off = off * shape_[d] + i[d];
    return data_[off];
  }

 private:
  T *data_ = nullptr;
  std::vector<long> shape_;
};

/* Stand-in for nda::array_contiguous_view<T, R> (the reference's U argument). */
template <typename T, int R>
class array_contiguous_view {
 public:
  array_contiguous_view(T *data, std::array<long, R> shape) : data_(data), shape_(shape) {}
  T *data() const { return data_; }
  const std::array<long, R> &shape() const { return shape_; }
  long size() const {
    long n = 1;
    for (long s : shape_) n *= s;
    return n;
  }

 private:
  T *data_;
  std::array<long, R> shape_;
};

template <typename Mesh>
inline std::vector<long> mesh_shape(const Mesh &m) {
  return {m.size()};
}
template <typename M0, typename M1>
inline std::vector<long> mesh_shape(const mesh::prod<M0, M1> &m) {
  return {std::get<0>(m).size(), std::get<1>(m).size()};
}

template <typename Mesh, typename Target>
class gf_view;
template <typename Mesh, typename Target>
class gf_const_view;

/* Green's function container: mesh, target shape and data [mesh..., target...]. */
template <typename Mesh, typename Target>
class gf {
 public:
  using mesh_t = Mesh;
  using view_type = gf_view<Mesh, Target>;
  using const_view_type = gf_const_view<Mesh, Target>;

  gf() = default;
  /* zero-filled; target_shape has Target::rank entries */
  gf(Mesh m, std::vector<long> target_shape) : mesh_(std::move(m)), target_(std::move(target_shape)) {
    if ((int)target_.size() != Target::rank) throw runtime_error("gf: target shape of the wrong rank");
    data_.assign((size_t)(mesh_.size() * target_size()), dcomplex(0.0, 0.0));
  }
  const Mesh &mesh() const { return mesh_; }
  const std::vector<long> &target_shape() const { return target_; }
  long target_size() const {
    long n = 1;
    for (long s : target_) n *= s;
    return n;
  }
  array_view<dcomplex> data() { return {data_.data(), full_shape()}; }
  array_view<const dcomplex> data() const { return {data_.data(), full_shape()}; }
  std::vector<long> full_shape() const {
    std::vector<long> s = mesh_shape(mesh_);
    s.insert(s.end(), target_.begin(), target_.end());
    return s;
  }

 private:
  Mesh mesh_;
  std::vector<long> target_;
  std::vector<dcomplex> data_;
};

/* Mutable view of a gf's (or any caller buffer's) data. */
template <typename Mesh, typename Target>
class gf_view {
 public:
  gf_view(Mesh m, std::vector<long> target_shape, dcomplex *data)
      : mesh_(std::move(m)), target_(std::move(target_shape)), data_(data) {}
  gf_view(gf<Mesh, Target> &g) : mesh_(g.mesh()), target_(g.target_shape()), data_(g.data().data()) {}  // NOLINT
  const Mesh &mesh() const { return mesh_; }
  const std::vector<long> &target_shape() const { return target_; }
  array_view<dcomplex> data() const {
    std::vector<long> s = mesh_shape(mesh_);
    s.insert(s.end(), target_.begin(), target_.end());
    return {data_, s};
  }

 private:
  Mesh mesh_;
  std::vector<long> target_;
  dcomplex *data_;
};

/* Read-only view. */
template <typename Mesh, typename Target>
class gf_const_view {
 public:
  gf_const_view(Mesh m, std::vector<long> target_shape, const dcomplex *data)
      : mesh_(std::move(m)), target_(std::move(target_shape)), data_(data) {}
  gf_const_view(const gf<Mesh, Target> &g)  // NOLINT: implicit, as TRIQS views
      : mesh_(g.mesh()), target_(g.target_shape()), data_(g.data().data()) {}
  gf_const_view(const gf_view<Mesh, Target> &v)  // NOLINT
      : mesh_(v.mesh()), target_(v.target_shape()), data_(v.data().data()) {}
  const Mesh &mesh() const { return mesh_; }
  const std::vector<long> &target_shape() const { return target_; }
  array_view<const dcomplex> data() const {
    std::vector<long> s = mesh_shape(mesh_);
    s.insert(s.end(), target_.begin(), target_.end());
    return {data_, s};
  }

 private:
  Mesh mesh_;
  std::vector<long> target_;
  const dcomplex *data_;
};

/* The reference's aliases (c++/triqs_tprf/types.hpp:109-213) on these stand-ins. */
using e_k_t = gf<mesh::brzone, matrix_valued>;
using e_k_cvt = e_k_t::const_view_type;
using e_k_vt = e_k_t::view_type;
using g_w_t = gf<mesh::imfreq, matrix_valued>;
using g_w_cvt = g_w_t::const_view_type;
using g_w_vt = g_w_t::view_type;
using g_wk_t = gf<mesh::prod<mesh::imfreq, mesh::brzone>, matrix_valued>;
using g_wk_cvt = g_wk_t::const_view_type;
using g_wk_vt = g_wk_t::view_type;
using g_wr_t = gf<mesh::prod<mesh::imfreq, mesh::cyclat>, matrix_valued>;
using g_wr_cvt = g_wr_t::const_view_type;
using g_wr_vt = g_wr_t::view_type;
using g_tr_t = gf<mesh::prod<mesh::imtime, mesh::cyclat>, matrix_valued>;
using g_tr_cvt = g_tr_t::const_view_type;
using g_tr_vt = g_tr_t::view_type;
using chi_tr_t = gf<mesh::prod<mesh::imtime, mesh::cyclat>, tensor_valued<4>>;
using chi_tr_cvt = chi_tr_t::const_view_type;
using chi_tr_vt = chi_tr_t::view_type;
using chi_wr_t = gf<mesh::prod<mesh::imfreq, mesh::cyclat>, tensor_valued<4>>;
using chi_wr_cvt = chi_wr_t::const_view_type;
using chi_wr_vt = chi_wr_t::view_type;
using chi_wk_t = gf<mesh::prod<mesh::imfreq, mesh::brzone>, tensor_valued<4>>;
using chi_wk_cvt = chi_wk_t::const_view_type;
using chi_wk_vt = chi_wk_t::view_type;

/* ---- the path (reference declarations cited in the file header) ---- */
g_wk_t lattice_dyson_g0_wk(double mu, e_k_cvt e_k, mesh::imfreq mesh);
g_wk_t lattice_dyson_g_wk(double mu, e_k_cvt e_k, g_w_cvt sigma_w);
g_wk_t lattice_dyson_g_wk(double mu, e_k_cvt e_k, g_wk_cvt sigma_wk);
g_wr_t fourier_wk_to_wr(g_wk_cvt g_wk);
g_wk_t fourier_wr_to_wk(g_wr_cvt g_wr);
/* nt = -1: 6 n_iw + 1 time points (TRIQS make_adjoint_mesh) */
g_tr_t fourier_wr_to_tr(g_wr_cvt g_wr, int nt = -1);
/* nw = -1: (n_tau - 1) / 6 positive fermionic frequencies */
g_wr_t fourier_tr_to_wr(g_tr_cvt g_tr, int nw = -1);
chi_tr_t chi0_tr_from_grt_PH(g_tr_cvt g_tr);
chi_wr_t chi0_wr_from_grt_PH(g_tr_cvt g_tr, int nw);
chi_wr_t chi0_w0r_from_grt_PH(g_tr_cvt g_tr);
chi_wr_t chi_w0r_from_chi_tr(chi_tr_cvt chi_tr);
chi_wr_t chi_wr_from_chi_tr(chi_tr_cvt chi_tr, int nw);
/* ntau = -1: 6 nw + 1 time points */
chi_tr_t chi_tr_from_chi_wr(chi_wr_cvt chi_wr, int ntau = -1);
chi_wk_t chi_wk_from_chi_wr(chi_wr_cvt chi_wr);
chi_wr_t chi_wr_from_chi_wk(chi_wk_cvt chi_wk);
chi_wk_t solve_rpa_PH(chi_wk_vt chi0, array_contiguous_view<dcomplex, 4> U);
chi_wk_t lindhard_chi00(e_k_cvt e_k, mesh::imfreq mesh, double mu);
/* g_wk -> chi0_wk as lattice_utils.imtime_bubble_chi0_wk (nw == 1: the static
 * trapezoid branch); chi0(tau, r) is never stored. */
chi_wk_t imtime_bubble_chi0_wk(g_wk_cvt g_wk, int nw = 1);

}  // namespace triqs_tprf

#endif  // TRIQS_TPRF_GB300_HPP
