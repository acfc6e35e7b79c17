// Test program of the C++ layer with TPRF's signatures, run by tests/test_cxx_layer.py.
//
//   test_triqs_tprf host
//     mesh conventions, TRIQS data order and the argument checks that throw
//     triqs_tprf::runtime_error before any device work (no GPU needed);
//   test_triqs_tprf chain <params.txt> <e_k.bin> <U.bin> <out prefix>
//     the reference's C++ chain, called as a TPRF user calls it:
//       lattice_dyson_g0_wk -> fourier_wk_to_wr -> fourier_wr_to_tr ->
//       chi0_tr_from_grt_PH -> chi_wr_from_chi_tr -> chi_wk_from_chi_wr -> solve_rpa_PH
//     plus chi0_wr_from_grt_PH, chi0_w0r_from_grt_PH, imtime_bubble_chi0_wk,
//     lindhard_chi00 and the inverse transforms, each result written as raw
//     complex128 to <prefix>.<name>.bin for the comparison with the oracle.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "triqs_tprf_gb300/triqs_tprf.hpp"

using namespace triqs_tprf;

namespace {

int failures = 0, checks = 0;

void expect(bool ok, const std::string &what) {
  ++checks;
  if (!ok) {
    ++failures;
    std::cerr << "FAILED: " << what << "\n";
  }
}

template <typename F>
void expect_throw(F &&f, const std::string &needle, const std::string &what) {
  ++checks;
  try {
    f();
    ++failures;
    std::cerr << "FAILED (no exception): " << what << "\n";
  } catch (const runtime_error &e) {
    if (std::string(e.what()).find(needle) == std::string::npos) {
      ++failures;
      std::cerr << "FAILED (message '" << e.what() << "' lacks '" << needle << "'): " << what << "\n";
    }
  }
}

int host_checks() {
  // Matsubara meshes: fermionic n = -n_iw .. n_iw - 1, bosonic -(n_iw - 1) .. n_iw - 1
  mesh::imfreq wf(10.0, Fermion, 4), wb(10.0, Boson, 4);
  expect(wf.size() == 8 && wf.first_index() == -4 && wf.last_index() == 3, "fermionic mesh size and indices");
  expect(wb.size() == 7 && wb.first_index() == -3 && wb.last_index() == 3, "bosonic mesh size and indices");
  expect(std::abs(wf.index_to_value(0) - dcomplex(0, M_PI / 10.0)) < 1e-15, "i nu_0 = i pi / beta");
  expect(std::abs(wb.index_to_value(-2) - dcomplex(0, -4 * M_PI / 10.0)) < 1e-15, "i omega_-2 = -4 i pi / beta");
  mesh::imtime tm(5.0, Fermion, 11);
  expect(tm.size() == 11 && std::abs(tm.index_to_value(10) - 5.0) < 1e-15, "tau_{n_tau-1} = beta");
  // periodic meshes: row-major linear index over dims
  mesh::brzone bz({4, 3, 2});
  expect(bz.size() == 24 && bz.linear_index(1, 2, 1) == (1 * 3 + 2) * 2 + 1, "brzone linear index");
  const auto idx = bz.index(bz.linear_index(3, 1, 0));
  expect(idx[0] == 3 && idx[1] == 1 && idx[2] == 0, "brzone index round trip");
  expect(std::abs(bz.index_to_value(bz.linear_index(2, 0, 1))[0] - M_PI) < 1e-15 &&
             std::abs(bz.index_to_value(bz.linear_index(2, 0, 1))[2] - M_PI) < 1e-15,
         "k = 2 pi i / n");
  // gf data order: [w, k, a, b] in C order
  g_wk_t g({wf, bz}, {2, 2});
  expect(g.data().shape() == std::vector<long>({8, 24, 2, 2}), "g_wk shape [n_w, n_k, nb, nb]");
  g.data()(3, 5, 1, 0) = dcomplex(7.0, -1.0);
  expect(g.data().data()[((3 * 24 + 5) * 2 + 1) * 2 + 0] == dcomplex(7.0, -1.0), "g_wk element offset");
  g_wk_cvt cv = g;
  expect(cv.data().data() == g.data().data() && cv.data()(3, 5, 1, 0) == dcomplex(7.0, -1.0), "const view aliases");
  chi_wk_t chi({wb, bz}, {2, 2, 2, 2});
  expect(chi.data().shape() == std::vector<long>({7, 24, 2, 2, 2, 2}), "chi_wk shape");

  // argument checks (thrown on the host, before any device work)
  e_k_t ek(bz, {2, 2});
  expect_throw([&] { lattice_dyson_g0_wk(0.0, ek, wb); }, "fermionic", "Dyson on a bosonic mesh");
  e_k_t ek9(bz, {9, 9});
  expect_throw([&] { lattice_dyson_g0_wk(0.0, ek9, wf); }, "nb <= 8", "nb = 9");
  e_k_t ek_rect(bz, {2, 3});
  expect_throw([&] { lattice_dyson_g0_wk(0.0, ek_rect, wf); }, "square", "non-square target");
  g_w_t sig(wf, {3, 3});
  expect_throw([&] { lattice_dyson_g_wk(0.0, ek, g_w_cvt(sig)); }, "different targets", "sigma target");
  g_wr_t gwr({wf, mesh::cyclat({4, 3, 2})}, {2, 2});
  expect_throw([&] { fourier_wr_to_tr(gwr, 8); }, "too few time points", "n_tau - 1 < 2 n_iw");
  g_tr_t gtr({mesh::imtime(10.0, Fermion, 41), mesh::cyclat({4, 3, 2})}, {2, 2});
  expect_throw([&] { chi0_wr_from_grt_PH(gtr, 21); }, "too few time points", "bubble nw too large");
  expect_throw([&] { chi0_wr_from_grt_PH(gtr, 0); }, "nw must be", "nw = 0");
  expect_throw([&] { fourier_tr_to_wr(gtr, 21); }, "too few time points", "tau -> iw nw too large");
  chi_tr_t ctr_f({mesh::imtime(10.0, Fermion, 41), mesh::cyclat({4, 3, 2})}, {2, 2, 2, 2});
  expect_throw([&] { chi_wr_from_chi_tr(ctr_f, 4); }, "bosonic time mesh", "chi on a fermionic time mesh");
  chi_wk_t chi_f({wf, bz}, {2, 2, 2, 2});
  std::vector<dcomplex> U(16), U3(81);
  expect_throw([&] { solve_rpa_PH(chi_f, array_contiguous_view<dcomplex, 4>(U.data(), {2, 2, 2, 2})); },
               "bosonic", "RPA on a fermionic mesh");
  expect_throw([&] { solve_rpa_PH(chi, array_contiguous_view<dcomplex, 4>(U3.data(), {3, 3, 3, 3})); }, "shape",
               "U of the wrong shape");
  expect_throw([&] { imtime_bubble_chi0_wk(g, 0); }, "nw must be", "chain nw = 0");
  expect_throw([&] { imtime_bubble_chi0_wk(g, 13); }, "too few time points", "chain nw > 3 n_iw");
  std::cout << "host checks: " << checks - failures << "/" << checks << " passed\n";
  return failures == 0 ? 0 : 1;
}

template <typename G>
void write(const std::string &prefix, const std::string &name, const G &g) {
  std::ofstream f(prefix + "." + name + ".bin", std::ios::binary);
  f.write(reinterpret_cast<const char *>(g.data().data()), (std::streamsize)(g.data().size() * sizeof(dcomplex)));
}

std::vector<dcomplex> read(const std::string &path, size_t n) {
  std::vector<dcomplex> v(n);
  std::ifstream f(path, std::ios::binary);
  f.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(n * sizeof(dcomplex)));
  if (!f) throw std::runtime_error("cannot read " + path);
  return v;
}

int chain(const std::string &params, const std::string &ek_path, const std::string &U_path, const std::string &prefix) {
  double beta, mu;
  long n_iw, nw, nb, d0, d1, d2;
  std::ifstream p(params);
  if (!(p >> beta >> mu >> n_iw >> nw >> nb >> d0 >> d1 >> d2)) throw std::runtime_error("cannot read " + params);
  mesh::brzone bz({d0, d1, d2});
  e_k_t e_k(bz, {nb, nb});
  const auto ek = read(ek_path, (size_t)(bz.size() * nb * nb));
  std::copy(ek.begin(), ek.end(), e_k.data().data());
  std::vector<dcomplex> U = read(U_path, (size_t)(nb * nb * nb * nb));

  g_wk_t g_wk = lattice_dyson_g0_wk(mu, e_k, mesh::imfreq(beta, Fermion, n_iw));
  g_wr_t g_wr = fourier_wk_to_wr(g_wk);
  g_tr_t g_tr = fourier_wr_to_tr(g_wr);
  chi_tr_t chi0_tr = chi0_tr_from_grt_PH(g_tr);
  chi_wr_t chi0_wr = chi_wr_from_chi_tr(chi0_tr, (int)nw);
  chi_wk_t chi0_wk = chi_wk_from_chi_wr(chi0_wr);
  chi_wk_t chi_wk = solve_rpa_PH(chi0_wk, array_contiguous_view<dcomplex, 4>(U.data(), {nb, nb, nb, nb}));
  write(prefix, "g_wk", g_wk);
  write(prefix, "g_tr", g_tr);
  write(prefix, "chi0_wr", chi0_wr);
  write(prefix, "chi0_wk", chi0_wk);
  write(prefix, "chi_wk", chi_wk);
  write(prefix, "chi0_wr_save_memory", chi0_wr_from_grt_PH(g_tr, (int)nw));
  write(prefix, "chi0_w0r", chi0_w0r_from_grt_PH(g_tr));
  write(prefix, "chi_w0r", chi_w0r_from_chi_tr(chi0_tr));
  write(prefix, "chi0_wk_chain", imtime_bubble_chi0_wk(g_wk, (int)nw));
  write(prefix, "chi0_wr_back", chi_wr_from_chi_wk(chi0_wk));
  write(prefix, "g_wk_back", fourier_wr_to_wk(g_wr));
  write(prefix, "g_wr_from_tr", fourier_tr_to_wr(g_tr, (int)n_iw));
  write(prefix, "chi0_tr_from_wr", chi_tr_from_chi_wr(chi0_wr));
  write(prefix, "lindhard", lindhard_chi00(e_k, mesh::imfreq(beta, Boson, nw), mu));
  // Dyson with a self energy on the frequency mesh: Sigma(iv) = 0.1 i nu / |nu| (causal)
  g_w_t sigma(mesh::imfreq(beta, Fermion, n_iw), {nb, nb});
  for (long n = 0; n < sigma.mesh().size(); ++n) {
    const double nu = sigma.mesh().index_to_value(n + sigma.mesh().first_index()).imag();
    for (long a = 0; a < nb; ++a) sigma.data()(n, a, a) = dcomplex(0.0, -0.1 * (nu > 0 ? 1.0 : -1.0));
  }
  write(prefix, "g_wk_sigma", lattice_dyson_g_wk(mu, e_k, g_w_cvt(sigma)));
  std::cout << "chain: wrote " << prefix << ".*.bin\n";
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  try {
    const std::string mode = argc > 1 ? argv[1] : "host";
    if (mode == "host") return host_checks();
    if (mode == "chain" && argc == 6) return chain(argv[2], argv[3], argv[4], argv[5]);
    std::cerr << "usage: test_triqs_tprf host | chain <params> <e_k.bin> <U.bin> <prefix>\n";
    return 2;
  } catch (const std::exception &e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
}
