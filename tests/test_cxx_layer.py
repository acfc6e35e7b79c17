"""The C++ layer with TPRF's signatures (include/triqs_tprf_gb300/triqs_tprf.hpp).

tests/cpp/test_triqs_tprf.cpp is built with g++ against the layer and the C
ABI. Without a GPU it runs its host checks (mesh conventions, TRIQS data
order, argument errors thrown before any device work); with one (``-m gpu``)
it runs the reference's C++ chain on a small model and pytest compares every
result with the oracle.
"""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from conftest import PARITY_RTOL, rel_err

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    from tprf_gb300.build import _cxx, build_library, cxx_flags
    build_library()
    exe = str(tmp_path_factory.mktemp("cxx") / "test_triqs_tprf")
    cflags, lflags = cxx_flags()
    src = os.path.join(HERE, "cpp", "test_triqs_tprf.cpp")
    res = subprocess.run([_cxx(), *cflags, "-Wall", "-o", exe, src, *lflags], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def test_layer_links_and_host_checks_pass(program):
    res = subprocess.run([program, "host"], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "passed" in res.stdout


def test_layer_exports_the_reference_signatures():
    """Every function of the reference's C++ API on this path is declared with
    its reference argument list (the cited declarations)."""
    text = open(os.path.join(ROOT, "include", "triqs_tprf_gb300", "triqs_tprf.hpp")).read()
    for decl in ["g_wk_t lattice_dyson_g0_wk(double mu, e_k_cvt e_k, mesh::imfreq mesh);",
                 "g_wk_t lattice_dyson_g_wk(double mu, e_k_cvt e_k, g_w_cvt sigma_w);",
                 "g_wk_t lattice_dyson_g_wk(double mu, e_k_cvt e_k, g_wk_cvt sigma_wk);",
                 "g_wr_t fourier_wk_to_wr(g_wk_cvt g_wk);", "g_wk_t fourier_wr_to_wk(g_wr_cvt g_wr);",
                 "g_tr_t fourier_wr_to_tr(g_wr_cvt g_wr, int nt = -1);",
                 "g_wr_t fourier_tr_to_wr(g_tr_cvt g_tr, int nw = -1);",
                 "chi_tr_t chi0_tr_from_grt_PH(g_tr_cvt g_tr);", "chi_wr_t chi0_wr_from_grt_PH(g_tr_cvt g_tr, int nw);",
                 "chi_wr_t chi0_w0r_from_grt_PH(g_tr_cvt g_tr);", "chi_wr_t chi_w0r_from_chi_tr(chi_tr_cvt chi_tr);",
                 "chi_wr_t chi_wr_from_chi_tr(chi_tr_cvt chi_tr, int nw);",
                 "chi_tr_t chi_tr_from_chi_wr(chi_wr_cvt chi_wr, int ntau = -1);",
                 "chi_wk_t chi_wk_from_chi_wr(chi_wr_cvt chi_wr);", "chi_wr_t chi_wr_from_chi_wk(chi_wk_cvt chi_wk);",
                 "chi_wk_t solve_rpa_PH(chi_wk_vt chi0, array_contiguous_view<dcomplex, 4> U);",
                 "chi_wk_t lindhard_chi00(e_k_cvt e_k, mesh::imfreq mesh, double mu);"]:
        assert decl in text, decl


@pytest.mark.gpu
def test_reference_cxx_chain_matches_the_oracle(program, cuda_lib, tmp_path):
    from tprf_gb300 import workloads
    dims, beta, mu, n_max, nw = (6, 4, 2), 8.0, 0.1, 32, 24
    hop = workloads.cubic_3orb(1)
    ek = O.ek_from_hoppings(hop, dims)
    nb = ek.shape[-1]
    rng = np.random.default_rng(5)
    U = 0.3 * rng.standard_normal((nb,) * 4) + 0j
    (tmp_path / "params.txt").write_text(f"{beta!r} {mu!r} {n_max} {nw} {nb} {dims[0]} {dims[1]} {dims[2]}\n")
    ek.astype(np.complex128).tofile(tmp_path / "ek.bin")
    U.astype(np.complex128).tofile(tmp_path / "U.bin")
    prefix = str(tmp_path / "out")
    res = subprocess.run([program, "chain", str(tmp_path / "params.txt"), str(tmp_path / "ek.bin"),
                          str(tmp_path / "U.bin"), prefix], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout + res.stderr

    def load(name, shape):
        return np.fromfile(f"{prefix}.{name}.bin", dtype=np.complex128).reshape(shape)

    nk, n_tau, nwt = int(np.prod(dims)), 6 * n_max + 1, 2 * nw - 1
    g_wk = O.lattice_dyson_g0_wk(mu, ek, beta, n_max)
    g_wr = O.fourier_wk_to_wr(g_wk, dims)
    g_tr = O.fourier_wr_to_tr(g_wr, beta)
    chi0_tr = O.chi0_tr_from_grt_PH(g_tr, dims)
    chi0_wr = O.chi_wr_from_chi_tr(chi0_tr, beta, nw)
    chi0_wk = O.fourier_wr_to_wk(chi0_wr, dims)
    t4 = (nb,) * 4
    assert rel_err(load("g_wk", (2 * n_max, nk, nb, nb)), g_wk) < PARITY_RTOL
    assert rel_err(load("g_tr", (n_tau, nk, nb, nb)), g_tr) < PARITY_RTOL
    assert rel_err(load("chi0_wr", (nwt, nk) + t4), chi0_wr) < PARITY_RTOL
    assert rel_err(load("chi0_wk", (nwt, nk) + t4), chi0_wk) < PARITY_RTOL
    assert rel_err(load("chi_wk", (nwt, nk) + t4), O.solve_rpa_PH(chi0_wk, U)) < PARITY_RTOL
    assert rel_err(load("chi0_wr_save_memory", (nwt, nk) + t4), chi0_wr) < PARITY_RTOL
    assert rel_err(load("chi0_w0r", (1, nk) + t4), O.chi0_w0r_from_grt_PH(g_tr, beta, dims)) < PARITY_RTOL
    assert rel_err(load("chi_w0r", (1, nk) + t4), O.chi_w0r_from_chi_tr(chi0_tr, beta)) < PARITY_RTOL
    assert rel_err(load("chi0_wk_chain", (nwt, nk) + t4),
                   O.imtime_bubble_chi0_wk(g_wk, beta, dims, nw=nw)) < PARITY_RTOL
    assert rel_err(load("chi0_wr_back", (nwt, nk) + t4), O.fourier_wk_to_wr(chi0_wk, dims)) < PARITY_RTOL
    assert rel_err(load("g_wk_back", (2 * n_max, nk, nb, nb)), g_wk) < PARITY_RTOL
    assert rel_err(load("g_wr_from_tr", (2 * n_max, nk, nb, nb)), O.fourier_tr_to_wr(g_tr, beta, n_max)) < PARITY_RTOL
    # the bosonic w -> tau transform of the program's own chi0(w, r), against the
    # oracle on that same input: its tail fit amplifies a change of its input
    # about a hundredfold (the chain's chi0(w, r), 7e-13 from the oracle's, gives
    # 9e-11 after it; the transform itself adds 4e-12), so each stage is held to
    # the bar on the input it is given, as in the Matsubara parity tests
    assert rel_err(load("chi0_tr_from_wr", (6 * nw + 1, nk) + t4),
                   O.chi_tr_from_chi_wr(load("chi0_wr", (nwt, nk) + t4), beta, -1)) < PARITY_RTOL
    assert rel_err(load("lindhard", (nwt, nk) + t4), O.lindhard_chi00(ek, dims, beta, mu, nw)) < PARITY_RTOL
    iw = O.fermionic_iw(beta, n_max)
    sigma = np.zeros((2 * n_max, nb, nb), complex)
    sigma[:] = (-0.1j * np.sign(iw.imag))[:, None, None] * np.eye(nb)
    assert rel_err(load("g_wk_sigma", (2 * n_max, nk, nb, nb)),
                   O.lattice_dyson_g_wk(mu, ek, beta, n_max, sigma=sigma)) < PARITY_RTOL
