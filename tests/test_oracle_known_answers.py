"""Pin the FP64 oracle against the known answers of the reference's own tests.

Tolerances are the reference tests' own (``np.testing`` decimal = d means
|diff| < 1.5 * 10**-d). Files cited relative to the TPRF source tree.
"""
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def test_lindhard_square_lattice():
    """test/python/chi00_square_lattice.py:90-180 (n_max = 500)."""
    f = _load("lindhard_square_2orb.npz")
    dims, beta, mu, ek = tuple(f["dims"]), float(f["beta"]), float(f["mu"]), f["e_k"]
    g0 = O.lattice_dyson_g0_wk(mu, ek, beta, 500)
    g0_tr = O.fourier_wr_to_tr(O.fourier_wk_to_wr(g0, dims), beta)
    chi_tr = O.chi0_tr_from_grt_PH(g0_tr, dims)
    lin_wr = O.chi_wr_from_chi_wk(f["chi00_wk_nw1"], dims)
    np.testing.assert_array_almost_equal(lin_wr, O.chi_wr_from_chi_tr(chi_tr, beta, 1), decimal=8)
    np.testing.assert_array_almost_equal(lin_wr, O.chi_w0r_from_chi_tr(chi_tr, beta), decimal=4)
    np.testing.assert_array_almost_equal(lin_wr, O.chi0_w0r_from_grt_PH(g0_tr, beta, dims), decimal=4)
    chi_wk = O.chi_wk_from_chi_wr(O.chi_wr_from_chi_tr(chi_tr, beta, 1), dims)
    np.testing.assert_array_almost_equal(f["chi00_wk_nw1"][0], chi_wk[0], decimal=7)
    np.testing.assert_array_almost_equal(f["chi00_wk_nw1"][0], O.imtime_bubble_chi0_wk(g0, beta, dims, nw=1)[0],
                                         decimal=4)
    # all bosonic frequencies, not only w = 0 (same bar as the w = 0 comparison)
    np.testing.assert_array_almost_equal(f["chi00_wk_nw4"], O.imtime_bubble_chi0_wk(g0, beta, dims, nw=4), decimal=7)


def _chain_1d(nk, nb, beta, mu, n_max, t=1.0):
    hop = {(0,): np.zeros((nb, nb)), (1,): -t * np.eye(nb), (-1,): -t * np.eye(nb)}
    dims = (nk, 1, 1)
    ek = O.ek_from_hoppings(hop, dims)
    return ek, dims, O.lattice_dyson_g0_wk(mu, ek, beta, n_max)


def test_hubbard_1d_bubble_and_fazekas_rpa():
    """test/python/mean_field.py:295-351 (half filling, m = 0: e(k) = -2 t cos k, mu = 0)."""
    f = _load("hubbard_1d_q0.npz")
    beta, U = float(f["beta"]), float(f["U"])
    ek, dims, g0 = _chain_1d(128, 2, beta, 0.0, 400)
    chi00 = O.imtime_bubble_chi0_wk(g0, beta, dims, nw=1)
    lin = O.lindhard_chi00(ek, dims, beta, 0.0, 1)
    np.testing.assert_almost_equal(chi00, lin, decimal=5)
    np.testing.assert_almost_equal(lin[0, 0, 0, 0, 0, 0], f["chi0_q0"])
    U_abcd = O.kanamori_quartic_tensor(1, U, 0.0, 0.0, 0.0)
    chi = O.solve_rpa_PH(chi00, U_abcd)
    Sz = 0.5 * np.diag([1.0, -1.0])
    szsz = np.einsum("wkabcd,ab,cd->wk", chi, Sz, Sz)
    np.testing.assert_almost_equal(szsz[0, 0], f["chi_szsz_q0"])


def general_vs_matrix_rpa_model():
    """The lattice of test/python/compare_general_rpa_to_matrix_rpa.py:18-60: two
    orbitals x spin (spin slow), nearest-neighbour hopping -1 on the square lattice
    with an inter-orbital part -0.1, 16 x 16 k, beta = 5, n_max = 30; Kanamori
    U = 1, U' = 0.8, J = J' = 0.1."""
    X = np.zeros((4, 4))
    X[0, 1] = X[1, 0] = X[2, 3] = X[3, 2] = 1.0
    T = -1.0 * np.eye(4) - 0.1 * X
    hop = {(0, 1): T, (0, -1): T, (1, 0): T, (-1, 0): T}
    return hop, (16, 16, 1), 5.0, 30, (1.0, 0.8, 0.1, 0.1)


def check_general_vs_matrix_rpa(chi00, chi, chi_spin, chi_charge, rtol):
    """The identities of compare_general_rpa_to_matrix_rpa.py:186-241, given the
    spin-resolved bubble and RPA chi (TPRF order) and the TPRF solves of the spin
    and charge channels: chi_uu = (chi_c + chi_s)/2, chi_ud = (chi_c - chi_s)/2,
    chi_xud = chi_s against the matrix formalism, the channel solves against it,
    and general -> charge/spin -> general."""
    norb = 2
    U, Up, J, Jp = general_vs_matrix_rpa_model()[-1]
    c0 = O.tprf_order_to_matrix_rpa_order(O.lose_spin_degree_of_freedom(chi00, 4, spin_fast=False))
    cs = O.chi_rpa_spin(c0, O.rpa_us_tensor(norb, U, Up, J, Jp))
    cc = O.chi_rpa_charge(c0, O.rpa_uc_tensor(norb, U, Up, J, Jp))
    m = O.tprf_order_to_matrix_rpa_order
    chi_uu, chi_ud = m(chi[..., :norb, :norb, :norb, :norb]), m(chi[..., :norb, :norb, norb:, norb:])
    chi_xud = m(chi[..., :norb, norb:, norb:, :norb])
    np.testing.assert_allclose(chi_uu, 0.5 * (cc + cs), rtol=rtol, atol=rtol * np.abs(cs).max())
    np.testing.assert_allclose(chi_ud, 0.5 * (cc - cs), rtol=rtol, atol=rtol * np.abs(cs).max())
    np.testing.assert_allclose(cs, chi_uu - chi_ud, rtol=rtol, atol=rtol * np.abs(cs).max())
    np.testing.assert_allclose(cc, chi_uu + chi_ud, rtol=rtol, atol=rtol * np.abs(cs).max())
    np.testing.assert_allclose(cs, chi_xud, rtol=rtol, atol=rtol * np.abs(cs).max())
    np.testing.assert_allclose(cs, m(chi_spin), rtol=rtol, atol=rtol * np.abs(cs).max())
    np.testing.assert_allclose(cc, m(chi_charge), rtol=rtol, atol=rtol * np.abs(cs).max())
    gen = O.general_susceptibility_from_charge_and_spin(chi_charge, chi_spin, spin_fast=False)
    np.testing.assert_allclose(chi, gen, rtol=rtol, atol=rtol * np.abs(chi).max())
    c, s = O.charge_and_spin_susceptibility_from_general(chi, spin_fast=False)
    np.testing.assert_allclose(chi, O.general_susceptibility_from_charge_and_spin(c, s, spin_fast=False), rtol=rtol,
                               atol=rtol * np.abs(chi).max())


def test_general_rpa_equals_matrix_rpa():
    """test/python/compare_general_rpa_to_matrix_rpa.py:150-241 on the oracle (the
    reference's rtol 1e-7; the restatement meets ~1e-15)."""
    hop, dims, beta, n_max, (U, Up, J, Jp) = general_vs_matrix_rpa_model()
    ek = O.ek_from_hoppings(hop, dims)
    chi00 = O.imtime_bubble_chi0_wk(O.lattice_dyson_g0_wk(0.0, ek, beta, n_max), beta, dims, nw=1)
    U_abcd = O.kanamori_quartic_tensor(2, U, Up, J, Jp)
    uc, us = O.split_quartic_tensor_in_charge_and_spin(U_abcd)
    np.testing.assert_allclose(O.rpa_us_tensor(2, U, Up, J, Jp), O.tprf_order_to_matrix_rpa_order(us))
    np.testing.assert_allclose(O.rpa_uc_tensor(2, U, Up, J, Jp), O.tprf_order_to_matrix_rpa_order(uc))
    c0 = O.lose_spin_degree_of_freedom(chi00, 4, spin_fast=False)
    check_general_vs_matrix_rpa(chi00, O.solve_rpa_PH(chi00, U_abcd), O.solve_rpa_PH(c0, us),
                                O.solve_rpa_PH(c0, -uc), rtol=1e-12)
    # the matrix-formalism index order is a permutation: tensor -> matrix -> tensor is exact
    x = np.random.default_rng(0).standard_normal((3,) + (2,) * 4)
    np.testing.assert_array_equal(O.matrix_to_tensor(O.tensor_to_matrix(x)), x)


def hartree_model():
    """test/python/hartree_response.py:33-85 (the branch it runs): one orbital x
    spin on a 4-site chain, t = 1, beta = 1, mu = 0, 100 fermionic frequencies,
    Kanamori U = 2.3, J = 0.4 (one orbital: the Hubbard U)."""
    T = -1.0 * np.eye(2)
    return {(0,): np.zeros((2, 2)), (1,): T, (-1,): T}, (4, 1, 1), 1.0, 100, 2.3, 0.4


def test_hartree_linear_response():
    """test/python/hartree_response.py:123-176 on the oracle: the static uniform
    bubble and RPA of the imaginary-time chain equal the Hartree linear response
    (finite differences of the mean-field density, eps = 1e-9) to the reference's
    decimal 7, density-density parts and Sz-Sz."""
    hop, dims, beta, n_max, U, J = hartree_model()
    ek = O.ek_from_hoppings(hop, dims)
    U_abcd = O.kanamori_quartic_tensor(1, U, U - 2 * J, J, J)
    chi0_ab, chi_ab = O.hartree_response(ek, beta, 0.0, U_abcd)
    chi00 = O.imtime_bubble_chi0_wk(O.lattice_dyson_g0_wk(0.0, ek, beta, n_max), beta, dims, nw=1)
    chi = O.solve_rpa_PH(chi00, U_abcd)
    check_hartree(chi00[0, 0], chi[0, 0], chi0_ab, chi_ab)


def check_hartree(chi0_abcd, chi_abcd, chi0_ab, chi_ab):
    dd = lambda x: np.array([[x[a, a, b, b] for b in range(2)] for a in range(2)])  # noqa: E731
    Sz = np.diag([0.5, -0.5])
    np.testing.assert_almost_equal(dd(chi0_abcd), chi0_ab)
    np.testing.assert_almost_equal(np.einsum("ab,abcd,cd->", Sz, chi0_abcd, Sz), np.einsum("aa,ab,bb->", Sz, chi0_ab, Sz))
    np.testing.assert_almost_equal(dd(chi_abcd), chi_ab)
    np.testing.assert_almost_equal(np.einsum("ab,abcd,cd->", Sz, chi_abcd, Sz), np.einsum("aa,ab,bb->", Sz, chi_ab, Sz))


def test_kanamori_1d_rpa_closed_form():
    """test/python/mean_field_kanamori.py:52-162 (2 orbitals x spin, spin fastest)."""
    f = _load("kanamori_1d_q0.npz")
    beta, U, J = float(f["beta"]), float(f["U"]), float(f["J"])
    ek, dims, g0 = _chain_1d(256, 4, beta, 0.0, 20)
    chi00 = O.imtime_bubble_chi0_wk(g0, beta, dims, nw=1)
    # Kanamori vertex (U' = U - 2J, J' = J), spin slow -> spin fast (up_0, do_0, up_1, do_1)
    Us = O.kanamori_quartic_tensor(2, U, U - 2 * J, J, J)
    perm = [0, 2, 1, 3]
    U_abcd = Us[np.ix_(perm, perm, perm, perm)]
    chi = O.solve_rpa_PH(chi00, U_abcd)
    Sz = 0.5 * np.diag([1.0, -1.0, 1.0, -1.0])
    szsz = np.einsum("wkabcd,ab,cd->wk", chi, Sz, Sz)
    np.testing.assert_array_almost_equal(szsz[0, 0].real, f["chi_szsz_q0"])


def test_k_r_round_trip():
    """test/python/g_wk_to_from_g_wr_py.py:13-31 (10 x 10, n_max = 1024, mu = 1)."""
    hop = {(1, 0): -np.eye(1), (-1, 0): -np.eye(1), (0, 1): -np.eye(1), (0, -1): -np.eye(1)}
    dims = (10, 10, 1)
    g0 = O.lattice_dyson_g0_wk(1.0, O.ek_from_hoppings(hop, dims), 1.0, 1024)
    np.testing.assert_array_almost_equal(g0, O.fourier_wr_to_wk(O.fourier_wk_to_wr(g0, dims), dims))


def test_save_memory_equals_plain():
    """test/python/chi0_save_memory.py:27-48 (create_model_for_tests, norb 2, dim 2)."""
    t_mat = -np.array([[1.0, 0.1], [0.1, 0.5]])
    hop = {(1, 0): t_mat, (-1, 0): t_mat, (0, 1): t_mat, (0, -1): t_mat}
    dims = (2, 2, 1)
    g0 = O.lattice_dyson_g0_wk(0.0, O.ek_from_hoppings(hop, dims), 1.0, 20)
    a = O.imtime_bubble_chi0_wk(g0, 1.0, dims, nw=10, save_memory=False)
    b = O.imtime_bubble_chi0_wk(g0, 1.0, dims, nw=10, save_memory=True)
    assert np.allclose(a, b)


def test_vandermonde_inverse_is_exact():
    V = np.array([[float(m) ** j for j in range(8)] for m in range(1, 9)])
    Vi = O.vandermonde_inverse(8)
    assert np.abs(Vi @ V - np.eye(8)).max() < 1e-8
    assert Vi[1, 3] == 172.75 and Vi[0, 0] == 8.0


def test_fit_derivative_rows_are_the_reference_table():
    """The oracle and the CUDA path apply rows 0 and 1 of the reference's rounded
    inverse Vandermonde table (fourier_matsubara.cpp:56-71); they lie within
    ~5e-12 relative of the exact rationals (a transcription check)."""
    exact = O.vandermonde_inverse(8)[:2]
    rel = np.abs(O.FIT_DERIVATIVE_ROWS - exact) / np.abs(exact)
    assert rel.max() < 6e-12 and rel.min() > 1e-13  # every entry rounded, none exact


def test_fit_derivatives_table_sensitivity():
    """The table's rounding (up to ~5e-12 relative of the exact inverse) is far
    below the accuracy bar: perturbing the rows by 1e-11 relative (about 3x that
    rounding) moves chi(i w) by < 1e-11 relative."""
    f = _load("lindhard_square_2orb.npz")
    dims, beta, ek = tuple(f["dims"]), float(f["beta"]), f["e_k"]
    g0 = O.lattice_dyson_g0_wk(0.0, ek, beta, 64)
    chi_tr = O.chi0_tr_from_grt_PH(O.fourier_wr_to_tr(O.fourier_wk_to_wr(g0, dims), beta), dims)
    base = O.chi_wr_from_chi_tr(chi_tr, beta, 16)
    saved = O.tprf_oracle._VINV.copy()
    try:
        rng = np.random.default_rng(1)
        O.tprf_oracle._VINV[...] = saved * (1 + 1e-11 * rng.standard_normal(saved.shape))
        pert = O.chi_wr_from_chi_tr(chi_tr, beta, 16)
    finally:
        O.tprf_oracle._VINV[...] = saved
    assert np.abs(pert - base).max() / np.abs(base).max() < 1e-11


def test_tail_fit_recovers_exact_g0_moments():
    f = _load("lindhard_square_2orb.npz")
    dims, beta, ek = tuple(f["dims"]), float(f["beta"]), f["e_k"]
    g_wr = O.fourier_wk_to_wr(O.lattice_dyson_g0_wk(0.0, ek, beta, 256), dims)
    g_fit, mom = O.fourier_wr_to_tr(g_wr, beta, return_moments=True)
    exact = O.g0_tail_moments_wr(ek, 0.0, dims)
    assert np.abs(mom - exact).max() < 1e-5
    g_exact = O.fourier_wr_to_tr(g_wr, beta, moments=exact)
    assert np.abs(g_fit - g_exact).max() < 1e-9


def test_mesh_too_short_raises():
    g = np.zeros((2 * 10, 1, 1, 1), complex)
    with pytest.raises(RuntimeError):
        O.fourier_wr_to_tr(g, 1.0, n_tau=20)
    with pytest.raises(RuntimeError):
        O.chi_wr_from_chi_tr(np.zeros((21, 1), complex), 1.0, nw=11)


def test_inverse_transforms_known_answers():
    """The inverse transforms (fourier_tr_to_wr, chi_tr_from_chi_wr) on analytic
    one-pole functions and as round trips with the forward transforms; the GW
    test of the reference (test/python/gw.py:88-103) uses both directions."""
    beta, n_max = 10.0, 64
    eps = np.array([-0.7, 0.3, 1.1])
    iv = O.fermionic_iw(beta, n_max)[:, None]
    g = 1.0 / (iv - eps[None])
    tau = O.tau_points(beta, 6 * n_max + 1)[:, None]
    g_tau = -np.exp(-eps[None] * tau) / (1 + np.exp(-beta * eps[None]))
    # analytic G(tau) of a level -> 1/(iv - e), up to the time mesh's discretisation
    assert np.abs(O.fourier_tr_to_wr(g_tau, beta, n_max) - g).max() < 1e-9
    # iv -> tau -> iv
    assert np.abs(O.fourier_tr_to_wr(O.fourier_wr_to_tr(g, beta), beta, n_max) - g).max() < 1e-10
    # bosonic: chi(iw) = 1/(iw - w0) - 1/(iw + w0) and its tau form
    nw = 64
    w = O.bosonic_iw(beta, nw)[:, None]
    w0 = np.array([0.5, 1.3])
    chi = 1.0 / (w - w0[None]) - 1.0 / (w + w0[None])
    taub = O.tau_points(beta, 6 * nw + 1)[:, None]

    def bos(x):
        return -np.exp(-x * taub) / (1 - np.exp(-beta * x))

    chi_tau = bos(w0[None]) - bos(-w0[None])
    ct = O.chi_tr_from_chi_wr(chi, beta)
    assert np.abs(ct - chi_tau).max() < 1e-5 * np.abs(chi_tau).max()
    assert np.abs(O.chi_wr_from_chi_tr(ct, beta, nw) - chi).max() < 1e-10 * np.abs(chi).max()
    with pytest.raises(RuntimeError):
        O.fourier_tr_to_wr(g_tau, beta, 200)  # time mesh shorter than 2 n_max


def _gw_chain_1d(beta=5.0, nk=8, n_max=64):
    dims = (nk, 1, 1)
    ek = O.ek_from_hoppings({(1, 0, 0): -np.eye(1), (-1, 0, 0): -np.eye(1)}, dims)
    return dims, ek, O.lattice_dyson_g0_wk(0.0, ek, beta, n_max)


def test_gw_tau_route_equals_matsubara_convolution():
    """GW self energy of the 1D Hubbard chain (the setting of test/python/gw.py:36-103):
    Sigma(k, iv) by the imaginary-time route (W(iw) -> W(tau), Sigma = -W G,
    Sigma(tau) -> Sigma(iv)) against the direct Matsubara convolution
    -1/(beta N) sum_{q, m} W(q, iw_m) G(k - q, iv - iw_m). The single-band W is
    V / (1 - PI V)."""
    beta, nk, n_max, V = 5.0, 8, 64, 1.0
    dims, ek, g_wk = _gw_chain_1d(beta, nk, n_max)
    PI = O.bubble_PI_wk(g_wk, beta, dims)
    assert PI.shape[0] == 2 * n_max - 1
    V_k = np.full((nk, 1, 1, 1, 1), V, complex)
    W = O.dynamical_screened_interaction_W(PI, V_k)
    assert np.abs(W[..., 0, 0, 0, 0] - V / (1 - PI[..., 0, 0, 0, 0] * V)).max() < 1e-14
    W_dyn, W_const = O.split_into_dynamic_wk_and_constant_k(W, beta)
    assert np.abs(W_const - V).max() < 1e-4  # W -> V at high frequency
    g_tr = O.fourier_wr_to_tr(O.fourier_wk_to_wr(g_wk, dims), beta)
    W_tr = O.chi_tr_from_chi_wr(O.chi_wr_from_chi_wk(W_dyn, dims), beta, g_tr.shape[0])
    sig = O.fourier_wr_to_wk(O.fourier_tr_to_wr(O.gw_dynamic_sigma(W_tr, g_tr), beta, n_max), dims)
    nv = np.arange(-n_max, n_max)
    direct = np.zeros((2 * n_max, nk), complex)
    for k in range(nk):
        for q in range(nk):
            for mi, m in enumerate(range(-(n_max - 1), n_max)):
                n2 = nv - m
                ok = (n2 >= -n_max) & (n2 < n_max)
                direct[ok, k] += W_dyn[mi, q, 0, 0, 0, 0] * g_wk[n2[ok] + n_max, (k - q) % nk, 0, 0]
    direct *= -1.0 / (beta * nk)
    low = slice(n_max - 8, n_max + 8)  # the truncated direct sum is exact only away from the mesh edge
    assert np.abs(sig[low, :, 0, 0] - direct[low]).max() < 1e-4 * np.abs(direct[low]).max()


def test_screened_interaction_index_conventions():
    """dynamical_screened_interaction.cpp:85-124 with PI = 0 gives W(a,b,c,d) = V(a,b,d,c)
    (the PH-grouped identity is delta_ad delta_bc); the dynamic-V form gives W = V."""
    rng = np.random.default_rng(5)
    nb, nk = 2, 3
    V = rng.standard_normal((nk,) + (nb,) * 4) + 1j * rng.standard_normal((nk,) + (nb,) * 4)
    W = O.dynamical_screened_interaction_W(np.zeros((2, nk) + (nb,) * 4, complex), V)
    assert np.allclose(W[0], np.swapaxes(V, -1, -2))
    Wd = O.dynamical_screened_interaction_W_wk(np.zeros((2, nk) + (nb,) * 4, complex), np.stack([V, V]))
    assert np.allclose(Wd[1], V)
