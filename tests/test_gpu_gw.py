"""GW consumers of the chain on the GPU against the FP64 oracle: bubble_PI_wk,
dynamical_screened_interaction_W (static and dynamic V), split into dynamic and
constant parts, gw_dynamic_sigma, and the whole imaginary-time GW self-energy
route of the reference's test/python/gw.py:88-103."""
import numpy as np
import pytest
import torch

import oracle as O
from conftest import PARITY_RTOL, rel_err

pytestmark = pytest.mark.gpu


def tp():
    import tprf_gb300 as T
    return T


def rand_c(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _model(nb, dims, beta, n_max, seed=0):
    T = tp()
    rng = np.random.default_rng(seed)
    hop = {}
    for R in [(1, 0, 0), (0, 1, 0)]:
        t = -np.eye(nb) + 0.2 * rng.standard_normal((nb, nb))
        hop[R] = t
        hop[tuple(-x for x in R)] = t.T
    ek = O.ek_from_hoppings(hop, dims)
    g_ref = O.lattice_dyson_g0_wk(0.0, ek, beta, n_max)
    e_k = T.Gf(mesh=T.MeshBrZone(dims=dims), data=ek)
    g_wk = T.lattice_dyson_g0_wk(0.0, e_k, T.MeshImFreq(beta, "Fermion", n_max))
    return ek, g_ref, g_wk


@pytest.mark.parametrize("nb", [1, 2])
def test_bubble_PI_wk(cuda_lib, nb):
    T = tp()
    dims, beta, n_max = (6, 4, 1), 5.0, 40
    _, g_ref, g_wk = _model(nb, dims, beta, n_max)
    PI = T.bubble_PI_wk(g_wk)
    ref = O.bubble_PI_wk(g_ref, beta, dims)
    assert tuple(PI.data.shape) == ref.shape == (2 * n_max - 1, 24) + (nb,) * 4
    assert rel_err(PI.data, ref) < PARITY_RTOL


@pytest.mark.parametrize("nb", [1, 2, 3])
@pytest.mark.parametrize("dynamic", [False, True])
def test_dynamical_screened_interaction_W(cuda_lib, nb, dynamic):
    T = tp()
    rng = np.random.default_rng(nb + 10 * dynamic)
    nw, dims = 5, (4, 3, 1)
    nk = 12
    PI = 0.2 * rand_c(rng, 2 * nw - 1, nk, *(nb,) * 4)
    kmesh = T.MeshBrZone(dims=dims)
    wmesh = T.MeshImFreq(3.0, "Boson", nw)
    pi = T.Gf(mesh=T.MeshProduct(wmesh, kmesh), data=PI)
    if dynamic:
        V = 0.5 * rand_c(rng, 2 * nw - 1, nk, *(nb,) * 4)
        v = T.Gf(mesh=T.MeshProduct(wmesh, kmesh), data=V)
        ref = O.dynamical_screened_interaction_W_wk(PI, V)
    else:
        V = 0.5 * rand_c(rng, nk, *(nb,) * 4)
        v = T.Gf(mesh=kmesh, data=V)
        ref = O.dynamical_screened_interaction_W(PI, V)
    W = T.dynamical_screened_interaction_W(pi, v)
    assert rel_err(W.data, ref) < PARITY_RTOL


def test_split_into_dynamic_wk_and_constant_k(cuda_lib):
    T = tp()
    dims, beta, n_max = (6, 4, 1), 5.0, 40
    _, g_ref, g_wk = _model(2, dims, beta, n_max)
    PI = T.bubble_PI_wk(g_wk)
    V = np.zeros((24,) + (2,) * 4, complex)
    for a in range(2):
        V[:, a, a, a, a] = 1.0
    W = T.dynamical_screened_interaction_W(PI, T.Gf(mesh=T.MeshBrZone(dims=dims), data=V))
    dyn, const = T.split_into_dynamic_wk_and_constant_k(W)
    dyn_ref, const_ref = O.split_into_dynamic_wk_and_constant_k(W.data.cpu().numpy(), beta)
    assert rel_err(const.data, const_ref) < PARITY_RTOL
    assert rel_err(dyn.data, dyn_ref) < PARITY_RTOL


def test_gw_dynamic_sigma(cuda_lib):
    T = tp()
    rng = np.random.default_rng(2)
    nb, n_tau, dims = 3, 37, (3, 2, 1)
    Wt = rand_c(rng, n_tau, 6, *(nb,) * 4)
    gt = rand_c(rng, n_tau, 6, nb, nb)
    rmesh = T.MeshCycLat(dims=dims)
    W = T.Gf(mesh=T.MeshProduct(T.MeshImTime(2.0, "Boson", n_tau), rmesh), data=Wt)
    g = T.Gf(mesh=T.MeshProduct(T.MeshImTime(2.0, "Fermion", n_tau), rmesh), data=gt)
    s = T.gw_dynamic_sigma(W, g)
    assert rel_err(s.data, O.gw_dynamic_sigma(Wt, gt)) < PARITY_RTOL
    with pytest.raises(RuntimeError):
        T.gw_dynamic_sigma(g, g)  # statistics


def test_gw_self_energy_route(cuda_lib):
    """The imaginary-time GW route of test/python/gw.py:88-103 on the GPU:
    bubble -> W (static V) -> split -> W_dyn(tau) -> Sigma(tau) = -W G -> Sigma(iv, k)."""
    T = tp()
    dims, beta, n_max = (8, 1, 1), 5.0, 64
    ek = O.ek_from_hoppings({(1, 0, 0): -np.eye(1), (-1, 0, 0): -np.eye(1)}, dims)
    kmesh = T.MeshBrZone(dims=dims)
    g_wk = T.lattice_dyson_g0_wk(0.0, T.Gf(mesh=kmesh, data=ek), T.MeshImFreq(beta, "Fermion", n_max))
    V_k = T.Gf(mesh=kmesh, data=np.full((8, 1, 1, 1, 1), 1.0, complex))
    PI = T.bubble_PI_wk(g_wk)
    W_dyn, _ = T.split_into_dynamic_wk_and_constant_k(T.dynamical_screened_interaction_W(PI, V_k))
    g_tr = T.fourier_wr_to_tr(T.fourier_wk_to_wr(g_wk))
    W_tr = T.chi_tr_from_chi_wr(T.chi_wr_from_chi_wk(W_dyn), ntau=len(g_tr.mesh.components[0]))
    sigma_wk = T.fourier_wr_to_wk(T.fourier_tr_to_wr(T.gw_dynamic_sigma(W_tr, g_tr), nw=n_max))
    # the same route in the oracle
    g_ref = O.lattice_dyson_g0_wk(0.0, ek, beta, n_max)
    W_ref = O.dynamical_screened_interaction_W(O.bubble_PI_wk(g_ref, beta, dims), np.full((8, 1, 1, 1, 1), 1.0, complex))
    Wd_ref, _ = O.split_into_dynamic_wk_and_constant_k(W_ref, beta)
    gt_ref = O.fourier_wr_to_tr(O.fourier_wk_to_wr(g_ref, dims), beta)
    Wt_ref = O.chi_tr_from_chi_wr(O.chi_wr_from_chi_wk(Wd_ref, dims), beta, gt_ref.shape[0])
    s_ref = O.fourier_wr_to_wk(O.fourier_tr_to_wr(O.gw_dynamic_sigma(Wt_ref, gt_ref), beta, n_max), dims)
    assert rel_err(sigma_wk.data, s_ref) < PARITY_RTOL
