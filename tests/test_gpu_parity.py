"""Parity of every CUDA kernel with the FP64 oracle (``-m gpu``).

Each test calls the C ABI through the ``tprf_gb300`` package on seeded inputs
small enough for the oracle, and compares with the oracle at the relative bar
PARITY_RTOL (max-abs error / max-abs value over the whole tensor). Mesh
indexing (output shapes, frequency and time ordering) is checked exactly.
"""
import numpy as np
import pytest
import torch

import oracle as O
from conftest import PARITY_RTOL, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True, params=["df64", "fp64", "df64_all"])
def arithmetic(request, cuda_lib):
    """Every parity test runs with the FFT stages in double-float (default), in
    native FP64, and with the RPA solve in double-float as well."""
    mode = {"df64": 0, "fp64": 1, "df64_all": 2}[request.param]
    assert cuda_lib.tprf_set_arithmetic(mode) == 0
    yield request.param
    cuda_lib.tprf_set_arithmetic(0)


def tp():
    import tprf_gb300 as T
    return T


def gf_ek(hop, dims):
    T = tp()
    ek = O.ek_from_hoppings(hop, dims)
    return ek, T.Gf(mesh=T.MeshBrZone(dims=dims), data=ek)


def rand_c(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


# ---------------------------------------------------------------------------
# (a) Dyson

@pytest.mark.parametrize("nb", [1, 2, 3, 4, 5, 8])
def test_dyson_g0_and_sigma(cuda_lib, nb):
    T = tp()
    rng = np.random.default_rng(nb)
    dims = (4, 3, 2)
    hop = {(1, 0, 0): rand_c(rng, nb, nb) * 0.3, (0, 1, 0): rand_c(rng, nb, nb) * 0.3}
    hop = {**hop, **{tuple(-x for x in R): t.conj().T for R, t in hop.items()}}
    ek, e_k = gf_ek(hop, dims)
    beta, n_max, mu = 7.0, 10, 0.3
    wmesh = T.MeshImFreq(beta, "Fermion", n_max)
    g0 = T.lattice_dyson_g0_wk(mu, e_k, wmesh)
    ref = O.lattice_dyson_g0_wk(mu, ek, beta, n_max)
    assert tuple(g0.data.shape) == ref.shape
    assert rel_err(g0.data, ref) < PARITY_RTOL
    sig_w = rand_c(rng, 2 * n_max, nb, nb)
    g1 = T.lattice_dyson_g_wk(mu, e_k, sigma_w=T.Gf(mesh=wmesh, data=sig_w))
    assert rel_err(g1.data, O.lattice_dyson_g_wk(mu, ek, beta, n_max, sigma=sig_w)) < PARITY_RTOL
    sig_wk = rand_c(rng, 2 * n_max, len(ek), nb, nb)
    g2 = T.lattice_dyson_g_wk(mu, e_k, sigma_wk=T.Gf(mesh=T.MeshProduct(wmesh, e_k.mesh), data=sig_wk))
    assert rel_err(g2.data, O.lattice_dyson_g_wk(mu, ek, beta, n_max, sigma=sig_wk)) < PARITY_RTOL


def test_dyson_matches_numpy_inverse(cuda_lib):
    """test/python/gf.py:60-73: G0 equals np.linalg.inv((iv + mu) I - e_k) per point."""
    T = tp()
    nb, dims, beta, mu, n_max = 2, (8, 1, 1), 3.0, 0.1, 16
    hop = {(1,): np.array([[-1.0, 0.2], [0.2, -0.5]]), (-1,): np.array([[-1.0, 0.2], [0.2, -0.5]])}
    ek, e_k = gf_ek(hop, dims)
    g0 = T.lattice_dyson_g0_wk(mu, e_k, T.MeshImFreq(beta, "Fermion", n_max)).data.cpu().numpy()
    iw = O.fermionic_iw(beta, n_max)
    for n in range(2 * n_max):
        for k in range(len(ek)):
            ref = np.linalg.inv((iw[n] + mu) * np.eye(nb) - ek[k])
            np.testing.assert_array_almost_equal(g0[n, k], ref, decimal=12)


# ---------------------------------------------------------------------------
# (b) lattice FFTs

@pytest.mark.parametrize("dims,nt", [((16, 16, 1), 5), ((4, 6, 5), 5), ((8, 1, 1), 5), ((7, 3, 10), 5),
                                     ((2, 2, 1), 5), ((1, 1, 1), 5), ((32, 8, 3), 5), ((64, 1, 1), 5),
                                     ((24, 48, 1), 5), ((8, 16, 32), 9), ((4, 64, 4), 25), ((2, 256, 1), 3),
                                     ((16, 1, 8), 1), ((32, 32, 4), 81)])
def test_lattice_fft(cuda_lib, dims, nt):
    """Every axis pattern: one-axis passes, the two-axis plane pass (powers of
    two, with and without a third axis, a trivial axis between), ragged target
    tiles."""
    from tprf_gb300 import _native
    rng = np.random.default_rng(sum(dims))
    nw = 3
    x = rand_c(rng, nw, int(np.prod(dims)), nt)
    xd = torch.as_tensor(x).cuda()
    out = torch.empty_like(xd)
    lib = _native.lib()
    _native.check(lib.tprf_fourier_wk_to_wr(nw, _native.dims3(dims), nt, xd.data_ptr(), out.data_ptr(), None))
    assert rel_err(out, O.fourier_wk_to_wr(x, dims)) < PARITY_RTOL
    back = torch.empty_like(xd)
    _native.check(lib.tprf_fourier_wr_to_wk(nw, _native.dims3(dims), nt, out.data_ptr(), back.data_ptr(), None))
    assert rel_err(back, x) < PARITY_RTOL
    # in place
    _native.check(lib.tprf_fourier_wr_to_wk(nw, _native.dims3(dims), nt, xd.data_ptr(), xd.data_ptr(), None))
    assert rel_err(xd, O.fourier_wr_to_wk(x, dims)) < PARITY_RTOL


@pytest.mark.parametrize("dims", [(11, 1, 1), (13, 22, 1), (3, 17, 2), (41, 1, 1)])
def test_lattice_fft_prime_lengths(cuda_lib, dims):
    """FFTW takes any length; so do the generic-radix stages."""
    from tprf_gb300 import _native
    rng = np.random.default_rng(7)
    x = rand_c(rng, 2, int(np.prod(dims)), 3)
    xd = torch.as_tensor(x).cuda()
    out = torch.empty_like(xd)
    _native.check(_native.lib().tprf_fourier_wk_to_wr(2, _native.dims3(dims), 3, xd.data_ptr(), out.data_ptr(), None))
    assert rel_err(out, O.fourier_wk_to_wr(x, dims)) < PARITY_RTOL


# ---------------------------------------------------------------------------
# (b) Matsubara transforms

def _g_wr(hop, dims, beta, n_max, mu=0.0):
    T = tp()
    ek, e_k = gf_ek(hop, dims)
    g_wk = T.lattice_dyson_g0_wk(mu, e_k, T.MeshImFreq(beta, "Fermion", n_max))
    g_wr = T.fourier_wk_to_wr(g_wk)
    ref = O.fourier_wk_to_wr(O.lattice_dyson_g0_wk(mu, ek, beta, n_max), dims)
    assert rel_err(g_wr.data, ref) < PARITY_RTOL
    return ek, g_wk, g_wr, ref


CASES = [
    (lambda: {(0, 1): -np.eye(1), (0, -1): -np.eye(1), (1, 0): -np.eye(1), (-1, 0): -np.eye(1)}, (8, 8, 1), 10.0, 64),
    (lambda: __import__("tprf_gb300.workloads", fromlist=["x"]).cubic_3orb(0), (4, 4, 4), 20.0, 32),
    (lambda: __import__("tprf_gb300.workloads", fromlist=["x"]).square_2orb(1), (6, 6, 1), 5.0, 45),
    # complex hoppings: G(tau, r) is complex, the bubble keeps one FFT per column
    (lambda: {(1, 0): np.array([[-1.0, 0.3j], [0.2j, -0.8]]), (-1, 0): np.array([[-1.0, 0.3j], [0.2j, -0.8]]).conj().T,
              (0, 1): np.array([[-0.5, 0.1], [-0.4j, -1.0]]), (0, -1): np.array([[-0.5, 0.1], [-0.4j, -1.0]]).conj().T},
     (6, 4, 1), 8.0, 40),
    # real hoppings with an odd number of bubble columns (25 x 81): the last real pair has one column
    (lambda: __import__("tprf_gb300.workloads", fromlist=["x"]).cubic_3orb(2), (5, 5, 1), 6.0, 30),
]


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("mode", ["fit", "moments"])
def test_nu_to_tau(cuda_lib, case, mode):
    T = tp()
    hopf, dims, beta, n_max = CASES[case]
    hop = hopf()
    ek, _, g_wr, g_wr_ref = _g_wr(hop, dims, beta, n_max)
    mom = O.g0_tail_moments_wr(ek, 0.0, dims) if mode == "moments" else None
    g_tr = T.fourier_wr_to_tr(g_wr, moments=mom)
    ref = O.fourier_wr_to_tr(g_wr_ref, beta, moments=mom)
    assert tuple(g_tr.data.shape) == ref.shape == (6 * n_max + 1,) + g_wr_ref.shape[1:]
    assert rel_err(g_tr.data, ref) < PARITY_RTOL
    for nt in (5 * n_max + 1, 4 * n_max + 7):  # a 5-smooth and a generic-prime time mesh
        g_tr2 = T.fourier_wr_to_tr(g_wr, nt=nt, moments=mom)
        assert rel_err(g_tr2.data, O.fourier_wr_to_tr(g_wr_ref, beta, nt, moments=mom)) < PARITY_RTOL


def test_nu_to_tau_tail_fit_error_is_reported(cuda_lib):
    T = tp()
    rng = np.random.default_rng(3)
    wmesh, rmesh = T.MeshImFreq(2.0, "Fermion", 100), T.MeshCycLat(dims=(2, 1, 1))
    data = rand_c(rng, 200, 2, 1, 1)
    assert O.tail_fit(data.reshape(200, -1), 2.0, 100)[1] > 1e-3  # the oracle sees the same misfit
    g = T.Gf(mesh=T.MeshProduct(wmesh, rmesh), data=data)
    with pytest.raises(RuntimeError, match="1e-3"):
        T.fourier_wr_to_tr(g)
    # the device error word is cleared: the next good call succeeds
    ek = O.ek_from_hoppings({(1,): -np.eye(1), (-1,): -np.eye(1)}, (2, 1, 1))
    g0 = O.fourier_wk_to_wr(O.lattice_dyson_g0_wk(0.0, ek, 2.0, 100), (2, 1, 1))
    T.fourier_wr_to_tr(T.Gf(mesh=g.mesh, data=g0))


@pytest.mark.parametrize("nw", [1, 2, 16, 64])
@pytest.mark.parametrize("n_tau", [-1, 263])  # L = 384 (7-smooth) and L = 262 = 2 x 131 (generic radix)
def test_tau_to_w(cuda_lib, nw, n_tau):
    T = tp()
    hopf, dims, beta, n_max = CASES[0]
    _, _, g_wr, g_wr_ref = _g_wr(hopf(), dims, beta, n_max)
    g_tr_ref = O.fourier_wr_to_tr(g_wr_ref, beta, n_tau)
    chi_tr_ref = O.chi0_tr_from_grt_PH(g_tr_ref, dims)
    tmesh = T.MeshImTime(beta, "Boson", chi_tr_ref.shape[0])
    chi_tr = T.Gf(mesh=T.MeshProduct(tmesh, T.MeshCycLat(dims=dims)), data=chi_tr_ref)
    chi_wr = T.chi_wr_from_chi_tr(chi_tr, nw)
    ref = O.chi_wr_from_chi_tr(chi_tr_ref, beta, nw)
    assert tuple(chi_wr.data.shape) == ref.shape == (2 * nw - 1,) + chi_tr_ref.shape[1:]
    assert rel_err(chi_wr.data, ref) < PARITY_RTOL
    assert rel_err(T.chi_w0r_from_chi_tr(chi_tr).data, O.chi_w0r_from_chi_tr(chi_tr_ref, beta)) < PARITY_RTOL


@pytest.mark.parametrize("n_iw,n_tau", [(64, -1), (40, 385), (17, 131)])  # 131: L = 2 5 13 (generic radix)
def test_fourier_tr_to_wr(cuda_lib, n_iw, n_tau):
    """Fermionic tau -> i nu (the inverse of fourier_wr_to_tr): G(tau, r) of the
    square lattice to G(i nu, r), against the oracle."""
    T = tp()
    hopf, dims, beta, n_max = CASES[0]
    _, _, g_wr, g_wr_ref = _g_wr(hopf(), dims, beta, n_max)
    g_tr_ref = O.fourier_wr_to_tr(g_wr_ref, beta, n_tau)
    tmesh = T.MeshImTime(beta, "Fermion", g_tr_ref.shape[0])
    g_tr = T.Gf(mesh=T.MeshProduct(tmesh, T.MeshCycLat(dims=dims)), data=g_tr_ref)
    nw = n_iw if n_tau > 0 else -1
    out = T.fourier_tr_to_wr(g_tr, nw=nw)
    n_expect = n_iw if n_tau > 0 else (g_tr_ref.shape[0] - 1) // 6
    ref = O.fourier_tr_to_wr(g_tr_ref, beta, n_expect)
    assert tuple(out.data.shape) == ref.shape == (2 * n_expect,) + g_tr_ref.shape[1:]
    assert rel_err(out.data, ref) < PARITY_RTOL


@pytest.mark.parametrize("nw,n_tau,mode", [(64, -1, "fit"), (40, 301, "fit"), (33, 250, "moments")])
def test_chi_tr_from_chi_wr(cuda_lib, nw, n_tau, mode):
    """Bosonic i omega -> tau (the inverse of chi_wr_from_chi_tr) with the tail fit on
    the bosonic mesh or given moments, against the oracle."""
    T = tp()
    hopf, dims, beta, n_max = CASES[0]
    _, _, _, g_wr_ref = _g_wr(hopf(), dims, beta, n_max)
    chi_tr_ref = O.chi0_tr_from_grt_PH(O.fourier_wr_to_tr(g_wr_ref, beta), dims)
    chi_wr_ref = O.chi_wr_from_chi_tr(chi_tr_ref, beta, nw)
    mom = None
    if mode == "moments":
        rng = np.random.default_rng(nw)
        mom = rand_c(rng, 3, *chi_wr_ref.shape[1:])
    wmesh = T.MeshImFreq(beta, "Boson", nw)
    chi_wr = T.Gf(mesh=T.MeshProduct(wmesh, T.MeshCycLat(dims=dims)), data=chi_wr_ref)
    out = T.chi_tr_from_chi_wr(chi_wr, ntau=n_tau, moments=mom)
    ref = O.chi_tr_from_chi_wr(chi_wr_ref, beta, n_tau, moments=mom)
    assert tuple(out.data.shape) == ref.shape == ((6 * nw + 1) if n_tau < 0 else n_tau,) + chi_wr_ref.shape[1:]
    assert rel_err(out.data, ref) < PARITY_RTOL


def test_inverse_transforms_reject_short_time_mesh(cuda_lib):
    T = tp()
    g_tr = T.Gf(mesh=T.MeshProduct(T.MeshImTime(5.0, "Fermion", 41), T.MeshCycLat(dims=(2, 1, 1))),
                data=np.zeros((41, 2, 1, 1), complex))
    with pytest.raises(T.TprfError):
        T.fourier_tr_to_wr(g_tr, nw=21)
    chi_wr = T.Gf(mesh=T.MeshProduct(T.MeshImFreq(5.0, "Boson", 30), T.MeshCycLat(dims=(2, 1, 1))),
                  data=np.zeros((59, 2, 1), complex))
    with pytest.raises(T.TprfError):
        T.chi_tr_from_chi_wr(chi_wr, ntau=50)


# ---------------------------------------------------------------------------
# (c) bubble

@pytest.mark.parametrize("case", range(len(CASES)))
def test_bubble_variants(cuda_lib, case):
    T = tp()
    hopf, dims, beta, n_max = CASES[case]
    _, _, g_wr, g_wr_ref = _g_wr(hopf(), dims, beta, n_max)
    g_tr = T.fourier_wr_to_tr(g_wr)
    g_tr_ref = O.fourier_wr_to_tr(g_wr_ref, beta)
    chi_tr = T.chi0_tr_from_grt_PH(g_tr)
    chi_tr_ref = O.chi0_tr_from_grt_PH(g_tr_ref, dims)
    assert rel_err(chi_tr.data, chi_tr_ref) < PARITY_RTOL
    nw = min(16, n_max)
    fused = T.chi0_wr_from_grt_PH(g_tr, nw)
    assert rel_err(fused.data, O.chi_wr_from_chi_tr(chi_tr_ref, beta, nw)) < PARITY_RTOL
    assert rel_err(T.chi0_w0r_from_grt_PH(g_tr).data, O.chi0_w0r_from_grt_PH(g_tr_ref, beta, dims)) < PARITY_RTOL


# ---------------------------------------------------------------------------
# (d) RPA

@pytest.mark.parametrize("nb", [1, 2, 3, 4, 5, 6, 8])
def test_rpa_random(cuda_lib, nb):
    T = tp()
    rng = np.random.default_rng(10 + nb)
    npts = 300
    chi0 = 0.1 * rand_c(rng, 3, npts // 3, nb, nb, nb, nb)
    U = 0.5 * rand_c(rng, nb, nb, nb, nb)
    mesh = T.MeshProduct(T.MeshImFreq(1.0, "Boson", 2), T.MeshBrZone(dims=(npts // 3, 1, 1)))
    chi = T.solve_rpa_PH(T.Gf(mesh=mesh, data=chi0), U)
    assert rel_err(chi.data, O.solve_rpa_PH(chi0, U)) < PARITY_RTOL


@pytest.mark.parametrize("nb,chunk,slots", [(1, 7, 2), (2, 50, 3), (3, 64, 1), (3, 1000, 3)])
def test_rpa_streamed_to_host(cuda_lib, nb, chunk, slots):
    """solve_rpa_PH(out=host) (chunks through a device ring, copies overlapped) gives
    the same bits as the device-resident solve, for ragged last chunks and a
    one-slot ring."""
    T = tp()
    rng = np.random.default_rng(40 + nb)
    chi0 = 0.1 * rand_c(rng, 7, 43, nb, nb, nb, nb)
    U = 0.5 * rand_c(rng, nb, nb, nb, nb)
    mesh = T.MeshProduct(T.MeshImFreq(1.0, "Boson", 4), T.MeshBrZone(dims=(43, 1, 1)))
    g = T.Gf(mesh=mesh, data=chi0)
    ref = T.solve_rpa_PH(g, U).data.cpu()
    out = torch.full(tuple(chi0.shape), complex("nan"), dtype=torch.complex128).pin_memory()
    ws = torch.empty(cuda_lib.tprf_solve_rpa_PH_to_host_workspace_bytes(chunk, nb, slots), dtype=torch.uint8,
                     device="cuda")
    res = T.solve_rpa_PH(g, U, out=out, chunk_points=chunk, workspace=ws)
    torch.cuda.synchronize()
    assert res.data.data_ptr() == out.data_ptr()
    assert torch.equal(out, ref)
    assert rel_err(out.numpy(), O.solve_rpa_PH(chi0, U)) < PARITY_RTOL


@pytest.mark.parametrize("gap", [1e-2, 1e-4, 1e-6])
def test_rpa_near_instability(cuda_lib, gap):
    """1 - U chi0 -> 0 at q = (pi, pi): the denominator's cancellation needs FP64
    (double-float points are re-solved in FP64 there)."""
    T = tp()
    dims, beta, n_max = (8, 8, 1), 10.0, 32
    ek = O.ek_from_hoppings({(0, 1): -np.eye(1), (0, -1): -np.eye(1), (1, 0): -np.eye(1), (-1, 0): -np.eye(1)}, dims)
    chi0 = O.imtime_bubble_chi0_wk(O.lattice_dyson_g0_wk(0.0, ek, beta, n_max), beta, dims, nw=4)
    c_max = chi0[:, :, 0, 0, 0, 0].real.max()
    U = np.full((1, 1, 1, 1), (1.0 - gap) / c_max + 0j)
    mesh = T.MeshProduct(T.MeshImFreq(beta, "Boson", 4), T.MeshBrZone(dims=dims))
    chi = T.solve_rpa_PH(T.Gf(mesh=mesh, data=chi0), U)
    ref = O.solve_rpa_PH(chi0, U)
    assert np.abs(ref).max() > 0.5 / gap * c_max  # the divergence is really there
    assert rel_err(chi.data, ref) < PARITY_RTOL


@pytest.mark.parametrize("gap", [1e-3, 1e-5])
def test_rpa_near_instability_multiorbital(cuda_lib, gap):
    T = tp()
    from tprf_gb300 import workloads
    dims, beta, n_max = (4, 4, 4), 20.0, 32
    ek = O.ek_from_hoppings(workloads.cubic_3orb(0), dims)
    chi0 = O.imtime_bubble_chi0_wk(O.lattice_dyson_g0_wk(0.0, ek, beta, n_max), beta, dims, nw=2)
    Us = workloads.kanamori_spin_vertex(3, 1.0, 0.2)
    # scale U so that the largest eigenvalue of chi0 U (grouped) is 1 - gap
    g = lambda x: np.swapaxes(x, -1, -2).reshape(x.shape[:-4] + (9, 9))  # noqa: E731
    lam = max(np.abs(np.linalg.eigvals(g(chi0) @ g(Us))).max(axis=-1).ravel())
    U = Us * (1.0 - gap) / lam
    mesh = T.MeshProduct(T.MeshImFreq(beta, "Boson", 2), T.MeshBrZone(dims=dims))
    chi = T.solve_rpa_PH(T.Gf(mesh=mesh, data=chi0), U)
    assert rel_err(chi.data, O.solve_rpa_PH(chi0, U)) < PARITY_RTOL


def test_rpa_singular_is_reported(cuda_lib):
    T = tp()
    mesh = T.MeshProduct(T.MeshImFreq(1.0, "Boson", 1), T.MeshBrZone(dims=(1, 1, 1)))
    chi0 = T.Gf(mesh=mesh, data=np.ones((1, 1, 1, 1, 1, 1), complex))
    with pytest.raises(RuntimeError, match="singular"):
        T.solve_rpa_PH(chi0, np.ones((1, 1, 1, 1), complex))


# ---------------------------------------------------------------------------
# whole chain and the reference's known answers

@pytest.mark.parametrize("nw", [1, 8])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_imtime_bubble_chain_and_rpa(cuda_lib, case, nw):
    T = tp()
    hopf, dims, beta, n_max = CASES[case]
    hop = hopf()
    ek, g_wk, _, _ = _g_wr(hop, dims, beta, n_max)
    chi0 = T.imtime_bubble_chi0_wk(g_wk, nw=nw, verbose=False)
    ref = O.imtime_bubble_chi0_wk(O.lattice_dyson_g0_wk(0.0, ek, beta, n_max), beta, dims, nw=nw)
    assert tuple(chi0.data.shape) == ref.shape
    assert rel_err(chi0.data, ref) < PARITY_RTOL
    nb = ek.shape[-1]
    rng = np.random.default_rng(case)
    U = 0.3 * (rng.standard_normal((nb,) * 4) + 0j)
    chi = T.solve_rpa_PH(chi0, U)
    assert rel_err(chi.data, O.solve_rpa_PH(ref, U)) < PARITY_RTOL


def test_lindhard_square_lattice_known_answer(cuda_lib):
    """test/python/chi00_square_lattice.py:90-180 through the CUDA path."""
    import os
    T = tp()
    f = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "lindhard_square_2orb.npz")))
    dims, beta = tuple(int(x) for x in f["dims"]), float(f["beta"])
    e_k = T.Gf(mesh=T.MeshBrZone(dims=dims), data=f["e_k"])
    g0 = T.lattice_dyson_g0_wk(0.0, e_k, T.MeshImFreq(beta, "Fermion", 500))
    g_tr = T.fourier_wr_to_tr(T.fourier_wk_to_wr(g0))
    chi_wr = T.chi_wr_from_chi_tr(T.chi0_tr_from_grt_PH(g_tr), 1)
    lin_wr = O.chi_wr_from_chi_wk(f["chi00_wk_nw1"], dims)
    np.testing.assert_array_almost_equal(lin_wr, chi_wr.data.cpu().numpy(), decimal=8)
    chi_wk = T.imtime_bubble_chi0_wk(g0, nw=4, verbose=False)
    np.testing.assert_array_almost_equal(f["chi00_wk_nw4"], chi_wk.data.cpu().numpy(), decimal=7)
    np.testing.assert_array_almost_equal(f["chi00_wk_nw1"][0], T.imtime_bubble_chi0_wk(g0, nw=1, verbose=False)
                                         .data.cpu().numpy()[0], decimal=4)


@pytest.mark.parametrize("nb,dims,nw", [(1, (6, 6, 1), 8), (2, (4, 4, 2), 70), (3, (3, 3, 3), 5)])
def test_lindhard_chi00_on_gpu(cuda_lib, nb, dims, nw):
    """Analytic Lindhard bubble (lindhard_chi00.cpp:34-94) on the GPU against the
    oracle; (2, 70) spans several output chunks per q."""
    T = tp()
    rng = np.random.default_rng(nb)
    hop = {}
    for R in [(1, 0, 0), (0, 1, 0), (0, 0, 1)]:
        t = -np.eye(nb) + 0.3 * (rng.standard_normal((nb, nb)) + 1j * rng.standard_normal((nb, nb)))
        hop[R] = t
        hop[tuple(-x for x in R)] = t.conj().T
    ek = O.ek_from_hoppings(hop, dims)
    beta, mu = 4.0, 0.2
    chi = T.lindhard_chi00(T.Gf(mesh=T.MeshBrZone(dims=dims), data=ek), T.MeshImFreq(beta, "Boson", nw), mu)
    ref = O.lindhard_chi00(ek, dims, beta, mu, nw)
    assert tuple(chi.data.shape) == ref.shape
    assert rel_err(chi.data, ref) < PARITY_RTOL


def test_lindhard_gpu_matches_imtime_chain(cuda_lib):
    """The known answer of test/python/chi00_square_lattice.py:90-180 with both sides on
    the GPU: the analytic Lindhard bubble against the imaginary-time chain."""
    import os
    T = tp()
    f = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "lindhard_square_2orb.npz")))
    dims, beta = tuple(int(x) for x in f["dims"]), float(f["beta"])
    e_k = T.Gf(mesh=T.MeshBrZone(dims=dims), data=f["e_k"])
    lin = T.lindhard_chi00(e_k, T.MeshImFreq(beta, "Boson", 4), float(f["mu"]))
    assert rel_err(lin.data, f["chi00_wk_nw4"]) < PARITY_RTOL
    g0 = T.lattice_dyson_g0_wk(float(f["mu"]), e_k, T.MeshImFreq(beta, "Fermion", 500))
    chi_wk = T.imtime_bubble_chi0_wk(g0, nw=4, verbose=False)
    np.testing.assert_array_almost_equal(lin.data.cpu().numpy(), chi_wk.data.cpu().numpy(), decimal=7)


def test_kanamori_rpa_closed_form(cuda_lib):
    """test/python/mean_field_kanamori.py:52-162 through the CUDA path."""
    import os
    T = tp()
    f = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "kanamori_1d_q0.npz")))
    beta, U, J = float(f["beta"]), float(f["U"]), float(f["J"])
    hop = {(1,): -np.eye(4), (-1,): -np.eye(4)}
    _, e_k = gf_ek(hop, (256, 1, 1))
    g0 = T.lattice_dyson_g0_wk(0.0, e_k, T.MeshImFreq(beta, "Fermion", 20))
    chi00 = T.imtime_bubble_chi0_wk(g0, nw=1, verbose=False)
    perm = [0, 2, 1, 3]
    U_abcd = O.kanamori_quartic_tensor(2, U, U - 2 * J, J, J)[np.ix_(perm, perm, perm, perm)]
    chi = T.solve_rpa_PH(chi00, U_abcd).data.cpu().numpy()
    Sz = 0.5 * np.diag([1.0, -1.0, 1.0, -1.0])
    szsz = np.einsum("wkabcd,ab,cd->wk", chi, Sz, Sz)
    np.testing.assert_array_almost_equal(szsz[0, 0].real, f["chi_szsz_q0"])


def test_general_rpa_equals_matrix_rpa_on_gpu(cuda_lib):
    """test/python/compare_general_rpa_to_matrix_rpa.py:150-241 through the CUDA
    path: the spin-resolved bubble (4 spin-orbitals) and RPA, and the spin and
    charge channels solved on their own (2 orbitals), obey chi_uu = (chi_c +
    chi_s)/2, chi_ud = (chi_c - chi_s)/2, chi_xud = chi_s and agree with the
    matrix formalism, to 1e-10 (the reference asserts rtol 1e-7)."""
    from test_oracle_known_answers import check_general_vs_matrix_rpa, general_vs_matrix_rpa_model
    T = tp()
    hop, dims, beta, n_max, (U, Up, J, Jp) = general_vs_matrix_rpa_model()
    ek, e_k = gf_ek(hop, dims)
    g0 = T.lattice_dyson_g0_wk(0.0, e_k, T.MeshImFreq(beta, "Fermion", n_max))
    chi00 = T.imtime_bubble_chi0_wk(g0, nw=1, verbose=False)
    U_abcd = O.kanamori_quartic_tensor(2, U, Up, J, Jp)
    uc, us = O.split_quartic_tensor_in_charge_and_spin(U_abcd)
    chi = T.solve_rpa_PH(chi00, U_abcd).data.cpu().numpy()
    c0 = O.lose_spin_degree_of_freedom(chi00.data.cpu().numpy(), 4, spin_fast=False).copy()
    c0g = T.Gf(mesh=chi00.mesh, data=c0)
    chi_s = T.solve_rpa_PH(c0g, us).data.cpu().numpy()
    chi_c = T.solve_rpa_PH(c0g, -uc).data.cpu().numpy()
    ref00 = O.imtime_bubble_chi0_wk(O.lattice_dyson_g0_wk(0.0, ek, beta, n_max), beta, dims, nw=1)
    assert rel_err(chi00.data, ref00) < PARITY_RTOL
    check_general_vs_matrix_rpa(chi00.data.cpu().numpy(), chi, chi_s, chi_c, rtol=PARITY_RTOL)


def test_hartree_linear_response_on_gpu(cuda_lib):
    """test/python/hartree_response.py:123-176 through the CUDA path: the static
    uniform bubble and RPA equal the Hartree linear response (finite differences
    of the mean-field density) to the reference's decimal 7."""
    from test_oracle_known_answers import check_hartree, hartree_model
    T = tp()
    hop, dims, beta, n_max, U, J = hartree_model()
    ek, e_k = gf_ek(hop, dims)
    U_abcd = O.kanamori_quartic_tensor(1, U, U - 2 * J, J, J)
    chi0_ab, chi_ab = O.hartree_response(ek, beta, 0.0, U_abcd)
    g0 = T.lattice_dyson_g0_wk(0.0, e_k, T.MeshImFreq(beta, "Fermion", n_max))
    chi00 = T.imtime_bubble_chi0_wk(g0, nw=1, verbose=False)
    chi = T.solve_rpa_PH(chi00, U_abcd)
    check_hartree(chi00.data.cpu().numpy()[0, 0], chi.data.cpu().numpy()[0, 0], chi0_ab, chi_ab)


def test_hubbard_1d_fazekas_rpa_on_gpu(cuda_lib):
    """test/python/mean_field.py:295-351 through the CUDA path: the 1D chain's
    static q = 0 bubble (imaginary-time chain and analytic Lindhard) and the RPA
    Sz-Sz response against the fixture's density-of-states integral and Fazekas
    closed form."""
    import os
    T = tp()
    f = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "hubbard_1d_q0.npz")))
    beta, U = float(f["beta"]), float(f["U"])
    hop = {(0,): np.zeros((2, 2)), (1,): -np.eye(2), (-1,): -np.eye(2)}
    _, e_k = gf_ek(hop, (128, 1, 1))
    g0 = T.lattice_dyson_g0_wk(0.0, e_k, T.MeshImFreq(beta, "Fermion", 400))
    chi00 = T.imtime_bubble_chi0_wk(g0, nw=1, verbose=False)
    lin = T.lindhard_chi00(e_k, T.MeshImFreq(beta, "Boson", 1), 0.0).data.cpu().numpy()
    np.testing.assert_almost_equal(chi00.data.cpu().numpy(), lin, decimal=5)
    np.testing.assert_almost_equal(lin[0, 0, 0, 0, 0, 0], f["chi0_q0"])
    chi = T.solve_rpa_PH(chi00, O.kanamori_quartic_tensor(1, U, 0.0, 0.0, 0.0)).data.cpu().numpy()
    Sz = 0.5 * np.diag([1.0, -1.0])
    np.testing.assert_almost_equal(np.einsum("wkabcd,ab,cd->wk", chi, Sz, Sz)[0, 0], f["chi_szsz_q0"])


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("u_kind", ["real", "complex", "kanamori"])
def test_rpa_on_the_wk_mesh_equals_the_point_solve(cuda_lib, case, u_kind):
    """solve_rpa_PH on a chi0 Gf (mesh-aware C ABI: conjugate point pairs solved
    once where chi0 and U allow, and with a symmetric U the transposition
    partner chi(w, -q) = chi(w, q)^T taken where chi0 is symmetric to within the
    solve's conditioning) gives the point-by-point solve (tprf_solve_rpa_PH) to
    rounding, and the oracle's chi. In the FP64 mode every point is solved on its
    own: the two agree exactly."""
    T = tp()
    from tprf_gb300 import _native
    hopf, dims, beta, n_max = CASES[case]
    ek, g_wk, _, _ = _g_wr(hopf(), dims, beta, n_max)
    chi0 = T.imtime_bubble_chi0_wk(g_wk, nw=6, verbose=False)
    nb = ek.shape[-1]
    rng = np.random.default_rng(10 + case)
    if u_kind == "kanamori":  # real and symmetric in the grouped indices: transposition partners apply
        from tprf_gb300.workloads import kanamori_spin_vertex
        U = np.full((1, 1, 1, 1), 0.8 + 0j) if nb == 1 else np.asarray(kanamori_spin_vertex(nb, 0.8, 0.15), complex)
    else:
        U = 0.3 * rng.standard_normal((nb,) * 4) + (0.1j * rng.standard_normal((nb,) * 4) if u_kind == "complex" else 0j)
    chi = T.solve_rpa_PH(chi0, U)
    flat = torch.empty_like(chi0.data)
    Ud = torch.as_tensor(U, dtype=torch.complex128, device="cuda").contiguous()
    n_points = chi0.data.numel() // nb ** 4
    _native.check(cuda_lib.tprf_solve_rpa_PH(n_points, nb, chi0.data.data_ptr(), Ud.data_ptr(), flat.data_ptr(), None))
    torch.cuda.synchronize()
    if cuda_lib.tprf_get_arithmetic() == 1:
        assert torch.equal(chi.data, flat)
    else:
        assert rel_err(chi.data, flat) < 1e-12
    ref0 = O.imtime_bubble_chi0_wk(O.lattice_dyson_g0_wk(0.0, ek, beta, n_max), beta, dims, nw=6)
    assert rel_err(chi.data, O.solve_rpa_PH(ref0, U)) < PARITY_RTOL


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("block_freqs,slots", [(2, 2), (1, 3), (8, 1)])
def test_fused_chain_and_rpa_to_host_equals_the_two_calls(cuda_lib, case, block_freqs, slots):
    """imtime_bubble_rpa_wk (r -> q, RPA and host copies in frequency blocks)
    gives exactly solve_rpa_PH(imtime_bubble_chi0_wk(...)), real and complex U."""
    T = tp()
    from tprf_gb300.lattice_utils import imtime_bubble_rpa_wk
    hopf, dims, beta, n_max = CASES[case]
    ek, g_wk, _, _ = _g_wr(hopf(), dims, beta, n_max)
    nb = ek.shape[-1]
    rng = np.random.default_rng(20 + case)
    for U in (0.3 * rng.standard_normal((nb,) * 4) + 0j,
              0.3 * rng.standard_normal((nb,) * 4) + 0.05j * rng.standard_normal((nb,) * 4)):
        two = T.solve_rpa_PH(T.imtime_bubble_chi0_wk(g_wk, nw=5, verbose=False), U)
        fused = imtime_bubble_rpa_wk(g_wk, U, 5, block_freqs=block_freqs, slots=slots)
        torch.cuda.synchronize()
        assert torch.equal(fused.data, two.data.cpu())


# Layouts of the last r -> q pass, which stores a real bubble's negative
# frequencies from their partners: the two-axis pass last (a trivial axis in
# front or in the middle), one axis (the first or the last), and an axis
# sequence ending on the middle axis (a length that is not a power of two).
PARTNER_MESHES = [(1, 8, 8), (4, 1, 4), (1, 1, 8), (8, 1, 1), (1, 6, 6), (1, 6, 4)]


def _real_nn_model(dims):
    """Two bands, real nearest-neighbour hoppings along every non-trivial axis."""
    t = np.array([[-1.0, 0.2], [0.2, -0.6]])
    hop = {(0, 0, 0): np.diag([0.3, -0.2])}
    for ax, d in enumerate(dims):
        if d > 1:
            R = [0, 0, 0]
            R[ax] = 1
            hop[tuple(R)] = t
            hop[tuple(-x for x in R)] = t.T
    return hop


@pytest.mark.parametrize("dims", PARTNER_MESHES)
def test_partner_stores_on_every_mesh_layout(cuda_lib, arithmetic, dims):
    """On every layout of the last r -> q pass: chi0 matches the oracle, its
    negative frequencies are exactly the partners' conjugates, chi0(-w, q) =
    conj(chi0(w, -q)) (the native FP64 mode transforms every row and meets the
    symmetry to the parity bar), and the fused call (partner stores per
    frequency block) gives exactly the two calls' chi."""
    T = tp()
    from tprf_gb300.lattice_utils import imtime_bubble_rpa_wk
    beta, n_max, nw = 8.0, 24, 5
    ek, g_wk, _, _ = _g_wr(_real_nn_model(dims), dims, beta, n_max)
    chi0 = T.imtime_bubble_chi0_wk(g_wk, nw=nw, verbose=False)
    ref = O.imtime_bubble_chi0_wk(O.lattice_dyson_g0_wk(0.0, ek, beta, n_max), beta, dims, nw=nw)
    assert rel_err(chi0.data, ref) < PARITY_RTOL
    x = chi0.data.cpu().reshape((2 * nw - 1,) + tuple(dims) + (-1,))
    partner = torch.conj(torch.flip(x, dims=[0]))  # row i <- row 2 (nw - 1) - i
    for ax in (1, 2, 3):  # k -> (N - k) mod N along every mesh axis
        partner = torch.roll(torch.flip(partner, dims=[ax]), shifts=1, dims=ax)
    if arithmetic == "fp64":
        assert rel_err(x[: nw - 1], partner[: nw - 1]) < PARITY_RTOL
    else:
        assert torch.equal(x[: nw - 1], partner[: nw - 1])
    rng = np.random.default_rng(sum(dims))
    U = 0.3 * rng.standard_normal((2,) * 4) + 0j
    two = T.solve_rpa_PH(chi0, U)
    assert rel_err(two.data, O.solve_rpa_PH(ref, U)) < PARITY_RTOL
    for block_freqs in (1, 2):
        fused = imtime_bubble_rpa_wk(g_wk, U, nw, block_freqs=block_freqs, slots=2)
        torch.cuda.synchronize()
        assert torch.equal(fused.data, two.data.cpu())


@pytest.mark.parametrize("fill", ["host", "half"])
@pytest.mark.parametrize("case", [0, 3, len(CASES) - 1])
def test_pipelined_fused_calls_equal_the_waiting_call(cuda_lib, arithmetic, case, fill):
    """imtime_bubble_rpa_wk(wait=False) back to back on several inputs sharing
    one workspace (the copies of a call running behind the next call's chain,
    whose solves wait for the ring slots they reuse), then join_host_copies:
    every output equals the waiting call's chi. fill: every negative frequency
    of a real chi filled on the host, or a fixed split with half of the blocks'
    negative frequencies over the link."""
    T = tp()
    from tprf_gb300 import _native
    from tprf_gb300.lattice_utils import imtime_bubble_rpa_wk, join_host_copies
    hopf, dims, beta, n_max = CASES[case]
    ek, g_wk, _, _ = _g_wr(hopf(), dims, beta, n_max)
    nb = ek.shape[-1]
    rng = np.random.default_rng(40 + case)
    Us = [0.3 * rng.standard_normal((nb,) * 4) + 0j for _ in range(3)]
    nw, block, slots = 5, 1, 2
    lib = _native.lib()
    need = lib.tprf_imtime_bubble_rpa_to_host_workspace_bytes(n_max, -1, nw, _native.dims3(dims), nb, block, slots)
    ws = torch.empty(int(need), dtype=torch.uint8, device="cuda")
    chi0 = torch.empty((2 * nw - 1, int(np.prod(dims))) + (nb,) * 4, dtype=torch.complex128, device="cuda")
    expect = [imtime_bubble_rpa_wk(g_wk, U, nw, block_freqs=block, slots=slots).data.clone() for U in Us]
    outs = [torch.empty_like(e).pin_memory() for e in expect]
    lib.tprf_set_sync_checks(0)
    if fill == "host":
        lib.tprf_set_host_fill(1)  # every negative frequency of a real chi filled on the host
    else:
        assert lib.tprf_set_host_fill_fraction(0.5) == 0
    try:
        for U, out in zip(Us, outs):
            imtime_bubble_rpa_wk(g_wk, U, nw, out=out, block_freqs=block, slots=slots, chi0=chi0, workspace=ws,
                                 wait=False)
        join_host_copies()
        torch.cuda.synchronize()
        _native.check(lib.tprf_check_device_status(None), "pipelined calls")
    finally:
        lib.tprf_set_sync_checks(1)
        lib.tprf_set_host_fill(-1)
    for e, out in zip(expect, outs):
        assert torch.equal(out, e)
    # real hoppings and a real U on the double-float path (which records that the
    # bubble is real): only the frequencies w >= 0 crossed to the host, plus, with
    # half the blocks (one frequency each) sending their negative rows, those of
    # blocks 2 and 4 (block 0 holds w = 0 alone)
    rows = (nw if fill == "host" else nw + 2) if case != 3 and arithmetic != "fp64" else 2 * nw - 1
    assert lib.tprf_imtime_bubble_rpa_to_host_last_d2h_bytes() == rows * int(np.prod(dims)) * nb ** 4 * 16
    with pytest.raises(ValueError):
        imtime_bubble_rpa_wk(g_wk, Us[0], nw, wait=False)


def _orbital_reversal(nb):
    """o = abcd (a slowest) -> dcba for the nb^4 bubble columns."""
    rev = []
    for o in range(nb ** 4):
        x, r = o, 0
        for _ in range(4):
            r, x = r * nb + x % nb, x // nb
        rev.append(r)
    return np.array(rev)


@pytest.mark.parametrize("model", ["cubic_3orb", "layered_5orb"])
@pytest.mark.parametrize("complex_hop", [False, True])
def test_compact_orbital_columns_on_a_3d_mesh(cuda_lib, arithmetic, complex_hop, model):
    """The chain on a three-dimensional mesh whose last two axes share one plane
    pass: with real hoppings the bubble is real and transpose-symmetric, so only
    the canonical orbital columns abcd <= dcba are transformed r -> q (45 of 81
    at nb = 3, 325 of 625 at nb = 5) and the last pass stores
    chi0(w, -q)_dcba = chi0(w, q)_abcd bit for bit; with complex hoppings the
    same mesh takes the full path. Both against the oracle."""
    T = tp()
    from tprf_gb300 import workloads
    hop = workloads.cubic_3orb(3) if model == "cubic_3orb" else workloads.layered_5orb(1)
    nbm = hop[(1, 0, 0)].shape[0]
    if complex_hop:
        extra = 0.2j * np.random.default_rng(9).standard_normal((nbm, nbm))
        hop[(1, 0, 0)] = hop[(1, 0, 0)] + extra
        hop[(-1, 0, 0)] = hop[(-1, 0, 0)] + extra.conj().T
    dims, beta, n_max, nw = (4, 4, 2), 12.0, 24, 6
    ek, g_wk, _, _ = _g_wr(hop, dims, beta, n_max)
    chi0 = T.imtime_bubble_chi0_wk(g_wk, nw=nw, verbose=False)
    ref = O.imtime_bubble_chi0_wk(O.lattice_dyson_g0_wk(0.0, ek, beta, n_max), beta, dims, nw=nw)
    assert rel_err(chi0.data, ref) < PARITY_RTOL
    nb4 = nbm ** 4
    x = chi0.data.cpu().numpy().reshape((2 * nw - 1,) + dims + (nb4,))
    mq = np.roll(x[:, ::-1, ::-1, ::-1, :], 1, axis=(1, 2, 3))  # chi0(w, -q)
    rev = _orbital_reversal(nbm)
    refl = mq[..., rev]  # chi0(w, -q)_dcba
    off = rev != np.arange(nb4)
    if complex_hop:
        assert not np.array_equal(x[..., off], refl[..., off])
    elif arithmetic != "fp64":  # the FP64 mode transforms every column
        assert np.array_equal(x[..., off], refl[..., off])
