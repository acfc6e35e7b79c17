"""Parity at the benchmark configurations' own frequency meshes (``-m gpu``).

The parity tests elsewhere keep n_max <= 64; these run the benched kernels at
the benched time and frequency meshes, on k meshes small enough for the
oracle:

* the 3-orbital cubic model with the 9 x 9 Kanamori vertex (U = 2.3, J = 0.4)
  at beta = 20, n_max = nw = 256 (FFT length L = 1536), on a 4 x 4 x 4 mesh;
* the 5-orbital layered model with a 25 x 25 Kanamori vertex at beta = 40,
  n_max = 512, nw = 256 (L = 3072), on a 4 x 2 x 2 mesh: with U = 1.5, J = 0.25
  end to end, and with the benchmark's U = 3, J = 0.5, which puts this small
  mesh near an instability, step by step;
* three instances of the 512-instance batch with its largest frequency mesh
  (beta = 40, n_max = nw = 512): a 1-band 48 x 48 and a 2-orbital 32 x 32
  model, and the seeded batch's own largest 2-orbital instance, through the
  batched graph;
* hoppings with a genuine imaginary part around the real-input threshold of
  the bubble chain (max |Im G(tau, r)| <= 1e-11 max |G|).

Each compares chi (and chi0) with the oracle at PARITY_RTOL, in the default
arithmetic and in native FP64.
"""
import numpy as np
import pytest
import torch

import oracle as O
from conftest import PARITY_RTOL, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["df64", "fp64"])
def arithmetic(request, cuda_lib):
    mode = {"df64": 0, "fp64": 1}[request.param]
    assert cuda_lib.tprf_set_arithmetic(mode) == 0
    yield request.param
    cuda_lib.tprf_set_arithmetic(0)


def _chain_and_rpa(hop, dims, beta, n_max, nw, U):
    """chi0 and chi through the public API (two calls and the fused call) and the oracle's."""
    import tprf_gb300 as T
    from tprf_gb300.lattice_utils import imtime_bubble_rpa_wk
    ek = O.ek_from_hoppings(hop, dims)
    e_k = T.Gf(mesh=T.MeshBrZone(dims=dims), data=ek)
    g0 = T.lattice_dyson_g0_wk(0.0, e_k, T.MeshImFreq(beta, "Fermion", n_max))
    chi0 = T.imtime_bubble_chi0_wk(g0, nw=nw, verbose=False)
    chi = T.solve_rpa_PH(chi0, U)
    fused = imtime_bubble_rpa_wk(g0, U, nw)
    torch.cuda.synchronize()
    ref0 = O.imtime_bubble_chi0_wk(O.lattice_dyson_g0_wk(0.0, ek, beta, n_max), beta, dims, nw=nw)
    ref = O.solve_rpa_PH(ref0, U)
    return chi0, chi, fused, ref0, ref


def test_cubic_3orb_at_the_benchmark_meshes(cuda_lib, arithmetic):
    """beta = 20, n_max = nw = 256, n_tau = 1537 (L = 1536), 9 x 9 Kanamori vertex."""
    from tprf_gb300 import workloads
    U = workloads.kanamori_spin_vertex(3, 2.3, 0.4)
    chi0, chi, fused, ref0, ref = _chain_and_rpa(workloads.cubic_3orb(0), (4, 4, 4), 20.0, 256, 256, U)
    assert tuple(chi.data.shape) == ref.shape == (511, 64, 3, 3, 3, 3)
    assert rel_err(chi0.data, ref0) < PARITY_RTOL
    assert rel_err(chi.data, ref) < PARITY_RTOL
    assert torch.equal(fused.data, chi.data.cpu())


def test_layered_5orb_at_the_benchmark_meshes(cuda_lib, arithmetic):
    """beta = 40, n_max = 512, nw = 256, n_tau = 3073 (L = 3072), 25 x 25 Kanamori
    vertex (the compiled 25 x 25 RPA group kernel) with U = 1.5, J = 0.25, where
    1 - chi0 U stays well conditioned (cond <= 48) on this small mesh."""
    from tprf_gb300 import workloads
    U = workloads.kanamori_spin_vertex(5, 1.5, 0.25)
    chi0, chi, fused, ref0, ref = _chain_and_rpa(workloads.layered_5orb(0), (4, 2, 2), 40.0, 512, 256, U)
    assert tuple(chi.data.shape) == ref.shape == (511, 16) + (5,) * 4
    assert rel_err(chi0.data, ref0) < PARITY_RTOL
    assert rel_err(chi.data, ref) < PARITY_RTOL
    assert torch.equal(fused.data, chi.data.cpu())


def test_layered_5orb_benchmark_vertex_near_instability(cuda_lib, arithmetic):
    """The benchmark's own vertex (U = 3, J = 0.5) on the 4 x 2 x 2 mesh puts
    1 - chi0 U near a magnetic instability: cond up to ~5e3, max |chi| ~ 500
    max |chi0|. There any two FP64 computations of chi differ by about cond times
    their chi0 difference (the numerical differentiation in fit_derivatives leaves
    ~2e-14 between this path and the oracle, in native FP64 as in double-float).
    Each step meets the bar on its own: chi0 against the oracle, and the RPA
    solve on the oracle's chi0 against the oracle's chi (the conditioning-
    triggered FP64 re-solve at work); the chain's chi stays within the
    first-order bound 2 cond_max err(chi0)."""
    import tprf_gb300 as T
    from tprf_gb300 import workloads
    U = workloads.kanamori_spin_vertex(5, 3.0, 0.5)
    chi0, chi, fused, ref0, ref = _chain_and_rpa(workloads.layered_5orb(0), (4, 2, 2), 40.0, 512, 256, U)
    grp = lambda x: np.swapaxes(x, -1, -2).reshape(x.shape[:-4] + (25, 25))  # noqa: E731
    cond = np.linalg.cond((np.eye(25) - grp(ref0) @ grp(U)).reshape(-1, 25, 25)).max()
    assert cond > 1e3 and np.abs(ref).max() > 100 * np.abs(ref0).max()  # the instability is really there
    e0 = rel_err(chi0.data, ref0)
    assert e0 < PARITY_RTOL
    on_exact = T.solve_rpa_PH(T.Gf(mesh=chi0.mesh, data=ref0), U)
    assert rel_err(on_exact.data, ref) < PARITY_RTOL
    assert rel_err(chi.data, ref) < 2.0 * cond * e0
    assert torch.equal(fused.data, chi.data.cpu())


def _largest_batch_instances():
    """Three instances with the batch's largest frequency mesh (beta = 40 gives
    n_max = nw = 512 under its rule n_max = 7-smooth nearest 12.8 beta in [32, 512])."""
    from tprf_gb300 import workloads
    specs = workloads.batched_instances(512, seed=0)
    two = max((d for d in specs if d["nb"] == 2), key=lambda d: (d["n_max"], d["dims"][0]))
    one = dict(hoppings=workloads.square_1band(1.0), dims=(48, 48, 1), beta=40.0, mu=0.3,
               n_max=workloads.smooth7_near(12.8 * 40.0, 32, 512), U=np.full((1, 1, 1, 1), 1.5 + 0j), nb=1)
    one["nw"] = one["n_max"]
    orb2 = dict(hoppings=workloads.square_2orb(0), dims=(32, 32, 1), beta=40.0, mu=-0.4, n_max=one["n_max"],
                nw=one["n_max"], U=workloads.kanamori_spin_vertex(2, 2.0, 0.2), nb=2)
    assert one["n_max"] == 512
    return [one, orb2, two]


def test_batch_instances_at_the_largest_meshes(cuda_lib, arithmetic):
    """The batched graph on uncapped instances: each chi equals the
    single-instance path bit for bit and the oracle to the parity bar."""
    import tprf_gb300 as T
    from tprf_gb300.batch import BatchedRPA, RPAInstance
    from tprf_gb300.tight_binding import ek_tensor
    specs = _largest_batch_instances()
    insts = [RPAInstance(e_k=ek_tensor(d["hoppings"], d["dims"]), U=d["U"], dims=d["dims"], beta=d["beta"],
                         mu=d["mu"], n_max=d["n_max"], nw=d["nw"]) for d in specs]
    batch = BatchedRPA(insts, n_streams=3)
    batch.run()
    torch.cuda.synchronize()
    for a, d in zip(batch.instances, specs):
        e_k = T.Gf(mesh=T.MeshBrZone(dims=d["dims"]), data=a.e_k)
        g0 = T.lattice_dyson_g0_wk(d["mu"], e_k, T.MeshImFreq(d["beta"], "Fermion", d["n_max"]))
        single = T.solve_rpa_PH(T.imtime_bubble_chi0_wk(g0, nw=d["nw"], verbose=False), d["U"])
        assert torch.equal(single.data, a.chi)
        ek = O.ek_from_hoppings(d["hoppings"], d["dims"])
        ref0 = O.imtime_bubble_chi0_wk(O.lattice_dyson_g0_wk(d["mu"], ek, d["beta"], d["n_max"]), d["beta"],
                                       d["dims"], nw=d["nw"])
        assert rel_err(a.chi, O.solve_rpa_PH(ref0, d["U"])) < PARITY_RTOL
    batch.close()


def _near_real_model(eps):
    """Two bands on a square lattice, hoppings real up to i eps A(R) (Hermitian:
    t(-R) = t(R)^dagger), so G(tau, r) has a genuine imaginary part of about eps."""
    rng = np.random.default_rng(0)
    hop = {}
    for R, base in [((1, 0), np.array([[-1.0, 0.2], [0.2, -0.8]])), ((0, 1), np.array([[-0.6, 0.1], [0.1, -1.0]]))]:
        t = base + 1j * eps * rng.standard_normal((2, 2))
        hop[R] = t
        hop[(-R[0], -R[1])] = t.conj().T
    return hop


@pytest.mark.parametrize("eps,real_path", [(0.0, True), (3e-12, True), (6e-12, True), (1e-11, None),
                                           (3e-11, False), (1e-9, False)])
def test_real_bubble_threshold(cuda_lib, arithmetic, eps, real_path):
    """Around the bubble chain's real-input cut (max |Im G(tau, r)| <= 1e-11
    max |G|): below it the imaginary parts are dropped and the negative
    frequencies filled by chi(-w, q) = conj(chi(w, -q)), which costs about the
    ratio itself in chi (~6e-12 at the cut); above it the complex path runs.
    Either way chi meets the parity bar. real_path: which path the double-float
    chain must take (None at the cut itself, where rounding decides), as the
    fused call's record says. The FP64 mode always takes the complex path."""
    import ctypes
    from tprf_gb300 import _native
    dims, beta, n_max, nw = (6, 6, 1), 8.0, 40, 6
    U = (0.5 * np.eye(4)).reshape(2, 2, 2, 2) + 0j
    chi0, chi, fused, ref0, ref = _chain_and_rpa(_near_real_model(eps), dims, beta, n_max, nw, U)
    assert rel_err(chi0.data, ref0) < PARITY_RTOL
    assert rel_err(chi.data, ref) < PARITY_RTOL
    assert rel_err(fused.data, ref) < PARITY_RTOL
    st = (ctypes.c_double * 10)()
    _native.check(_native.lib().tprf_imtime_bubble_rpa_to_host_last_stats(st, 10))
    took_real = bool(st[8])
    if arithmetic == "fp64":
        assert not took_real
    elif real_path is not None:
        assert took_real == real_path


def _scaled_non_hermitian_g0(scale, dims, beta, n_max, nb=2, seed=7):
    """G0(iv, k) of a random non-Hermitian e(k) (so G(-iv) != G(iv)^dagger and the
    real-input words must say no), times `scale`: on the device and in the oracle."""
    import tprf_gb300 as T
    rng = np.random.default_rng(seed)
    nk = int(np.prod(dims))
    ek = rng.standard_normal((nk, nb, nb)) + 1j * rng.standard_normal((nk, nb, nb))
    g0 = T.lattice_dyson_g0_wk(0.0, T.Gf(mesh=T.MeshBrZone(dims=dims), data=ek), T.MeshImFreq(beta, "Fermion", n_max))
    g0.data.mul_(scale)
    return g0, scale * O.lattice_dyson_g0_wk(0.0, ek, beta, n_max)


@pytest.mark.parametrize("scale", [1e-12, 1e8])
def test_scaled_non_hermitian_g_takes_the_complex_path(cuda_lib, arithmetic, scale):
    """Far from 1 but inside the double-float range: the decision words compare
    magnitudes (no squares to overflow or underflow), send the non-Hermitian G down
    the complex path, and chi0 meets the parity bar."""
    import tprf_gb300 as T
    dims, beta, n_max, nw = (4, 4, 1), 6.0, 32, 4
    cuda_lib.tprf_set_sync_checks(1)
    g0, ref_g = _scaled_non_hermitian_g0(scale, dims, beta, n_max)
    chi0 = T.imtime_bubble_chi0_wk(g0, nw=nw, verbose=False)
    ref0 = O.imtime_bubble_chi0_wk(ref_g, beta, dims, nw=nw)
    assert rel_err(chi0.data, ref0) < PARITY_RTOL


@pytest.mark.parametrize("scale", [1e-25, 1e25])
def test_chain_outside_the_double_float_range_is_reported(cuda_lib, scale):
    """max |G| beyond [1e-15, 1e15]: the double-float chain (FP32 exponent range)
    reports TPRF_ERR_RANGE and names the FP64 mode instead of returning a chi0
    whose products overflowed or lost their low words; the FP64 mode computes it
    (shown at 1e-25, where the absolute tail-fit residual stays small)."""
    import tprf_gb300 as T
    from tprf_gb300._native import TprfError
    dims, beta, n_max, nw = (4, 4, 1), 6.0, 32, 4
    cuda_lib.tprf_set_sync_checks(1)
    assert cuda_lib.tprf_set_arithmetic(0) == 0
    g0, ref_g = _scaled_non_hermitian_g0(scale, dims, beta, n_max)
    with pytest.raises(TprfError) as err:
        T.imtime_bubble_chi0_wk(g0, nw=nw, verbose=False)
    assert err.value.status == -9 and "TPRF_ARITH_FP64" in str(err.value)
    if scale < 1:
        assert cuda_lib.tprf_set_arithmetic(1) == 0
        try:
            chi0 = T.imtime_bubble_chi0_wk(g0, nw=nw, verbose=False)
        finally:
            cuda_lib.tprf_set_arithmetic(0)
        assert rel_err(chi0.data, O.imtime_bubble_chi0_wk(ref_g, beta, dims, nw=nw)) < PARITY_RTOL
