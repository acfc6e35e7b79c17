"""Host checks of the synthetic workloads the benchmark runs (no GPU).

The benchmark configs are seeded tight-binding models with the shapes of the
reference's benchmark cases; these tests pin what they contain: Hermitian
dispersions, the vertex shapes, the 5-orbital bandwidth, and the batched
instances' ranges, frequency counts and determinism.
"""
import numpy as np
import pytest

import oracle as O
from tprf_gb300 import workloads as W


def _is_smooth7(n):
    for p in (2, 3, 5, 7):
        while n % p == 0:
            n //= p
    return n == 1


@pytest.mark.parametrize("key", ["cfg0", "cfg1", "cfg3", "cfg4"])
def test_models_give_hermitian_dispersions(key):
    c = W.config(key)
    for R, t in c["hoppings"].items():
        back = c["hoppings"][tuple(-x for x in R)]
        assert np.array_equal(np.asarray(back), np.asarray(t).T)  # real t(R): t(-R) = t(R)^T
    small = tuple(min(d, 6) for d in c["dims"])
    ek = O.ek_from_hoppings(c["hoppings"], small)
    assert np.abs(ek - np.conj(np.transpose(ek, (0, 2, 1)))).max() < 1e-14


@pytest.mark.parametrize("key,nb", [("cfg0", 1), ("cfg1", 3), ("cfg3", 2), ("cfg4", 5)])
def test_vertex_shapes(key, nb):
    c = W.config(key)
    U = np.asarray(c["U"])
    assert U.shape == (nb,) * 4
    assert np.all(U.imag == 0)
    assert next(iter(c["hoppings"].values())).shape == (nb, nb)


def test_layered_5orb_bandwidth_is_about_four():
    """Each of the five bands is about 4 wide (nearest-neighbour -0.5 in the plane)."""
    c = W.config("cfg4")
    ek = O.ek_from_hoppings(c["hoppings"], (32, 32, 4))
    ev = np.linalg.eigvalsh(ek)  # [N_k, 5], ascending per k
    widths = ev.max(axis=0) - ev.min(axis=0)
    assert np.all((widths > 3.0) & (widths < 5.0))


def test_smooth7_near():
    assert W.smooth7_near(12.8 * 5.0, 32, 512) == 64
    assert W.smooth7_near(12.8 * 40.0, 32, 512) == 512
    assert W.smooth7_near(1.0, 32, 512) == 32
    for x in (100.3, 257.9, 333.0):
        n = W.smooth7_near(x, 32, 512)
        assert _is_smooth7(n)
        assert all(abs(m - x) >= abs(n - x) for m in range(32, 513) if _is_smooth7(m))


def test_batched_instances_follow_the_spec():
    a = W.batched_instances(512, seed=0)
    b = W.batched_instances(512, seed=0)
    assert len(a) == 512
    nbs = set()
    for x, y in zip(a, b):
        assert x["dims"] == y["dims"] and x["beta"] == y["beta"] and x["mu"] == y["mu"]
        assert np.array_equal(x["U"], y["U"])
        L0, L1, L2 = x["dims"]
        assert L0 == L1 and L0 in (8, 16, 24, 32, 48) and L2 == 1
        assert 5.0 <= x["beta"] <= 40.0 and -1.0 <= x["mu"] <= 1.0
        assert x["nw"] == x["n_max"] and 32 <= x["n_max"] <= 512 and _is_smooth7(x["n_max"])
        assert x["n_max"] == W.smooth7_near(12.8 * x["beta"], 32, 512)
        assert np.asarray(x["U"]).shape == (x["nb"],) * 4
        if x["nb"] == 1:
            assert 0.5 <= float(np.asarray(x["U"]).real.ravel()[0]) <= 2.5
        nbs.add(x["nb"])
    assert nbs == {1, 2}
    assert W.batched_instances(8, seed=1)[0]["beta"] != a[0]["beta"]


def test_vertex_builders_equal_the_oracle_restatement():
    """tprf_gb300.rpa_tensor (delta-tensor form) gives the oracle's Kanamori tensors
    (a loop restatement of python/triqs_tprf/rpa_tensor.py:87-233) exactly."""
    import oracle as O
    from tprf_gb300 import rpa_tensor as R
    for norb, pars in [(1, (2.3, 1.5, 0.4, 0.4)), (2, (1.0, 0.8, 0.1, 0.1)), (3, (2.3, 1.5, 0.4, 0.3)),
                       (5, (3.0, 2.0, 0.5, 0.5))]:
        for a, b in zip(R.kanamori_charge_and_spin_quartic_interaction_tensors(norb, *pars),
                        O.kanamori_charge_and_spin_quartic_interaction_tensors(norb, *pars)):
            assert np.array_equal(a, b)
        assert np.array_equal(R.kanamori_quartic_tensor(norb, *pars), O.kanamori_quartic_tensor(norb, *pars))


def test_bench_models_the_compact_orbital_columns():
    """bench.py's algorithmic bytes follow the library's compact r -> q path: the
    45 canonical orbital columns abcd <= dcba of a 3-orbital bubble on a 3-d mesh
    whose last two axes are powers of two, none on a 2-d mesh or where the compact
    rows would not fit the free rows of G(tau, r)."""
    import bench
    assert bench.compact_columns((32, 32, 32), 3, 1537, 256) == 45
    assert bench.compact_columns((16, 16, 8), 3, 1537, 256) == 45
    assert bench.compact_columns((64, 64, 4), 5, 3073, 256) is None  # 256 x 325 > 3055 x 25
    assert bench.compact_columns((48, 48, 1), 2, 1537, 256) is None
    assert bench.compact_columns((32, 32, 32), 3, 1537, 256, real=False) is None
    m = bench.stage_model(3, 32768, 512, 1537, 256, real=True, nc=45)
    assert m["fft_r_to_q"]["bytes"] == 16 * 32768 * (45 * 256 + 81 * 511)
