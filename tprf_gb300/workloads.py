"""Synthetic tight-binding workloads with the shapes of the benchmark configs.

No dataset is involved: every model is a seeded tight-binding Hamiltonian.

* ``cfg0``: 1-band square lattice, t = 1, mu = 0, 16 x 16 k, beta = 10,
  n_max = 64 fermionic frequencies, nw = 64, Hubbard U = 1 (1x1x1x1 vertex).
* ``cfg1``: 3-orbital cubic lattice, nearest- and next-nearest-neighbour
  hoppings: t(R) = -I (nearest) plus N(0, 0.25^2) entries drawn from the seed,
  t(-R) = t(R)^T so e(k) is Hermitian; 32^3 k, beta = 20, n_max = 256, nw = 256,
  Kanamori spin-channel vertex U = 2.3, J = 0.4 (U' = U - 2J, J' = J), 9 x 9.
* ``cfg3``: 2-orbital square lattice, 32 x 32, beta = 16, n_max = 128, nw = 128,
  Kanamori spin-channel vertex (U = 1.2, J = 0.2, 4 x 4), 8 seeded hoppings.
* ``cfg4``: 5-orbital layered lattice (bandwidth ~4), 64 x 64 x 4, beta = 40,
  n_max = 512, Kanamori U = 3, J = 0.5 (25 x 25).
"""
from __future__ import annotations

import itertools

import numpy as np

from .rpa_tensor import kanamori_charge_and_spin_quartic_interaction_tensors

__all__ = ["square_1band", "cubic_3orb", "square_2orb", "layered_5orb", "config", "CONFIGS"]


def square_1band(t: float = 1.0):
    T = -t * np.eye(1)
    return {(0, 1): T, (0, -1): T, (1, 0): T, (-1, 0): T}


def _symmetrise(hop):
    out = {}
    for R, t in hop.items():
        out[R] = t
        out[tuple(-x for x in R)] = t.T
    return out


def cubic_3orb(seed: int = 0, sigma: float = 0.25):
    rng = np.random.default_rng(seed)
    hop = {}
    nn = [(1, 0, 0), (0, 1, 0), (0, 0, 1)]
    nnn = [(1, 1, 0), (1, -1, 0), (1, 0, 1), (1, 0, -1), (0, 1, 1), (0, 1, -1)]
    for R in nn:
        hop[R] = -np.eye(3) + sigma * rng.standard_normal((3, 3))
    for R in nnn:
        hop[R] = sigma * rng.standard_normal((3, 3))
    return _symmetrise(hop)


def square_2orb(seed: int = 0, sigma: float = 0.25):
    rng = np.random.default_rng(seed)
    hop = {}
    for R in [(1, 0), (0, 1), (1, 1), (1, -1)]:
        base = -np.eye(2) if abs(R[0]) + abs(R[1]) == 1 else np.zeros((2, 2))
        hop[R] = base + sigma * rng.standard_normal((2, 2))
    return _symmetrise(hop)


def layered_5orb(seed: int = 0):
    rng = np.random.default_rng(seed)
    hop = {}
    for R in [(1, 0, 0), (0, 1, 0), (1, 1, 0), (1, -1, 0)]:
        base = -0.5 * np.eye(5) if sum(abs(x) for x in R) == 1 else np.zeros((5, 5))
        hop[R] = base + 0.1 * rng.standard_normal((5, 5))
    hop[(0, 0, 1)] = 0.05 * rng.standard_normal((5, 5))
    out = _symmetrise(hop)
    onsite = 0.2 * rng.standard_normal((5, 5))
    out[(0, 0, 0)] = 0.5 * (onsite + onsite.T)
    return out


def kanamori_spin_vertex(norb, U, J):
    _, U_s = kanamori_charge_and_spin_quartic_interaction_tensors(norb, U, U - 2 * J, J, J)
    return U_s


CONFIGS = {
    "cfg0": dict(name="square_1band_16x16_beta10_nmax64", hop=lambda: square_1band(1.0), dims=(16, 16, 1),
                 beta=10.0, mu=0.0, n_max=64, nw=64, vertex=lambda: np.full((1, 1, 1, 1), 1.0 + 0j),
                 vertex_label="Hubbard U=1"),
    "cfg1": dict(name="cubic_3orb_32x32x32_beta20_nmax256", hop=lambda: cubic_3orb(0), dims=(32, 32, 32),
                 beta=20.0, mu=0.0, n_max=256, nw=256, vertex=lambda: kanamori_spin_vertex(3, 2.3, 0.4),
                 vertex_label="Kanamori spin channel U=2.3 J=0.4"),
    # cfg1's model on a 16 x 16 x 8 mesh: the profiling case (about 2 GB on the device)
    "cfg1_small": dict(name="cubic_3orb_16x16x8_beta20_nmax256", hop=lambda: cubic_3orb(0), dims=(16, 16, 8),
                       beta=20.0, mu=0.0, n_max=256, nw=256, vertex=lambda: kanamori_spin_vertex(3, 2.3, 0.4),
                 vertex_label="Kanamori spin channel U=2.3 J=0.4"),
    "cfg3": dict(name="square_2orb_32x32_beta16_nmax128", hop=lambda: square_2orb(0), dims=(32, 32, 1),
                 beta=16.0, mu=0.0, n_max=128, nw=128, vertex=lambda: kanamori_spin_vertex(2, 1.2, 0.2),
                 vertex_label="Kanamori spin channel U=1.2 J=0.2"),
    "cfg4": dict(name="layered_5orb_64x64x4_beta40_nmax512", hop=lambda: layered_5orb(0), dims=(64, 64, 4),
                 beta=40.0, mu=0.0, n_max=512, nw=256, vertex=lambda: kanamori_spin_vertex(5, 3.0, 0.5),
                 vertex_label="Kanamori spin channel U=3 J=0.5"),
}


def smooth7_near(x: float, lo: int, hi: int) -> int:
    """The 7-smooth integer in [lo, hi] closest to x (FFT-friendly frequency counts)."""
    cands = [n for n in range(lo, hi + 1) if _smooth7(n)]
    return min(cands, key=lambda n: (abs(n - x), n))


def _smooth7(n: int) -> bool:
    for p in (2, 3, 5, 7):
        while n % p == 0:
            n //= p
    return n == 1


def batched_instances(n: int = 512, seed: int = 0):
    """cfg2: n instances of the 1-band and 2-orbital square lattices.

    k meshes drawn from {8, 16, 24, 32, 48}^2, beta ~ U[5, 40], mu ~ U[-1, 1],
    U ~ U[0.5, 2.5] (2-orbital: Kanamori spin vertex with J = U / 10); the
    fermionic frequency count scales with beta, n_max = the 7-smooth integer
    nearest 12.8 beta in [32, 512], and nw = n_max. Returns dicts.
    """
    rng = np.random.default_rng(seed)
    two = square_2orb(0)
    out = []
    for _ in range(n):
        nb = int(rng.integers(1, 3))
        L = int(rng.choice([8, 16, 24, 32, 48]))
        beta = float(rng.uniform(5.0, 40.0))
        mu = float(rng.uniform(-1.0, 1.0))
        U = float(rng.uniform(0.5, 2.5))
        n_max = smooth7_near(12.8 * beta, 32, 512)
        hop = square_1band(1.0) if nb == 1 else two
        vertex = np.full((1, 1, 1, 1), U + 0j) if nb == 1 else kanamori_spin_vertex(2, U, U / 10)
        out.append(dict(hoppings=hop, dims=(L, L, 1), beta=beta, mu=mu, n_max=n_max, nw=n_max, U=vertex, nb=nb))
    return out


def cfg3_model(dims=(32, 32, 1), beta=16.0, n_max=128, nw=128, seed=0):
    """cfg3: the 2-orbital square lattice with 8 seeded hopping amplitudes t(R).

    Pattern a is a seeded real 2 x 2 matrix T_a on a lattice vector R_a (two
    per R in (1,0), (0,1), (1,1), (1,-1)) with its Hermitian partner on -R_a;
    theta_a multiplies it. Returns (HoppingModel, theta0 [8], U [2,2,2,2]).
    """
    from .autodiff import HoppingModel
    rng = np.random.default_rng(seed + 7)
    patterns = []
    for R in [(1, 0), (0, 1), (1, 1), (1, -1)]:
        for _ in range(2):
            T = rng.standard_normal((2, 2))
            patterns.append({R: T, tuple(-x for x in R): T.T})
    theta0 = 0.1 * rng.standard_normal(len(patterns))
    model = HoppingModel(base=square_2orb(seed), patterns=patterns, dims=dims, beta=beta, mu=0.0, n_max=n_max, nw=nw)
    return model, theta0, kanamori_spin_vertex(2, 1.2, 0.2)


def cfg3_loss(chi):
    """Re Tr chi(q = (pi, pi), i w = 0) over the PH-grouped matrix, plus sum |chi|^2."""
    nwt, nk = chi.shape[0], chi.shape[1]
    n1 = int(round(np.sqrt(nk)))
    q = (n1 // 2) * n1 + n1 // 2
    static = chi[nwt // 2, q]
    nb = chi.shape[-1]
    tr = sum(static[a, b, b, a] for a in range(nb) for b in range(nb))
    return tr.real + (chi.abs() ** 2).sum()


def config(key: str, **overrides) -> dict:
    c = dict(CONFIGS[key])
    c["hoppings"] = c.pop("hop")()
    c["U"] = c.pop("vertex")()
    c.update(overrides)
    return c
