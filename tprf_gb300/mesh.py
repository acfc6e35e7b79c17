"""Mesh descriptors with TRIQS's conventions (the parts the bubble/RPA path uses).

* ``MeshImFreq(beta, S, n_max)``: full Matsubara mesh; fermionic n = -n_max..n_max-1
  (2 n_max points), bosonic m = -(n_max-1)..n_max-1 (2 n_max - 1 points).
* ``MeshImTime(beta, S, n_tau)``: tau_i = i beta / (n_tau - 1).
* ``MeshBrZone(dims)`` / ``MeshCycLat(dims)``: periodic 3-dimensional meshes
  (unused dims = 1), linear index (i1 n2 + i2) n3 + i3.
* ``MeshProduct(*meshes)``: ``.components`` as in TRIQS.
"""
from __future__ import annotations

import math

import numpy as np

__all__ = ["MeshImFreq", "MeshImTime", "MeshBrZone", "MeshCycLat", "MeshProduct"]


def _stat(S: str) -> str:
    s = str(S).lower()
    if s.startswith("f"):
        return "Fermion"
    if s.startswith("b"):
        return "Boson"
    raise ValueError(f"statistic must be 'Fermion' or 'Boson', got {S!r}")


class MeshImFreq:
    def __init__(self, beta: float, S: str = "Fermion", n_max: int = 1025, n_iw: int | None = None):
        self.beta = float(beta)
        self.statistic = _stat(S)
        self.n_max = int(n_iw if n_iw is not None else n_max)
        if self.beta <= 0 or self.n_max < 1:
            raise ValueError("MeshImFreq needs beta > 0 and n_max >= 1")

    def __len__(self) -> int:
        return 2 * self.n_max if self.statistic == "Fermion" else 2 * self.n_max - 1

    @property
    def first_index(self) -> int:
        return -self.n_max if self.statistic == "Fermion" else -(self.n_max - 1)

    @property
    def last_index(self) -> int:
        return self.n_max - 1

    def values(self) -> np.ndarray:
        n = np.arange(self.first_index, self.last_index + 1)
        shift = 1 if self.statistic == "Fermion" else 0
        return 1j * (2 * n + shift) * np.pi / self.beta

    def __eq__(self, other):
        return (isinstance(other, MeshImFreq) and other.beta == self.beta and other.statistic == self.statistic
                and other.n_max == self.n_max)

    def __repr__(self):
        return f"MeshImFreq(beta={self.beta}, S='{self.statistic}', n_max={self.n_max})"


class MeshImTime:
    def __init__(self, beta: float, S: str = "Fermion", n_tau: int = 10001):
        self.beta = float(beta)
        self.statistic = _stat(S)
        self.n_tau = int(n_tau)
        if self.beta <= 0 or self.n_tau < 2:
            raise ValueError("MeshImTime needs beta > 0 and n_tau >= 2")

    def __len__(self) -> int:
        return self.n_tau

    def values(self) -> np.ndarray:
        return np.arange(self.n_tau) * (self.beta / (self.n_tau - 1))

    def __eq__(self, other):
        return (isinstance(other, MeshImTime) and other.beta == self.beta and other.statistic == self.statistic
                and other.n_tau == self.n_tau)

    def __repr__(self):
        return f"MeshImTime(beta={self.beta}, S='{self.statistic}', n_tau={self.n_tau})"


class _PeriodicMesh:
    kind = "periodic"

    def __init__(self, dims=None, bz=None, lattice=None, **_):
        if dims is None:
            raise ValueError(f"{type(self).__name__} needs dims")
        d = [int(x) for x in dims] + [1] * (3 - len(dims))
        if len(d) != 3 or any(x < 1 for x in d):
            raise ValueError("mesh dims must be 1 to 3 positive integers")
        self.dims = tuple(d)

    def __len__(self) -> int:
        return int(math.prod(self.dims))

    def __eq__(self, other):
        return type(other) is type(self) and other.dims == self.dims

    def __repr__(self):
        return f"{type(self).__name__}(dims={self.dims})"


class MeshBrZone(_PeriodicMesh):
    def values(self) -> np.ndarray:
        grids = np.meshgrid(*[2 * np.pi * np.arange(n) / n for n in self.dims], indexing="ij")
        return np.stack([g.ravel() for g in grids], axis=-1)


class MeshCycLat(_PeriodicMesh):
    def values(self) -> np.ndarray:
        grids = np.meshgrid(*[np.arange(n) for n in self.dims], indexing="ij")
        return np.stack([g.ravel() for g in grids], axis=-1)


class MeshProduct:
    def __init__(self, *components):
        self.components = tuple(components)

    def __len__(self) -> int:
        return int(math.prod(len(c) for c in self.components))

    def __iter__(self):
        return iter(self.components)

    def __eq__(self, other):
        return isinstance(other, MeshProduct) and other.components == self.components

    def __repr__(self):
        return "MeshProduct(" + ", ".join(map(repr, self.components)) + ")"
