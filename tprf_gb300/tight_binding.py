"""Tight-binding dispersions e(k) on a brzone mesh, computed on the GPU.

``e(k) = sum_R t(R) exp(i k.R)`` as TRIQS's ``TBLattice.fourier`` gives it
(used through ``python/triqs_tprf/tight_binding.py:27``), with
``k_i = 2 pi i / n`` on the mesh dims. ``create_square_lattice`` restates
``tight_binding.py:31-97``.
"""
from __future__ import annotations

import numpy as np
import torch

from .gf import Gf
from .mesh import MeshBrZone

__all__ = ["TBLattice", "create_square_lattice", "ek_tensor"]


def ek_tensor(hoppings: dict, dims, device=None) -> torch.Tensor:
    """[N_k, nb, nb] complex128 CUDA tensor of e(k) for hoppings {R: t(R)}."""
    dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    d = [int(x) for x in dims] + [1] * (3 - len(dims))
    grids = torch.meshgrid(*[2 * np.pi * torch.arange(n, dtype=torch.float64, device=dev) / n for n in d],
                           indexing="ij")
    k = torch.stack([g.reshape(-1) for g in grids], dim=-1)
    Rs = list(hoppings.keys())
    R = torch.zeros(len(Rs), 3, dtype=torch.float64, device=dev)
    for i, r in enumerate(Rs):
        R[i, : len(r)] = torch.tensor([float(x) for x in r], dtype=torch.float64)
    T = torch.stack([torch.as_tensor(np.asarray(hoppings[r]), dtype=torch.complex128) for r in Rs]).to(dev)
    phase = torch.exp(1j * (k @ R.T))  # [N_k, n_R]
    return torch.einsum("kr,rab->kab", phase, T).contiguous()


class TBLattice:
    """Minimal tight-binding lattice: hoppings {R: t(R) (nb x nb)}."""

    def __init__(self, units=None, hopping=None, orbital_positions=None, orbital_names=None):
        self.units = units
        self.hopping = {tuple(k): np.asarray(v, dtype=complex) for k, v in (hopping or {}).items()}
        self.n_orbitals = next(iter(self.hopping.values())).shape[0]

    def get_kmesh(self, n_k):
        return MeshBrZone(dims=n_k)

    def fourier(self, kmesh):
        return Gf(mesh=kmesh, data=ek_tensor(self.hopping, kmesh.dims))


def create_square_lattice(norb, t, tp=0.0, zeeman=0.0, spin=False, **kwargs):
    if zeeman != 0.0 and not spin:
        raise AttributeError("There can not be a Zeeman term in a spinless model.")
    if spin:
        norb *= 2
    t_m = -t * np.eye(norb)
    tp_m = -tp * np.eye(norb)
    z_m = zeeman * np.diag([(-1) ** o for o in range(norb)])
    hopping = {(0, 0): z_m, (0, 1): t_m, (0, -1): t_m, (1, 0): t_m, (-1, 0): t_m,
               (1, 1): tp_m, (-1, -1): tp_m, (1, -1): tp_m, (-1, 1): tp_m}
    return TBLattice([(1, 0, 0), (0, 1, 0)], hopping, [(0, 0, 0)] * norb)
