"""A light Green's-function container: a mesh plus a complex128 CUDA tensor.

Data layout is TRIQS's: ``data.shape == mesh shape + target_shape``, C order.
The data always lives on the GPU; host arrays given to the constructor are
copied there.
"""
from __future__ import annotations

import numpy as np
import torch

from .mesh import MeshProduct

__all__ = ["Gf"]


def _mesh_shape(mesh):
    if isinstance(mesh, MeshProduct):
        return tuple(len(c) for c in mesh.components)
    return (len(mesh),)


def as_device_c128(x, device=None) -> torch.Tensor:
    """Contiguous complex128 CUDA tensor view/copy of x."""
    if isinstance(x, torch.Tensor):
        t = x
    else:
        t = torch.as_tensor(np.asarray(x))
    if device is None:
        device = t.device if t.is_cuda else torch.device("cuda", torch.cuda.current_device())
    t = t.to(device=device, dtype=torch.complex128)
    return t.contiguous()


class Gf:
    def __init__(self, mesh=None, target_shape=None, data=None, device=None):
        if mesh is None:
            raise ValueError("Gf needs a mesh")
        self.mesh = mesh
        mshape = _mesh_shape(mesh)
        if data is not None:
            t = as_device_c128(data, device)
            if tuple(t.shape[: len(mshape)]) != mshape:
                raise ValueError(f"data shape {tuple(t.shape)} does not start with mesh shape {mshape}")
            self.data = t
        else:
            if target_shape is None:
                raise ValueError("Gf needs target_shape or data")
            dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
            self.data = torch.zeros(mshape + tuple(int(s) for s in target_shape), dtype=torch.complex128, device=dev)
        self._nmesh = len(mshape)

    @property
    def target_shape(self):
        return tuple(self.data.shape[self._nmesh:])

    @property
    def target_rank(self) -> int:
        return len(self.target_shape)

    def copy(self) -> "Gf":
        return Gf(mesh=self.mesh, data=self.data.clone())

    def __repr__(self):
        return f"Gf(mesh={self.mesh!r}, target_shape={self.target_shape})"
