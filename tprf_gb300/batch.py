"""Batched bubble + RPA over many independent instances in one graph launch.

The reference computes instances one at a time (a Python loop over
``lattice_dyson_g0_wk``, ``imtime_bubble_chi0_wk`` and ``solve_rpa_PH``).
``BatchedRPA`` takes the whole list (each with its own beta, mu, k mesh,
frequency counts, orbital count and vertex), plans it once and runs every
instance with one CUDA-graph launch (C ABI ``tprf_batch_*``).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native
from ._native import Instance, check

__all__ = ["RPAInstance", "BatchedRPA"]


@dataclass
class RPAInstance:
    """One instance: e(k) [N_k, nb, nb] on dims, vertex U [nb]^4, meshes."""
    e_k: torch.Tensor
    U: np.ndarray
    dims: tuple
    beta: float
    mu: float
    n_max: int
    nw: int
    n_tau: int = -1
    chi: torch.Tensor = field(default=None, repr=False)

    @property
    def nb(self) -> int:
        return int(self.e_k.shape[-1])

    @property
    def points(self) -> int:
        return (2 * self.nw - 1) * int(np.prod(self.dims))


class BatchedRPA:
    """chi(iw, q) of every instance from one graph launch.

    ``run()`` recomputes all instances (their e_k / U tensors may be updated
    in place between runs); results are in ``instances[i].chi`` with shape
    (2 nw - 1, N_k, nb, nb, nb, nb).
    """

    def __init__(self, instances, n_streams: int = 32, device=None):
        self.lib = _native.lib()
        dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.instances = list(instances)
        self._keep = []
        arr = (Instance * len(self.instances))()
        for i, a in enumerate(self.instances):
            a.e_k = a.e_k.to(dev, torch.complex128).contiguous()
            u = torch.as_tensor(np.asarray(a.U), dtype=torch.complex128).to(dev).contiguous()
            nk = int(np.prod(a.dims))
            if a.chi is None:
                a.chi = torch.empty((2 * a.nw - 1, nk) + (a.nb,) * 4, dtype=torch.complex128, device=dev)
            self._keep += [a.e_k, u, a.chi]
            d = list(a.dims) + [1] * (3 - len(a.dims))
            arr[i] = Instance(float(a.beta), float(a.mu), int(a.n_max), int(a.n_tau), int(a.nw), a.nb,
                              (ctypes.c_int * 3)(*d), a.e_k.data_ptr(), u.data_ptr(), a.chi.data_ptr())
        self._arr = arr
        need = self.lib.tprf_batch_workspace_bytes(arr, len(arr), n_streams)
        self.workspace = torch.empty(int(need), dtype=torch.uint8, device=dev)
        handle = ctypes.c_void_p()
        check(self.lib.tprf_batch_create(arr, len(arr), n_streams, self.workspace.data_ptr(), self.workspace.numel(),
                                         ctypes.byref(handle)), "batch_create")
        self.handle = handle

    @property
    def points(self) -> int:
        return sum(a.points for a in self.instances)

    def run(self, stream=None):
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(self.lib.tprf_batch_run(self.handle, s), "batch_run")

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.lib.tprf_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
