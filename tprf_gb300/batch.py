"""Batched bubble + RPA over many independent instances in one graph launch.

The reference computes instances one at a time (a Python loop over
``lattice_dyson_g0_wk``, ``imtime_bubble_chi0_wk`` and ``solve_rpa_PH``).
``BatchedRPA`` takes the whole list (each with its own beta, mu, k mesh,
frequency counts, orbital count and vertex), plans it once and runs every
instance with one CUDA-graph launch (C ABI ``tprf_batch_*``).
``BatchedRPAGrad`` is the differentiable form: a forward graph that also keeps
chi0, and a backward graph that runs every instance's hand-written adjoint
chain, giving the gradients with respect to U, e(k) and the hoppings t(R).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native
from ._native import GradInstance, Instance, check

__all__ = ["RPAInstance", "BatchedRPA", "BatchedRPAGrad", "batched_chi_rpa"]


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


def _instance_struct(a, u):
    d = list(a.dims) + [1] * (3 - len(a.dims))
    return Instance(float(a.beta), float(a.mu), int(a.n_max), int(a.n_tau), int(a.nw), a.nb, (ctypes.c_int * 3)(*d),
                    a.e_k.data_ptr(), u.data_ptr(), a.chi.data_ptr())


class BatchedRPAGrad:
    """chi(iw, q) of every instance and its gradients, one graph launch each way.

    ``forward()`` computes chi of every instance into views of one flat buffer
    (``chi_flat``; ``instances[i].chi`` is the view) and keeps chi0.
    ``backward(chi_grad=None)`` reads dL/d conj(chi) from ``chi_grad_flat`` (or
    copies the given flat tensor there) and writes, per instance i,
    ``U_grad[i]`` [nb]^4, ``e_grad[i]`` [N_k, nb, nb] and ``t_grad[i]``
    [N_k, nb, nb]: the gradient with respect to t(R) for every lattice vector R
    of the periodic mesh (row-major R index, as the k index), for
    e(k) = sum_R t(R) exp(i k.R). Gradients follow torch's conjugate-Wirtinger
    convention. e_k and U may be updated in place between runs.
    """

    def __init__(self, instances, n_streams: int = 32, device=None):
        self.lib = _native.lib()
        dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.instances = list(instances)
        n = len(self.instances)
        for a in self.instances:
            a.e_k = a.e_k.to(dev, torch.complex128).contiguous()
        self.U = [torch.as_tensor(np.asarray(a.U), dtype=torch.complex128).to(dev).contiguous()
                  for a in self.instances]
        chi_sizes = [a.points * a.nb ** 4 for a in self.instances]
        ek_sizes = [int(np.prod(a.dims)) * a.nb ** 2 for a in self.instances]
        u_sizes = [a.nb ** 4 for a in self.instances]
        c128 = dict(dtype=torch.complex128, device=dev)
        self.chi_flat = torch.empty(sum(chi_sizes), **c128)
        self.chi0_flat = torch.empty(sum(chi_sizes), **c128)
        self.chi_grad_flat = torch.zeros(sum(chi_sizes), **c128)
        self.U_grad_flat = torch.zeros(sum(u_sizes), **c128)
        self.e_grad_flat = torch.zeros(sum(ek_sizes), **c128)
        self.t_grad_flat = torch.zeros(sum(ek_sizes), **c128)

        def views(flat, sizes, shapes):
            out, off = [], 0
            for sz, sh in zip(sizes, shapes):
                out.append(flat[off:off + sz].view(sh))
                off += sz
            return out

        chi_shapes = [(2 * a.nw - 1, int(np.prod(a.dims))) + (a.nb,) * 4 for a in self.instances]
        ek_shapes = [(int(np.prod(a.dims)), a.nb, a.nb) for a in self.instances]
        for a, v in zip(self.instances, views(self.chi_flat, chi_sizes, chi_shapes)):
            a.chi = v
        self.chi0 = views(self.chi0_flat, chi_sizes, chi_shapes)
        self.chi_grad = views(self.chi_grad_flat, chi_sizes, chi_shapes)
        self.U_grad = views(self.U_grad_flat, u_sizes, [(a.nb,) * 4 for a in self.instances])
        self.e_grad = views(self.e_grad_flat, ek_sizes, ek_shapes)
        self.t_grad = views(self.t_grad_flat, ek_sizes, ek_shapes)
        arr = (GradInstance * n)()
        for i, a in enumerate(self.instances):
            arr[i] = GradInstance(_instance_struct(a, self.U[i]), self.chi0[i].data_ptr(), self.chi_grad[i].data_ptr(),
                                  self.U_grad[i].data_ptr(), self.e_grad[i].data_ptr(), self.t_grad[i].data_ptr())
        self._arr = arr
        need = self.lib.tprf_batch_grad_workspace_bytes(arr, n, n_streams)
        self.workspace = torch.empty(int(need), dtype=torch.uint8, device=dev)
        handle = ctypes.c_void_p()
        check(self.lib.tprf_batch_grad_create(arr, n, n_streams, self.workspace.data_ptr(), self.workspace.numel(),
                                              ctypes.byref(handle)), "batch_grad_create")
        self.handle = handle

    @property
    def points(self) -> int:
        return sum(a.points for a in self.instances)

    def forward(self, stream=None):
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(self.lib.tprf_batch_run(self.handle, s), "batch_run")
        return self.chi_flat

    def backward(self, chi_grad=None, stream=None):
        if chi_grad is not None:
            self.chi_grad_flat.copy_(chi_grad.reshape(-1))
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(self.lib.tprf_batch_backward(self.handle, s), "batch_backward")

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.lib.tprf_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _BatchedChiRPA(torch.autograd.Function):
    @staticmethod
    def forward(ctx, batch, *eu):
        n = len(batch.instances)
        with torch.no_grad():
            for a, e in zip(batch.instances, eu[:n]):
                a.e_k.copy_(e)
            for u_dst, u in zip(batch.U, eu[n:]):
                u_dst.copy_(u)
        ctx.batch = batch
        return batch.forward()

    @staticmethod
    def backward(ctx, chi_grad):
        b = ctx.batch
        b.backward(chi_grad)
        return (None, *[g.clone() for g in b.e_grad], *[g.clone() for g in b.U_grad])


def batched_chi_rpa(batch: BatchedRPAGrad, e_ks, Us):
    """Flat chi of every instance of ``batch`` (``batch.instances[i].chi`` views it),
    differentiable in the e(k) tensors and vertices ``Us`` through the batched
    adjoint graph. The result is the batch's own buffer: the next call overwrites it."""
    return _BatchedChiRPA.apply(batch, *e_ks, *Us)
