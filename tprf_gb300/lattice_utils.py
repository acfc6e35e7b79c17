"""GB300 drop-in for ``triqs_tprf.lattice_utils.imtime_bubble_chi0_wk``.

Restates ``python/triqs_tprf/lattice_utils.py:191-269``: g_wk -> G(iv, r) ->
G(tau, r) -> bubble -> chi0(w, r) (tau -> w, or the trapezoid integral when
nw == 1) -> chi0(w, q). The whole chain runs as one C-ABI call
(``tprf_imtime_bubble_chi0_wk``); chi0(tau, r) is never stored, so the
reference's ``save_memory`` switch changes nothing here (same numbers).
"""
from __future__ import annotations

import torch

from . import _native
from ._native import check, dims3
from .gf import Gf, as_device_c128
from .lattice import _components, _stream, default_n_tau
from .mesh import MeshBrZone, MeshImFreq, MeshProduct

__all__ = ["imtime_bubble_chi0_wk", "bubble_workspace_bytes"]


def bubble_workspace_bytes(n_max: int, n_tau: int, dims, nb: int) -> int:
    return int(_native.lib().tprf_imtime_bubble_workspace_bytes(int(n_max), int(n_tau), dims3(dims), int(nb)))


def imtime_bubble_chi0_wk(g_wk, nw=1, save_memory=False, verbose=True, nt=-1, moments=None, workspace=None):
    """chi0(w, q) from G(iv, k) by the imaginary-time bubble.

    ``nt`` (time-mesh size, default 6 n_max + 1) and ``moments`` (the first
    three tail moments of G(iv, r), default: fitted) are extensions that map to
    the reference's internal defaults. ``workspace`` may be a preallocated
    uint8 CUDA tensor of at least ``bubble_workspace_bytes`` bytes.
    """
    wmesh, kmesh = _components(g_wk, (MeshImFreq, MeshBrZone), "imtime_bubble_chi0_wk")
    nb = g_wk.target_shape[0]
    n_tau = default_n_tau(wmesh.n_max) if nt is None or nt < 0 else int(nt)
    dev = g_wk.data.device
    need = bubble_workspace_bytes(wmesh.n_max, n_tau, kmesh.dims, nb)
    if workspace is None:
        workspace = torch.empty(need, dtype=torch.uint8, device=dev)
    elif workspace.numel() < need:
        raise ValueError(f"imtime_bubble_chi0_wk: workspace needs {need} bytes")
    if verbose:
        ngb = (need + (2 * nw - 1) * len(kmesh) * nb ** 4 * 16) / 1024.0 ** 3
        print(f"tprf_gb300 imtime_bubble_chi0_wk: beta={wmesh.beta} nk={kmesh.dims} nw={len(wmesh)} norb={nb} "
              f"device memory {ngb:.2f} GB")
    out = Gf(mesh=MeshProduct(MeshImFreq(wmesh.beta, "Boson", nw), kmesh), target_shape=(nb,) * 4, device=dev)
    mom = None
    if moments is not None:
        mom = as_device_c128(moments, dev)
    src = g_wk.data.contiguous()
    check(_native.lib().tprf_imtime_bubble_chi0_wk(
        wmesh.beta, wmesh.n_max, n_tau, int(nw), dims3(kmesh.dims), nb, src.data_ptr(),
        mom.data_ptr() if mom is not None else None, out.data.data_ptr(), workspace.data_ptr(), workspace.numel(),
        _stream()), "imtime_bubble_chi0_wk")
    return out


def imtime_bubble_rpa_wk(g_wk, U, nw, out=None, nt=-1, moments=None, block_freqs=None, slots=3, chi0=None,
                         workspace=None, wait=True):
    """chi(iw, q) = solve_rpa_PH(imtime_bubble_chi0_wk(g_wk, nw), U) with chi written
    to host memory (``out``: a pinned complex128 host tensor of chi's shape,
    allocated if None), the two reference calls in one: the r -> q transform,
    the RPA and the copies to the host run in blocks of ``block_freqs`` bosonic
    frequencies, the copy of one block overlapping the solve of the next, with
    ``slots`` device buffers of one block (1..32): with one per block the solves
    never wait for the call's own copies (the fastest pipeline, for a device
    ring of chi's size). ``chi0`` (device tensor of chi's shape) and
    ``workspace`` (uint8 device tensor) may be given to avoid allocations.
    Returns a host Gf.

    ``wait=False`` returns without waiting for the copies: they run on behind
    the compute, so that the next call's chain overlaps them (a pipeline over
    many inputs). ``out`` is then complete after :func:`join_host_copies` and a
    synchronisation of the current stream (a device synchronisation alone does
    not wait for the host threads that fill the negative frequencies); ``out`` and
    ``chi0`` must not be reused before, and ``workspace`` (whose ring buffers
    the copies read) must be given and held by the caller."""
    if not wait and workspace is None:
        raise ValueError("imtime_bubble_rpa_wk: wait=False needs a workspace held by the caller")
    wmesh, kmesh = _components(g_wk, (MeshImFreq, MeshBrZone), "imtime_bubble_rpa_wk")
    nb = g_wk.target_shape[0]
    nw = int(nw)
    n_tau = default_n_tau(wmesh.n_max) if nt is None or nt < 0 else int(nt)
    dev = g_wk.data.device
    lib = _native.lib()
    shape = (2 * nw - 1, len(kmesh)) + (nb,) * 4
    if block_freqs is None:
        block_freqs = max(1, -(-nw // 16))
    need = lib.tprf_imtime_bubble_rpa_to_host_workspace_bytes(wmesh.n_max, n_tau, nw, dims3(kmesh.dims), nb,
                                                              int(block_freqs), int(slots))
    if workspace is None:
        workspace = torch.empty(int(need), dtype=torch.uint8, device=dev)
    elif workspace.numel() < need:
        raise ValueError(f"imtime_bubble_rpa_wk: workspace needs {need} bytes")
    if chi0 is None:
        chi0 = torch.empty(shape, dtype=torch.complex128, device=dev)
    if out is None:
        out = torch.empty(shape, dtype=torch.complex128, pin_memory=True)
    if tuple(out.shape) != shape or out.dtype != torch.complex128 or out.device.type != "cpu" or not out.is_contiguous():
        raise ValueError("imtime_bubble_rpa_wk: out must be a contiguous complex128 host tensor of chi's shape")
    Ud = as_device_c128(U, dev)
    if tuple(Ud.shape) != (nb,) * 4:
        raise ValueError(f"imtime_bubble_rpa_wk: U must have shape {(nb,) * 4}")
    mom = as_device_c128(moments, dev) if moments is not None else None
    src = g_wk.data.contiguous()
    fn = lib.tprf_imtime_bubble_rpa_to_host if wait else lib.tprf_imtime_bubble_rpa_to_host_async
    check(fn(
        wmesh.beta, wmesh.n_max, n_tau, nw, dims3(kmesh.dims), nb, src.data_ptr(),
        mom.data_ptr() if mom is not None else None, Ud.data_ptr(), chi0.data_ptr(), out.data_ptr(), int(block_freqs),
        int(slots), workspace.data_ptr(), workspace.numel(), _stream()), "imtime_bubble_rpa_wk")
    return Gf(mesh=MeshProduct(MeshImFreq(wmesh.beta, "Boson", nw), kmesh), data=out, device=torch.device("cpu"))


def join_host_copies():
    """Make the current stream wait for every copy to host memory that
    ``imtime_bubble_rpa_wk(..., wait=False)`` has started on this device."""
    check(_native.lib().tprf_imtime_bubble_rpa_to_host_join(_stream()), "join_host_copies")

