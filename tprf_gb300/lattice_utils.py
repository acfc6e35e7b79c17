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
