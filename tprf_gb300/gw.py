"""GB300 drop-in for the GW consumers of the bubble chain.

Same names and argument meaning as ``triqs_tprf.gw`` / ``triqs_tprf.lattice``:
``bubble_PI_wk`` (python/triqs_tprf/gw.py:56-91), ``dynamical_screened_interaction_W``
(lattice/dynamical_screened_interaction.cpp:30-124) and ``gw_dynamic_sigma``
(lattice/gw.cpp:66-84). Every call goes through the C ABI of the CUDA library.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native
from ._native import check
from .gf import Gf, as_device_c128
from .lattice import _components, _ntarget, _stream
from .lattice_utils import imtime_bubble_chi0_wk
from .mesh import MeshBrZone, MeshCycLat, MeshImFreq, MeshImTime, MeshProduct

__all__ = ["bubble_PI_wk", "dynamical_screened_interaction_W", "gw_dynamic_sigma"]


def bubble_PI_wk(g_wk, workspace=None):
    """PI_abcd(iw, k) = - F{G_da(tau, r) G_bc(-tau, -r)} with nw = n_max bosonic
    frequencies: the imaginary-time bubble chain (gw.py:56-91)."""
    wmesh, _ = _components(g_wk, (MeshImFreq, MeshBrZone), "bubble_PI_wk")
    return imtime_bubble_chi0_wk(g_wk, nw=wmesh.n_max, verbose=False, workspace=workspace)


def dynamical_screened_interaction_W(PI_wk, V_k):
    """W(iw, k) from the bubble PI(iw, k) and a static V(k) (a Gf on the same
    MeshBrZone) or a dynamic V(iw, k) (a Gf on PI's mesh)."""
    wmesh, kmesh = _components(PI_wk, (MeshImFreq, MeshBrZone), "dynamical_screened_interaction_W")
    nb = PI_wk.target_shape[0]
    if not isinstance(V_k, Gf) or tuple(V_k.target_shape) != (nb,) * 4:
        raise TypeError("dynamical_screened_interaction_W: V must be a rank-4 Gf with PI's target shape")
    if isinstance(V_k.mesh, MeshBrZone):
        if V_k.mesh.dims != kmesh.dims:
            raise RuntimeError("dynamical_screened_interaction_W: k-space meshes are not the same")
        kind = 0
    else:
        _, vk = _components(V_k, (MeshImFreq, MeshBrZone), "dynamical_screened_interaction_W")
        if vk.dims != kmesh.dims or V_k.data.shape[0] != PI_wk.data.shape[0]:
            raise RuntimeError("dynamical_screened_interaction_W: meshes are not the same")
        kind = 1
    dev = PI_wk.data.device
    out = Gf(mesh=PI_wk.mesh, data=torch.empty_like(PI_wk.data))
    pi = PI_wk.data.contiguous()
    v = as_device_c128(V_k.data, dev)
    check(_native.lib().tprf_dynamical_screened_interaction_W(len(wmesh), len(kmesh), nb, pi.data_ptr(), v.data_ptr(),
                                                               kind, out.data.data_ptr(), _stream()),
          "dynamical_screened_interaction_W")
    return out


def gw_dynamic_sigma(W_tr, g_tr):
    """sigma_ab(tau, r) = - sum_cd W_acdb(tau, r) G_cd(tau, r) (gw.cpp:66-84)."""
    wt, wr = _components(W_tr, (MeshImTime, MeshCycLat), "gw_dynamic_sigma")
    gt, gr = _components(g_tr, (MeshImTime, MeshCycLat), "gw_dynamic_sigma")
    if wt.n_tau != gt.n_tau or wt.beta != gt.beta:
        raise RuntimeError("gw_sigma_tr: tau meshes are not the same.")
    if wt.statistic != "Boson" or gt.statistic != "Fermion":
        raise RuntimeError("gw_sigma_tr: statistics are incorrect.")
    if wr.dims != gr.dims:
        raise RuntimeError("gw_sigma_tr: real-space meshes are not the same.")
    nb = g_tr.target_shape[0]
    out = Gf(mesh=g_tr.mesh, data=torch.empty_like(g_tr.data))
    w = W_tr.data.contiguous()
    g = g_tr.data.contiguous()
    check(_native.lib().tprf_gw_dynamic_sigma(gt.n_tau, len(gr), nb, w.data_ptr(), g.data_ptr(), out.data.data_ptr(),
                                              _stream()), "gw_dynamic_sigma")
    return out
