"""GB300 drop-in for the ``triqs_tprf.lattice`` functions on the bubble + RPA path.

Same names, argument meaning and keyword names as the reference's cpp2py
module (``python/triqs_tprf/lattice_desc.py``); each call goes through the C
ABI of the CUDA library. Green's functions are ``tprf_gb300.Gf`` objects whose
data lives on the GPU. Errors raise ``TprfError`` (a ``RuntimeError``, as the
reference's ``TRIQS_RUNTIME_ERROR`` does through cpp2py).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native
from ._native import check, dims3
from .gf import Gf, as_device_c128
from .mesh import MeshBrZone, MeshCycLat, MeshImFreq, MeshImTime, MeshProduct

__all__ = [
    "lattice_dyson_g0_wk", "lattice_dyson_g_wk", "fourier_wk_to_wr", "fourier_wr_to_wk",
    "fourier_wr_to_tr", "chi0_tr_from_grt_PH", "chi0_wr_from_grt_PH", "chi0_w0r_from_grt_PH",
    "chi_wr_from_chi_tr", "chi_w0r_from_chi_tr", "chi_wk_from_chi_wr", "chi_wr_from_chi_wk",
    "solve_rpa_PH", "default_n_tau", "fourier_tr_to_wr", "chi_tr_from_chi_wr",
    "split_into_dynamic_wk_and_constant_k", "lindhard_chi00",
]


def _bosonic_wk_mesh(g):
    """(nw, dims) when g lives on (bosonic MeshImFreq, MeshBrZone), else None."""
    m = g.mesh
    if not isinstance(m, MeshProduct) or len(m.components) != 2:
        return None
    w, k = m.components
    if not isinstance(w, MeshImFreq) or w.statistic != "Boson" or not isinstance(k, MeshBrZone):
        return None
    return w.n_max, tuple(k.dims)


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _ptr(t: torch.Tensor):
    return t.data_ptr() if t is not None else None


def default_n_tau(n_max: int) -> int:
    """Time-mesh size the reference's make_adjoint_mesh picks for a fermionic mesh: 6 n_max + 1."""
    return 6 * int(n_max) + 1


def _components(g, kinds, name):
    if not isinstance(g, Gf) or not isinstance(g.mesh, MeshProduct) or len(g.mesh.components) != 2:
        raise TypeError(f"{name}: expected a Gf on a MeshProduct of two meshes")
    a, b = g.mesh.components
    if not isinstance(a, kinds[0]) or not isinstance(b, kinds[1]):
        raise TypeError(f"{name}: expected meshes ({kinds[0].__name__}, {kinds[1].__name__}), got ({type(a).__name__}, {type(b).__name__})")
    return a, b


def _ntarget(g: Gf) -> int:
    return int(np.prod(g.target_shape)) if g.target_shape else 1


# ---------------------------------------------------------------------------
# Dyson (c++/triqs_tprf/lattice/gf.cpp:42-58, 91-132)


def lattice_dyson_g0_wk(mu, e_k, mesh):
    """G0(iv, k) = [(iv + mu) I - e(k)]^-1 (lattice_desc.py:27)."""
    return _dyson(mu, e_k, mesh, None, 0)


def lattice_dyson_g_wk(mu, e_k, sigma_w=None, sigma_wk=None, sigma=None):
    """G(iv, k) = [(iv + mu) I - e(k) - Sigma]^-1 with Sigma(iv) or Sigma(iv, k) (lattice_desc.py:57,119)."""
    if sigma is not None:
        if isinstance(sigma.mesh, MeshProduct):
            sigma_wk = sigma
        else:
            sigma_w = sigma
    if (sigma_w is None) == (sigma_wk is None):
        raise TypeError("lattice_dyson_g_wk: give exactly one of sigma_w, sigma_wk")
    if sigma_w is not None:
        return _dyson(mu, e_k, sigma_w.mesh, sigma_w, 1)
    wmesh, _ = _components(sigma_wk, (MeshImFreq, MeshBrZone), "lattice_dyson_g_wk")
    return _dyson(mu, e_k, wmesh, sigma_wk, 2)


def _dyson(mu, e_k, wmesh, sigma, kind):
    if not isinstance(e_k, Gf) or not isinstance(e_k.mesh, MeshBrZone):
        raise TypeError("lattice_dyson: e_k must be a Gf on a MeshBrZone")
    if not isinstance(wmesh, MeshImFreq) or wmesh.statistic != "Fermion":
        raise TypeError("lattice_dyson: needs a fermionic MeshImFreq")
    nb = e_k.target_shape[0]
    nk = len(e_k.mesh)
    out = Gf(mesh=MeshProduct(wmesh, e_k.mesh), target_shape=(nb, nb), device=e_k.data.device)
    sig = None
    if sigma is not None:
        sig = as_device_c128(sigma.data, e_k.data.device)
        expect = (len(wmesh), nb, nb) if kind == 1 else (len(wmesh), nk, nb, nb)
        if tuple(sig.shape) != expect:
            raise ValueError(f"lattice_dyson_g_wk: sigma shape {tuple(sig.shape)} != {expect}")
    ek = e_k.data.contiguous()
    check(_native.lib().tprf_lattice_dyson_g_wk(wmesh.beta, wmesh.n_max, nk, nb, float(mu), _ptr(ek), _ptr(sig),
                                                kind, _ptr(out.data), _stream()), "lattice_dyson_g_wk")
    return out


# ---------------------------------------------------------------------------
# k <-> r (lattice/fourier.hpp:166-231, fourier/fourier_lattice.cpp:28-59)


def _lattice(g, forward, name):
    kinds = (object, MeshBrZone) if forward else (object, MeshCycLat)
    wmesh, pmesh = _components(g, kinds, name)
    new_p = MeshCycLat(dims=pmesh.dims) if forward else MeshBrZone(dims=pmesh.dims)
    out = Gf(mesh=MeshProduct(wmesh, new_p), data=torch.empty_like(g.data))
    src = g.data.contiguous()
    fn = _native.lib().tprf_fourier_wk_to_wr if forward else _native.lib().tprf_fourier_wr_to_wk
    check(fn(len(wmesh), dims3(pmesh.dims), _ntarget(g), _ptr(src), _ptr(out.data), _stream()), name)
    return out


def fourier_wk_to_wr(g_wk):
    """k -> r, FFTW_FORWARD / N_k (lattice_desc.py:277)."""
    return _lattice(g_wk, True, "fourier_wk_to_wr")


def fourier_wr_to_wk(g_wr):
    """r -> k, FFTW_BACKWARD unscaled (lattice_desc.py:293)."""
    return _lattice(g_wr, False, "fourier_wr_to_wk")


def chi_wk_from_chi_wr(chi_wr):
    """r -> q for chi(w, r) (lattice_desc.py:1450)."""
    return _lattice(chi_wr, False, "chi_wk_from_chi_wr")


def chi_wr_from_chi_wk(chi_wk):
    """q -> r for chi(w, q) (chi_imtime.cpp:294-297)."""
    return _lattice(chi_wk, True, "chi_wr_from_chi_wk")


# ---------------------------------------------------------------------------
# iv -> tau (fourier/fourier_matsubara.cpp:218-308)


def fourier_wr_to_tr(g_wr, nt=-1, moments=None):
    """G(iv, r) -> G(tau, r) (lattice_desc.py:309).

    ``moments`` (an extension; the reference always fits the tail) may hold the
    first three high-frequency moments, shape (3, N_r) + target_shape.
    """
    wmesh, rmesh = _components(g_wr, (MeshImFreq, MeshCycLat), "fourier_wr_to_tr")
    if wmesh.statistic != "Fermion":
        raise TypeError("fourier_wr_to_tr: needs a fermionic frequency mesh")
    n_tau = default_n_tau(wmesh.n_max) if nt is None or nt < 0 else int(nt)
    tmesh = MeshImTime(wmesh.beta, "Fermion", n_tau)
    out = Gf(mesh=MeshProduct(tmesh, rmesh), target_shape=g_wr.target_shape, device=g_wr.data.device)
    mom = None
    if moments is not None:
        mom = as_device_c128(moments, g_wr.data.device)
        if mom.numel() != 3 * len(rmesh) * _ntarget(g_wr):
            raise ValueError("fourier_wr_to_tr: moments must have shape (3, N_r) + target_shape")
    src = g_wr.data.contiguous()
    check(_native.lib().tprf_fourier_wr_to_tr(wmesh.beta, wmesh.n_max, n_tau, len(rmesh), _ntarget(g_wr), _ptr(src),
                                              _ptr(mom), _ptr(out.data), _stream()), "fourier_wr_to_tr")
    return out


# ---------------------------------------------------------------------------
# Bubble and chi transforms (lattice/chi_imtime.cpp)


def _gtr(g_tr, name):
    tmesh, rmesh = _components(g_tr, (MeshImTime, MeshCycLat), name)
    ts = g_tr.target_shape
    if len(ts) != 2 or ts[0] != ts[1]:
        raise ValueError(f"{name}: G(tau, r) must be matrix valued")
    return tmesh, rmesh, ts[0]


def chi0_tr_from_grt_PH(g_tr):
    """chi0_abcd(tau, r) = G_da(tau, r) G_bc(beta - tau, -r) (lattice_desc.py:1317)."""
    tmesh, rmesh, nb = _gtr(g_tr, "chi0_tr_from_grt_PH")
    out = Gf(mesh=MeshProduct(MeshImTime(tmesh.beta, "Boson", tmesh.n_tau), rmesh), target_shape=(nb,) * 4,
             device=g_tr.data.device)
    src = g_tr.data.contiguous()
    check(_native.lib().tprf_chi0_tr_from_grt_PH(tmesh.n_tau, dims3(rmesh.dims), nb, _ptr(src), _ptr(out.data),
                                                 _stream()), "chi0_tr_from_grt_PH")
    return out


def chi0_wr_from_grt_PH(g_tr, nw):
    """Bubble fused with tau -> w, chi0(tau, r) never stored (lattice_desc.py:1360)."""
    tmesh, rmesh, nb = _gtr(g_tr, "chi0_wr_from_grt_PH")
    out = Gf(mesh=MeshProduct(MeshImFreq(tmesh.beta, "Boson", nw), rmesh), target_shape=(nb,) * 4,
             device=g_tr.data.device)
    src = g_tr.data.contiguous()
    check(_native.lib().tprf_chi0_wr_from_grt_PH(tmesh.beta, tmesh.n_tau, int(nw), dims3(rmesh.dims), nb, _ptr(src),
                                                 _ptr(out.data), _stream()), "chi0_wr_from_grt_PH")
    return out


def chi0_w0r_from_grt_PH(g_tr):
    """Static bubble by trapezoid integration over tau (lattice_desc.py:1362)."""
    tmesh, rmesh, nb = _gtr(g_tr, "chi0_w0r_from_grt_PH")
    out = Gf(mesh=MeshProduct(MeshImFreq(tmesh.beta, "Boson", 1), rmesh), target_shape=(nb,) * 4,
             device=g_tr.data.device)
    src = g_tr.data.contiguous()
    check(_native.lib().tprf_chi0_w0r_from_grt_PH(tmesh.beta, tmesh.n_tau, dims3(rmesh.dims), nb, _ptr(src),
                                                  _ptr(out.data), _stream()), "chi0_w0r_from_grt_PH")
    return out


def chi_wr_from_chi_tr(chi_tr, nw):
    """Bosonic tau -> w with fit_derivatives tails (lattice_desc.py:1402)."""
    tmesh, rmesh = _components(chi_tr, (MeshImTime, MeshCycLat), "chi_wr_from_chi_tr")
    out = Gf(mesh=MeshProduct(MeshImFreq(tmesh.beta, "Boson", nw), rmesh), target_shape=chi_tr.target_shape,
             device=chi_tr.data.device)
    src = chi_tr.data.contiguous()
    check(_native.lib().tprf_chi_wr_from_chi_tr(tmesh.beta, tmesh.n_tau, int(nw), len(rmesh), _ntarget(chi_tr),
                                                _ptr(src), _ptr(out.data), _stream()), "chi_wr_from_chi_tr")
    return out


def fourier_tr_to_wr(g_tr, nw=-1):
    """Fermionic G(tau, r) -> G(iv, r) with fit_derivatives tails (lattice_desc.py:325,
    gf.cpp:257-260). nw < 0: (n_tau - 1) / 6 positive frequencies."""
    tmesh, rmesh = _components(g_tr, (MeshImTime, MeshCycLat), "fourier_tr_to_wr")
    if tmesh.statistic != "Fermion":
        raise TypeError("fourier_tr_to_wr: needs a fermionic time mesh")
    n_iw = (tmesh.n_tau - 1) // 6 if nw is None or nw < 0 else int(nw)
    out = Gf(mesh=MeshProduct(MeshImFreq(tmesh.beta, "Fermion", n_iw), rmesh), target_shape=g_tr.target_shape,
             device=g_tr.data.device)
    src = g_tr.data.contiguous()
    check(_native.lib().tprf_fourier_tr_to_wr(tmesh.beta, tmesh.n_tau, n_iw, len(rmesh), _ntarget(g_tr), _ptr(src),
                                              _ptr(out.data), _stream()), "fourier_tr_to_wr")
    return out


def chi_tr_from_chi_wr(chi_wr, ntau=-1, moments=None):
    """Bosonic chi(iw, r) -> chi(tau, r) with the tail fit (lattice_desc.py:1426,
    chi_imtime.cpp:284-287). ntau < 0: 6 nw + 1 points; ``moments`` (an extension)
    may hold m1..m3 with shape (3, N_r) + target_shape."""
    wmesh, rmesh = _components(chi_wr, (MeshImFreq, MeshCycLat), "chi_tr_from_chi_wr")
    if wmesh.statistic != "Boson":
        raise TypeError("chi_tr_from_chi_wr: needs a bosonic frequency mesh")
    n_tau = 6 * wmesh.n_max + 1 if ntau is None or ntau < 0 else int(ntau)
    out = Gf(mesh=MeshProduct(MeshImTime(wmesh.beta, "Boson", n_tau), rmesh), target_shape=chi_wr.target_shape,
             device=chi_wr.data.device)
    mom = None
    if moments is not None:
        mom = as_device_c128(moments, chi_wr.data.device)
        if mom.numel() != 3 * len(rmesh) * _ntarget(chi_wr):
            raise ValueError("chi_tr_from_chi_wr: moments must have shape (3, N_r) + target_shape")
    src = chi_wr.data.contiguous()
    check(_native.lib().tprf_chi_tr_from_chi_wr(wmesh.beta, wmesh.n_max, n_tau, len(rmesh), _ntarget(chi_wr),
                                                _ptr(src), _ptr(mom), _ptr(out.data), _stream()),
          "chi_tr_from_chi_wr")
    return out


def lindhard_chi00(e_k, mesh, mu):
    """Analytic band-basis bubble chi00(iw, q) on a bosonic MeshImFreq (lattice_desc.py:411,
    lindhard_chi00.cpp:34-100). Cost O(N_k^2): a validation tool for small meshes."""
    if not isinstance(e_k, Gf) or not isinstance(e_k.mesh, MeshBrZone):
        raise TypeError("lindhard_chi00: e_k must be a Gf on a MeshBrZone")
    if not isinstance(mesh, MeshImFreq) or mesh.statistic != "Boson":
        raise RuntimeError("lindhard_chi00: statistic is incorrect.")
    nb = e_k.target_shape[0]
    nk = len(e_k.mesh)
    dev = e_k.data.device
    lib = _native.lib()
    out = Gf(mesh=MeshProduct(mesh, e_k.mesh), target_shape=(nb,) * 4, device=dev)
    ws = torch.empty(lib.tprf_lindhard_chi00_workspace_bytes(nk, nb), dtype=torch.uint8, device=dev)
    ek = e_k.data.contiguous()
    check(lib.tprf_lindhard_chi00(nk, dims3(e_k.mesh.dims), nb, _ptr(ek), mesh.beta, float(mu), mesh.n_max,
                                  _ptr(out.data), _ptr(ws), ws.numel(), _stream()), "lindhard_chi00")
    return out


def split_into_dynamic_wk_and_constant_k(chi_wk):
    """(chi_dyn_wk, chi_const_k): chi_const(k) is the constant tail moment of
    chi(iw, k) on the bosonic mesh, chi_dyn = chi - chi_const (lattice_desc.py:598,
    lattice_utility.cpp:57-85)."""
    wmesh, kmesh = _components(chi_wk, (MeshImFreq, MeshBrZone), "split_into_dynamic_wk_and_constant_k")
    if wmesh.statistic != "Boson":
        raise TypeError("split_into_dynamic_wk_and_constant_k: needs a bosonic frequency mesh")
    dev = chi_wk.data.device
    dyn = Gf(mesh=chi_wk.mesh, data=torch.empty_like(chi_wk.data))
    const = Gf(mesh=kmesh, target_shape=chi_wk.target_shape, device=dev)
    src = chi_wk.data.contiguous()
    check(_native.lib().tprf_split_into_dynamic_wk_and_constant_k(wmesh.beta, wmesh.n_max, len(kmesh),
                                                                  _ntarget(chi_wk), _ptr(src), _ptr(dyn.data),
                                                                  _ptr(const.data), _stream()),
          "split_into_dynamic_wk_and_constant_k")
    return dyn, const


def chi_w0r_from_chi_tr(chi_tr):
    """Trapezoid integral over tau (lattice_desc.py:1381)."""
    tmesh, rmesh = _components(chi_tr, (MeshImTime, MeshCycLat), "chi_w0r_from_chi_tr")
    out = Gf(mesh=MeshProduct(MeshImFreq(tmesh.beta, "Boson", 1), rmesh), target_shape=chi_tr.target_shape,
             device=chi_tr.data.device)
    src = chi_tr.data.contiguous()
    check(_native.lib().tprf_chi_w0r_from_chi_tr(tmesh.beta, tmesh.n_tau, len(rmesh), _ntarget(chi_tr), _ptr(src),
                                                 _ptr(out.data), _stream()), "chi_w0r_from_chi_tr")
    return out


# ---------------------------------------------------------------------------
# RPA (lattice/rpa.cpp:29-68)


def solve_rpa_PH(chi0, U, out=None, chunk_points=None, workspace=None):
    """chi = [1 - chi0 U]^-1 chi0 in the PH grouping (lattice_desc.py:547).

    With ``out`` (a host tensor of chi0's shape, ideally pinned) the result is
    written to host memory as it is solved: chunks of ``chunk_points`` (q, iw)
    points go through a device ring in ``workspace`` (allocated here if None) and
    their copies to the host overlap the solve of the next chunk. The returned Gf
    then holds the host tensor.
    """
    if not isinstance(chi0, Gf) or chi0.target_rank != 4:
        raise TypeError("solve_rpa_PH: chi0 must be a rank-4 tensor valued Gf")
    nb = chi0.target_shape[0]
    Ud = as_device_c128(U, chi0.data.device)
    if tuple(Ud.shape) != (nb,) * 4:
        raise ValueError(f"solve_rpa_PH: U must have shape {(nb,) * 4}")
    n_points = chi0.data.numel() // nb ** 4
    src = chi0.data.contiguous()
    lib = _native.lib()
    if out is None:
        res = Gf(mesh=chi0.mesh, data=torch.empty_like(chi0.data))
        wk = _bosonic_wk_mesh(chi0)
        if wk is not None:  # the mesh-aware solve: conjugate point pairs solved once
            nw, dims = wk
            check(lib.tprf_solve_rpa_PH_wk(nw, dims3(dims), nb, _ptr(src), _ptr(Ud), _ptr(res.data), _stream()),
                  "solve_rpa_PH")
        else:
            check(lib.tprf_solve_rpa_PH(n_points, nb, _ptr(src), _ptr(Ud), _ptr(res.data), _stream()), "solve_rpa_PH")
        return res
    if out.device.type != "cpu" or out.dtype != torch.complex128 or tuple(out.shape) != tuple(chi0.data.shape) \
            or not out.is_contiguous():
        raise ValueError("solve_rpa_PH: out must be a contiguous complex128 host tensor of chi0's shape")
    if chunk_points is None:
        chunk_points = max(1, -(-n_points // 32))
    if workspace is None:
        nbytes = lib.tprf_solve_rpa_PH_to_host_workspace_bytes(chunk_points, nb, 3)
        workspace = torch.empty(nbytes, dtype=torch.uint8, device=chi0.data.device)
    check(lib.tprf_solve_rpa_PH_to_host(n_points, nb, _ptr(src), _ptr(Ud), out.data_ptr(), chunk_points,
                                        _ptr(workspace), workspace.numel() * workspace.element_size(), _stream()),
          "solve_rpa_PH")
    return Gf(mesh=chi0.mesh, data=out, device=torch.device("cpu"))
