"""Dense FP64 CPU autograd reference of the bubble + RPA chain (torch complex128).

TEST INFRASTRUCTURE ONLY: the checker for the GPU adjoint kernels. It restates
the same reference files as ``tprf_oracle.py`` with differentiable torch ops
(``lattice/gf.cpp:42-58`` Dyson, ``fourier_lattice.cpp:28-59`` k<->r,
``fourier_matsubara.cpp:218-308`` iv -> tau with the tail fit,
``chi_imtime.cpp:88-136`` bubble, ``fourier_matsubara.cpp:42-97,123-184``
tau -> iw, ``rpa.cpp:29-64`` RPA) so torch.autograd gives reference gradients.
"""
from __future__ import annotations

import numpy as np
import torch

from . import tprf_oracle as O

C128 = torch.complex128


def _t(x):
    return torch.as_tensor(np.asarray(x), dtype=C128)


def dyson(e_k, beta, mu, n_max):
    nb = e_k.shape[-1]
    iw = _t(O.fermionic_iw(beta, n_max))
    m = (iw + mu)[:, None, None, None] * torch.eye(nb, dtype=C128) - e_k[None]
    return torch.linalg.inv(m)


def k_to_r(g, dims):
    sh = g.shape
    a = g.reshape((sh[0],) + tuple(dims) + sh[2:])
    return (torch.fft.fftn(a, dim=(1, 2, 3)) / int(np.prod(dims))).reshape(sh)


def r_to_k(g, dims):
    sh = g.shape
    a = g.reshape((sh[0],) + tuple(dims) + sh[2:])
    return (torch.fft.ifftn(a, dim=(1, 2, 3)) * int(np.prod(dims))).reshape(sh)


def nu_to_tau(g_wr, beta, n_tau):
    n_nu = g_wr.shape[0]
    n_max = n_nu // 2
    L = n_tau - 1
    rest = g_wr.shape[1:]
    g = g_wr.reshape(n_nu, -1)
    idx, F, _ = O.tail_fit_matrix(beta, n_max)
    c = _t(F) @ g[torch.as_tensor(idx)]
    m1, m2, m3 = c[1], c[2], c[3]
    a1, a2, a3 = m1 - m3, (m2 + m3) / 2, (m3 - m2) / 2
    iw = _t(O.fermionic_iw(beta, n_max))[:, None]
    model = a1 / (iw - 0.0) + a2 / (iw - 1.0) + a3 / (iw + 1.0)
    n = np.arange(-n_max, n_max)
    rows = torch.as_tensor((n + L) % L)
    gin = torch.zeros((L, g.shape[1]), dtype=C128).index_copy(0, rows, (1.0 / beta) * (g - model))
    out = torch.fft.fft(gin, dim=0)
    tau = O.tau_points(beta, n_tau)[:L]
    ph = _t(np.exp(-1j * np.pi * tau / beta))[:, None]

    def f(b):
        v = np.exp(-b * tau) / (1 + np.exp(-beta * b)) if b >= 0 else np.exp(b * (beta - tau)) / (1 + np.exp(beta * b))
        return _t(-v)[:, None]

    gt = out * ph + a1[None] * f(0.0) + a2[None] * f(1.0) + a3[None] * f(-1.0)
    gL = -(gt[0] + m1)
    return torch.cat([gt, gL[None]], 0).reshape((n_tau,) + rest)


def bubble(g_tr, dims):
    nt = g_tr.shape[0]
    sh = g_tr.shape
    a = g_tr.reshape((nt,) + tuple(dims) + sh[2:])
    a = torch.roll(torch.flip(a, dims=(1, 2, 3)), shifts=(1, 1, 1), dims=(1, 2, 3)).reshape(sh)
    gm = torch.flip(a, dims=(0,))
    return torch.einsum("trda,trbc->trabcd", g_tr, gm)


def tau_to_w(chi_tr, beta, nw):
    n_tau = chi_tr.shape[0]
    L = n_tau - 1
    rest = chi_tr.shape[1:]
    g = chi_tr.reshape(n_tau, -1)
    dtau = beta / (n_tau - 1)
    V = _t(O.FIT_DERIVATIVE_ROWS)
    taus = torch.as_tensor(np.arange(1, 9) * dtau, dtype=torch.float64)[:, None]
    d_left = (g[1:9] - g[0][None]) / taus
    d_right = (g[n_tau - 1][None] - g[n_tau - 2 - torch.arange(8)]) / taus
    gl, gr = V @ d_left, V @ d_right
    m2 = gl[0] - gr[0]
    m3 = -(gl[1] + gr[1]) * 2 / dtau
    m1 = -(g[0] - g[L])
    a1, a2, a3 = 4 * (m1 - m3) / 3, m3 - (m1 + m2) / 2, m1 / 6 + m2 / 2 + m3 / 3
    tau = O.tau_points(beta, n_tau)[:L]

    def h(b):
        v = np.exp(-b * tau) / (np.exp(-beta * b) - 1) if b >= 0 else np.exp(b * (beta - tau)) / (1 - np.exp(b * beta))
        return _t(v)[:, None]

    gin = (beta / L) * (g[:L] - (a1[None] * h(-0.5) + a2[None] * h(-1.0) + a3[None] * h(1.0)))
    out = torch.fft.ifft(gin, dim=0) * L
    m = np.arange(-(nw - 1), nw)
    iw = _t(O.bosonic_iw(beta, nw))[:, None]
    gw = out[torch.as_tensor((m + L) % L)] + a1 / (iw + 0.5) + a2 / (iw + 1.0) + a3 / (iw - 1.0)
    return gw.reshape((2 * nw - 1,) + rest)


def solve_rpa(chi0, U):
    nb = U.shape[0]
    g = lambda x: torch.swapaxes(x, -1, -2).reshape(x.shape[:-4] + (nb * nb, nb * nb))  # noqa: E731
    c0, Ug = g(chi0), g(U)
    chi = torch.linalg.solve(torch.eye(nb * nb, dtype=C128) - c0 @ Ug, c0)
    return torch.swapaxes(chi.reshape(chi.shape[:-2] + (nb,) * 4), -1, -2)


def chi_rpa(e_k, U, dims, beta, mu, n_max, nw):
    """chi(iw, q) of the whole chain, differentiable in e_k and U."""
    n_tau = 6 * n_max + 1
    g_tr = nu_to_tau(k_to_r(dyson(e_k, beta, mu, n_max), dims), beta, n_tau)
    chi0 = r_to_k(tau_to_w(bubble(g_tr, dims), beta, nw), dims)
    return solve_rpa(chi0, U)
