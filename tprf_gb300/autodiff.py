"""Differentiable bubble + RPA: gradients of chi(q, iw) with respect to the
interaction tensor U and real hopping amplitudes t(R).

``chi_rpa(theta, U, model)`` runs the whole chain (Dyson -> k->r -> iv->tau ->
bubble + tau->iw -> r->q -> RPA) through the CUDA kernels; its backward pass is
hand-written: every stage's adjoint kernel runs in reverse order
(tprf_*_adjoint). G(tau, r) is recomputed in the backward pass rather than
kept from the forward one. Gradients follow torch's conjugate-Wirtinger
convention, so they compose with any real-valued torch loss of chi.

The dispersion is e(k) = e0(k) + sum_a theta_a E_a(k): theta are real
amplitudes multiplying fixed hopping patterns (see ``HoppingModel``).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from . import _native
from ._native import check, dims3
from .tight_binding import ek_tensor

__all__ = ["HoppingModel", "chi_rpa", "ChiRPA"]


@dataclass
class HoppingModel:
    """e(k) = e0(k) + sum_a theta_a E_a(k) on a k mesh, with fixed hopping patterns.

    base: {R: t(R)} of the fixed part; patterns: list of {R: matrix} (each
    pattern should be Hermitian as a whole, e.g. {R: T, -R: T^H}).
    """
    base: dict
    patterns: list
    dims: tuple
    beta: float
    mu: float
    n_max: int
    nw: int

    def tensors(self, device):
        e0 = ek_tensor(self.base, self.dims, device=device)
        E = torch.stack([ek_tensor(p, self.dims, device=device) for p in self.patterns])
        return e0, E


def _s():
    return torch.cuda.current_stream().cuda_stream


def _forward_intermediates(e_k, m: HoppingModel):
    lib = _native.lib()
    dev = e_k.device
    nk, nb = e_k.shape[0], e_k.shape[-1]
    nb2, nb4 = nb * nb, nb ** 4
    n_nu, n_tau, nwt = 2 * m.n_max, 6 * m.n_max + 1, 2 * m.nw - 1
    d3 = dims3(m.dims)
    g_wk = torch.empty(n_nu, nk, nb, nb, dtype=torch.complex128, device=dev)
    check(lib.tprf_lattice_dyson_g_wk(m.beta, m.n_max, nk, nb, m.mu, e_k.data_ptr(), None, 0, g_wk.data_ptr(), _s()))
    g_wr = torch.empty_like(g_wk)
    check(lib.tprf_fourier_wk_to_wr(n_nu, d3, nb2, g_wk.data_ptr(), g_wr.data_ptr(), _s()))
    g_tr = torch.empty(n_tau, nk, nb, nb, dtype=torch.complex128, device=dev)
    check(lib.tprf_fourier_wr_to_tr(m.beta, m.n_max, n_tau, nk, nb2, g_wr.data_ptr(), None, g_tr.data_ptr(), _s()))
    chi0 = torch.empty(nwt, nk, nb4, dtype=torch.complex128, device=dev)
    check(lib.tprf_chi0_wr_from_grt_PH(m.beta, n_tau, m.nw, d3, nb, g_tr.data_ptr(), chi0.data_ptr(), _s()))
    check(lib.tprf_fourier_wr_to_wk(nwt, d3, nb4, chi0.data_ptr(), chi0.data_ptr(), _s()))
    return g_wk, g_tr, chi0


class ChiRPA(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, U, e0, E, model: HoppingModel):
        lib = _native.lib()
        e_k = (e0 + torch.einsum("a,akij->kij", theta.to(e0.dtype), E)).contiguous()
        nb = e_k.shape[-1]
        g_wk, g_tr, chi0 = _forward_intermediates(e_k, model)
        Uc = U.to(torch.complex128).contiguous()
        chi = torch.empty_like(chi0)
        n_points = chi0.shape[0] * chi0.shape[1]
        check(lib.tprf_solve_rpa_PH(n_points, nb, chi0.data_ptr(), Uc.data_ptr(), chi.data_ptr(), _s()))
        ctx.model = model
        ctx.save_for_backward(e_k, Uc, E, chi0, chi)
        nk = e_k.shape[0]
        return chi.view(chi0.shape[0], nk, nb, nb, nb, nb)

    @staticmethod
    def backward(ctx, chi_grad):
        lib = _native.lib()
        m = ctx.model
        e_k, Uc, E, chi0, chi = ctx.saved_tensors
        nk, nb = e_k.shape[0], e_k.shape[-1]
        nb2, nb4 = nb * nb, nb ** 4
        n_tau, nwt = 6 * m.n_max + 1, 2 * m.nw - 1
        d3 = dims3(m.dims)
        g = chi_grad.to(torch.complex128).contiguous()
        # RPA
        chi0_grad = torch.empty_like(chi0)
        U_grad = torch.zeros_like(Uc)
        check(lib.tprf_solve_rpa_PH_adjoint(nwt * nk, nb, chi0.data_ptr(), Uc.data_ptr(), chi.data_ptr(),
                                            g.data_ptr(), chi0_grad.data_ptr(), U_grad.data_ptr(), _s()))
        # r -> q (FFTW_BACKWARD, unscaled): transpose = N_k (1/N_k FFTW_FORWARD)
        chi0wr_grad = torch.empty_like(chi0_grad)
        check(lib.tprf_fourier_wk_to_wr(nwt, d3, nb4, chi0_grad.data_ptr(), chi0wr_grad.data_ptr(), _s()))
        chi0wr_grad.mul_(float(nk))
        # the bubble fused with tau -> iw, transposed (G recomputed: the forward pass
        # does not keep it); chi0_grad(tau, r) never exists in device memory
        g_wk, g_tr, _ = _forward_intermediates_g(e_k, m)
        g_tr_grad = torch.empty_like(g_tr)
        check(lib.tprf_chi0_wr_from_grt_PH_adjoint(m.beta, n_tau, m.nw, d3, nb, g_tr.data_ptr(),
                                                   chi0wr_grad.data_ptr(), g_tr_grad.data_ptr(), _s()))
        del chi0wr_grad
        # iv -> tau with the fitted tail, k -> r (1/N_k FFTW_FORWARD): transpose = FFTW_BACKWARD / N_k
        g_wr_grad = torch.empty_like(g_wk)
        check(lib.tprf_fourier_wr_to_tr_adjoint(m.beta, m.n_max, n_tau, nk, nb2, g_tr_grad.data_ptr(), 1,
                                                g_wr_grad.data_ptr(), _s()))
        g_wk_grad = torch.empty_like(g_wk)
        check(lib.tprf_fourier_wr_to_wk(2 * m.n_max, d3, nb2, g_wr_grad.data_ptr(), g_wk_grad.data_ptr(), _s()))
        g_wk_grad.mul_(1.0 / nk)
        # Dyson
        e_grad = torch.empty_like(e_k)
        check(lib.tprf_lattice_dyson_g_wk_adjoint(m.n_max, nk, nb, g_wk.data_ptr(), g_wk_grad.data_ptr(),
                                                  e_grad.data_ptr(), _s()))
        theta_grad = torch.einsum("akij,kij->a", E.conj(), e_grad).real
        return theta_grad, U_grad, None, None, None


def _forward_intermediates_g(e_k, m):
    """G(iv, k) and G(tau, r) of the forward pass, recomputed."""
    lib = _native.lib()
    dev = e_k.device
    nk, nb = e_k.shape[0], e_k.shape[-1]
    nb2 = nb * nb
    n_nu, n_tau = 2 * m.n_max, 6 * m.n_max + 1
    g_wk = torch.empty(n_nu, nk, nb, nb, dtype=torch.complex128, device=dev)
    check(lib.tprf_lattice_dyson_g_wk(m.beta, m.n_max, nk, nb, m.mu, e_k.data_ptr(), None, 0, g_wk.data_ptr(), _s()))
    g_wr = torch.empty_like(g_wk)
    check(lib.tprf_fourier_wk_to_wr(n_nu, dims3(m.dims), nb2, g_wk.data_ptr(), g_wr.data_ptr(), _s()))
    g_tr = torch.empty(n_tau, nk, nb, nb, dtype=torch.complex128, device=dev)
    check(lib.tprf_fourier_wr_to_tr(m.beta, m.n_max, n_tau, nk, nb2, g_wr.data_ptr(), None, g_tr.data_ptr(), _s()))
    return g_wk, g_tr, None


def chi_rpa(theta: torch.Tensor, U: torch.Tensor, model: HoppingModel):
    """chi(iw, q) [2nw-1, N_k, nb, nb, nb, nb], differentiable in theta (real) and U (complex)."""
    dev = theta.device
    e0, E = model.tensors(dev)
    return ChiRPA.apply(theta, U, e0, E, model)
