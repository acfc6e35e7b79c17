"""Gradients of chi w.r.t. U and the hopping amplitudes t(R) through the
hand-written adjoint kernels, against a dense FP64 CPU autograd reference and
against central finite differences (h = 1e-6)."""
import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _reference_grads(model, theta0, U):
    from oracle import torch_chain as TC
    e0, E = model.tensors(torch.device("cpu"))
    theta = torch.as_tensor(theta0, dtype=torch.float64).clone().requires_grad_(True)
    Ut = torch.as_tensor(U, dtype=torch.complex128).clone().requires_grad_(True)
    e_k = e0 + torch.einsum("a,akij->kij", theta.to(torch.complex128), E)
    from tprf_gb300.workloads import cfg3_loss
    chi = TC.chi_rpa(e_k, Ut, model.dims, model.beta, model.mu, model.n_max, model.nw)
    L = cfg3_loss(chi)
    L.backward()
    return L.item(), theta.grad.numpy(), Ut.grad.numpy()


def _gpu(model, theta0, U, grad=True):
    from tprf_gb300.autodiff import chi_rpa
    from tprf_gb300.workloads import cfg3_loss
    theta = torch.as_tensor(theta0, dtype=torch.float64, device="cuda").clone().requires_grad_(grad)
    Ut = torch.as_tensor(U, dtype=torch.complex128, device="cuda").clone().requires_grad_(grad)
    L = cfg3_loss(chi_rpa(theta, Ut, model))
    if grad:
        L.backward()
        return L.item(), theta.grad.cpu().numpy(), Ut.grad.cpu().numpy()
    return L.item()


def test_gradients_match_dense_cpu_autograd(cuda_lib):
    from tprf_gb300.workloads import cfg3_model
    model, theta0, U = cfg3_model(dims=(6, 6, 1), beta=5.0, n_max=24, nw=6)
    L_ref, gt_ref, gu_ref = _reference_grads(model, theta0, U)
    L, gt, gu = _gpu(model, theta0, U)
    assert abs(L - L_ref) <= 1e-10 * abs(L_ref)
    assert rel_err(gt, gt_ref) < 1e-9
    assert rel_err(gu, gu_ref) < 1e-9


def _fd_check(model, theta0, U, n_theta=3, n_u=2, rtol=1e-6):
    L, gt, gu = _gpu(model, theta0, U)
    h = 1e-6
    for a in range(n_theta):
        tp, tm = theta0.copy(), theta0.copy()
        tp[a] += h
        tm[a] -= h
        fd = (_gpu(model, tp, U, grad=False) - _gpu(model, tm, U, grad=False)) / (2 * h)
        assert abs(fd - gt[a]) <= rtol * max(abs(fd), np.abs(gt).max()), (a, fd, gt[a])
    flat = np.flatnonzero(np.abs(U.ravel()) > 0)[:n_u]
    for f in flat:
        for part, unit in ((0, 1.0), (1, 1j)):
            Up, Um = U.copy().ravel(), U.copy().ravel()
            Up[f] += h * unit
            Um[f] -= h * unit
            fd = (_gpu(model, theta0, Up.reshape(U.shape), grad=False)
                  - _gpu(model, theta0, Um.reshape(U.shape), grad=False)) / (2 * h)
            g = gu.ravel()[f]
            comp = g.real if part == 0 else g.imag
            assert abs(fd - comp) <= rtol * max(abs(fd), np.abs(gu).max()), (f, part, fd, comp)


def test_gradients_match_finite_differences_small(cuda_lib):
    from tprf_gb300.workloads import cfg3_model
    model, theta0, U = cfg3_model(dims=(8, 8, 1), beta=8.0, n_max=32, nw=8)
    _fd_check(model, theta0, U)


def test_gradients_match_finite_differences_cfg3(cuda_lib):
    """cfg3 itself: 32 x 32, beta = 16, 128 fermionic / bosonic frequencies."""
    from tprf_gb300.workloads import cfg3_model
    model, theta0, U = cfg3_model()
    _fd_check(model, theta0, U, n_theta=2, n_u=1)
