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
    """Central differences (h = 1e-6) of the loss in the first n_theta amplitudes
    and in the real and imaginary parts of the first n_u non-zero entries of U
    (None: all of them) against the adjoint gradients."""
    L, gt, gu = _gpu(model, theta0, U)
    h = 1e-6
    for a in range(len(theta0) if n_theta is None else n_theta):
        tp, tm = theta0.copy(), theta0.copy()
        tp[a] += h
        tm[a] -= h
        fd = (_gpu(model, tp, U, grad=False) - _gpu(model, tm, U, grad=False)) / (2 * h)
        assert abs(fd - gt[a]) <= rtol * max(abs(fd), np.abs(gt).max()), (a, fd, gt[a])
    flat = np.flatnonzero(np.abs(U.ravel()) > 0)
    flat = flat if n_u is None else flat[:n_u]
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
    """The differentiation configuration itself (2-orbital square lattice, 32 x 32,
    beta = 16, 128 fermionic / bosonic frequencies): every one of the 8 hopping
    amplitudes and every non-zero entry of the 4 x 4 vertex, real and imaginary
    directions."""
    from tprf_gb300.workloads import cfg3_model
    model, theta0, U = cfg3_model()
    assert len(theta0) == 8 and np.count_nonzero(U) > 0
    _fd_check(model, theta0, U, n_theta=None, n_u=None)


@pytest.mark.parametrize("nb,dims", [(1, (6, 5, 1)), (2, (4, 4, 2)), (3, (3, 3, 2))])
def test_fused_bubble_adjoint_equals_the_two_unfused_adjoints(cuda_lib, nb, dims):
    """tprf_chi0_wr_from_grt_PH_adjoint (the tau -> iw transpose and the bubble
    transpose in one kernel, chi0_grad(tau, r) never stored) equals the tau -> iw
    adjoint followed by the bubble adjoint, and is the adjoint of the forward
    fused bubble: <y, A g> = <A^H y, g>."""
    from tprf_gb300 import _native
    rng = np.random.default_rng(nb)
    beta, n_tau, nw = 6.0, 97, 9
    nk = int(np.prod(dims))
    crand = lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)  # noqa: E731
    g = torch.as_tensor(crand(n_tau, nk, nb, nb)).cuda()
    y = torch.as_tensor(crand(2 * nw - 1, nk, nb ** 4)).cuda()
    d3 = _native.dims3(dims)
    fused = torch.empty_like(g)
    _native.check(cuda_lib.tprf_chi0_wr_from_grt_PH_adjoint(beta, n_tau, nw, d3, nb, g.data_ptr(), y.data_ptr(),
                                                             fused.data_ptr(), None))
    ytr = torch.empty(n_tau, nk, nb ** 4, dtype=torch.complex128, device="cuda")
    _native.check(cuda_lib.tprf_chi_wr_from_chi_tr_adjoint(beta, n_tau, nw, nk, nb ** 4, y.data_ptr(), ytr.data_ptr(),
                                                            None))
    two = torch.empty_like(g)
    _native.check(cuda_lib.tprf_chi0_tr_from_grt_PH_adjoint(n_tau, d3, nb, g.data_ptr(), ytr.data_ptr(),
                                                             two.data_ptr(), None))
    torch.cuda.synchronize()
    assert rel_err(fused, two) < 1e-13
    # the forward map is bilinear in G (the product of G at tau and beta - tau), so
    # check the adjoint of its linearisation at g: d chi0 = A(g; dg) with
    # <y, A(g; dg)> = <A^H(g; y), dg>, A^H = the fused adjoint
    dg = torch.as_tensor(crand(n_tau, nk, nb, nb)).cuda()
    outp, outm = torch.empty_like(y), torch.empty_like(y)
    # Q(g) = B(g, g) is quadratic, so (Q(g + dg) - Q(g - dg)) / 2 = B(g, dg) + B(dg, g)
    # exactly for a unit step; a small step would only divide the forward's rounding
    # (about 1e-11 relative after the tail fit of random data) by the step
    for sign, out in ((1.0, outp), (-1.0, outm)):
        gs = (g + sign * dg).contiguous()
        _native.check(cuda_lib.tprf_chi0_wr_from_grt_PH(beta, n_tau, nw, d3, nb, gs.data_ptr(), out.data_ptr(), None))
    torch.cuda.synchronize()
    lin = (outp - outm) / 2
    lhs = torch.vdot(y.reshape(-1), lin.reshape(-1))
    rhs = torch.vdot(fused.reshape(-1), dg.reshape(-1))
    assert abs(complex(lhs - rhs)) <= 1e-9 * abs(complex(lhs))
