"""The RPA adjoint kernel (tprf_solve_rpa_PH_adjoint) against torch's CPU
autograd of the dense FP64 solve, for every vertex size the kernel serves."""
import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nb,npts", [(1, 97), (2, 130), (3, 75), (4, 40), (5, 23), (6, 9)])
def test_rpa_adjoint_matches_cpu_autograd(cuda_lib, nb, npts):
    from oracle import torch_chain as TC
    from tprf_gb300 import _native
    rng = np.random.default_rng(70 + nb)
    c = lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)  # noqa: E731
    chi0 = 0.1 * c(npts, nb, nb, nb, nb)
    U = 0.4 * c(nb, nb, nb, nb)
    U[np.abs(U) < 0.3] = 0.0  # a sparse vertex, as Kanamori's
    Y = c(npts, nb, nb, nb, nb)
    x0 = torch.tensor(chi0, requires_grad=True)
    u = torch.tensor(U, requires_grad=True)
    chi_ref = TC.solve_rpa(x0, u)
    (chi_ref.conj() * torch.tensor(Y)).real.sum().backward()  # torch gradient w.r.t. chi: Y
    d = torch.device("cuda")
    dx0, du, dy = (torch.tensor(a, device=d) for a in (chi0, U, Y))
    chi = torch.empty_like(dx0)
    lib = _native.lib()
    s = torch.cuda.current_stream().cuda_stream
    _native.check(lib.tprf_solve_rpa_PH(npts, nb, dx0.data_ptr(), du.data_ptr(), chi.data_ptr(), s))
    g0 = torch.empty_like(dx0)
    gu = torch.zeros_like(du)
    # torch's gradient of Re<chi, Y> w.r.t. chi is Y
    _native.check(lib.tprf_solve_rpa_PH_adjoint(npts, nb, dx0.data_ptr(), du.data_ptr(), chi.data_ptr(),
                                                 dy.data_ptr(), g0.data_ptr(), gu.data_ptr(), s))
    torch.cuda.synchronize()
    assert rel_err(chi.cpu().numpy(), chi_ref.detach().numpy()) < 1e-10
    assert rel_err(g0.cpu().numpy(), x0.grad.numpy()) < 1e-10
    assert rel_err(gu.cpu().numpy(), u.grad.numpy()) < 1e-10
