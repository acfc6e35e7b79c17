"""The dense torch autograd reference equals the numpy oracle (forward), CPU only."""
import numpy as np
import torch

import oracle as O
from oracle import torch_chain as TC


def test_torch_chain_forward_equals_oracle():
    from tprf_gb300 import workloads
    dims, beta, mu, n_max, nw = (4, 4, 1), 5.0, 0.1, 16, 4
    hop = workloads.square_2orb(0)
    ek = O.ek_from_hoppings(hop, dims)
    U = workloads.kanamori_spin_vertex(2, 1.0, 0.1)
    ref = O.solve_rpa_PH(O.imtime_bubble_chi0_wk(O.lattice_dyson_g0_wk(mu, ek, beta, n_max), beta, dims, nw=nw), U)
    got = TC.chi_rpa(torch.as_tensor(ek), torch.as_tensor(U), dims, beta, mu, n_max, nw).detach().numpy()
    assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-12


def test_torch_chain_gradient_matches_finite_differences():
    from tprf_gb300 import workloads
    dims, beta, mu, n_max, nw = (4, 4, 1), 5.0, 0.1, 16, 4
    ek0 = torch.as_tensor(O.ek_from_hoppings(workloads.square_2orb(0), dims))
    U = torch.as_tensor(workloads.kanamori_spin_vertex(2, 1.0, 0.1))
    pert = torch.as_tensor(O.ek_from_hoppings({(1, 0): np.array([[0.3, 0.1], [0.0, -0.2]]),
                                               (-1, 0): np.array([[0.3, 0.0], [0.1, -0.2]])}, dims))

    def loss(t):
        chi = TC.chi_rpa(ek0 + t * pert, U, dims, beta, mu, n_max, nw)
        return (chi.abs() ** 2).sum()

    t = torch.zeros((), dtype=torch.float64, requires_grad=True)
    loss(t.to(torch.complex128)).backward()
    h = 1e-6
    fd = (loss(torch.tensor(h, dtype=torch.complex128)) - loss(torch.tensor(-h, dtype=torch.complex128))) / (2 * h)
    assert abs(t.grad.item() - fd.item()) < 1e-6 * max(1.0, abs(fd.item()))
