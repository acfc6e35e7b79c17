"""Batched execution (tprf_batch_*): one graph launch over many uneven instances
gives, instance by instance, what the single-instance path gives, and what the
oracle gives."""
import numpy as np
import pytest
import torch

import oracle as O
from conftest import PARITY_RTOL, rel_err

pytestmark = pytest.mark.gpu


def _make(insts):
    from tprf_gb300.batch import RPAInstance
    from tprf_gb300.tight_binding import ek_tensor
    out = []
    for d in insts:
        out.append(RPAInstance(e_k=ek_tensor(d["hoppings"], d["dims"]), U=d["U"], dims=d["dims"], beta=d["beta"],
                               mu=d["mu"], n_max=d["n_max"], nw=d["nw"]))
    return out


def test_batch_matches_single_instance_path_and_oracle(cuda_lib):
    import tprf_gb300 as T
    from tprf_gb300 import workloads
    from tprf_gb300.batch import BatchedRPA
    specs = workloads.batched_instances(12, seed=3)
    for d in specs:  # keep the oracle fast: small meshes
        d["dims"] = (int(min(d["dims"][0], 16)),) * 2 + (1,)
        d["n_max"] = d["nw"] = int(min(d["n_max"], 64))
    specs[0]["nw"] = 1  # one instance through the static branch
    batch = BatchedRPA(_make(specs), n_streams=4)
    for rep in range(2):
        batch.run()
        torch.cuda.synchronize()
        for a, d in zip(batch.instances, specs):
            e_k = T.Gf(mesh=T.MeshBrZone(dims=d["dims"]), data=a.e_k)
            g0 = T.lattice_dyson_g0_wk(d["mu"], e_k, T.MeshImFreq(d["beta"], "Fermion", d["n_max"]))
            single = T.solve_rpa_PH(T.imtime_bubble_chi0_wk(g0, nw=d["nw"], verbose=False), d["U"])
            assert torch.equal(single.data, a.chi), "batched and single-instance results differ"
            ek = O.ek_from_hoppings(d["hoppings"], d["dims"])
            ref0 = O.imtime_bubble_chi0_wk(O.lattice_dyson_g0_wk(d["mu"], ek, d["beta"], d["n_max"]), d["beta"],
                                           d["dims"], nw=d["nw"])
            assert rel_err(a.chi, O.solve_rpa_PH(ref0, d["U"])) < PARITY_RTOL
    batch.close()


def test_batch_rejects_bad_instance(cuda_lib):
    from tprf_gb300.batch import BatchedRPA, RPAInstance
    from tprf_gb300.tight_binding import ek_tensor
    bad = RPAInstance(e_k=ek_tensor({(1, 0): -np.eye(1), (-1, 0): -np.eye(1)}, (4, 4, 1)), U=np.ones((1, 1, 1, 1)),
                      dims=(4, 4, 1), beta=1.0, mu=0.0, n_max=8, nw=8, n_tau=10)  # time mesh too short
    with pytest.raises(RuntimeError, match="time mesh"):
        BatchedRPA([bad])


def test_batch_gradients_match_dense_cpu_autograd(cuda_lib):
    """tprf_batch_grad_*: every instance's U, e(k) and t(R) gradients from one
    backward graph launch against torch.autograd through the dense FP64 CPU
    restatement, on two runs in a row (graph replay)."""
    from oracle import torch_chain as TC
    from tprf_gb300 import workloads
    from tprf_gb300.batch import BatchedRPAGrad
    specs = workloads.batched_instances(6, seed=5)
    for i, d in enumerate(specs):  # small meshes keep the dense reference fast
        d["dims"] = ((4, 6, 8)[i % 3], 6, 1)
        d["n_max"] = (16, 20, 24)[i % 3]
        d["nw"] = (2, 5, 8)[i % 3]
    batch = BatchedRPAGrad(_make(specs), n_streams=3)
    rng = np.random.default_rng(11)
    for rep in range(2):
        w = rng.standard_normal(batch.chi_grad_flat.numel()) + 1j * rng.standard_normal(batch.chi_grad_flat.numel())
        batch.forward()
        batch.backward(torch.as_tensor(w, device="cuda"))
        torch.cuda.synchronize()
        for i, (a, d) in enumerate(zip(batch.instances, specs)):
            e_k = a.e_k.detach().cpu().clone().requires_grad_(True)
            U = torch.as_tensor(d["U"], dtype=torch.complex128).clone().requires_grad_(True)
            chi = TC.chi_rpa(e_k, U, d["dims"], d["beta"], d["mu"], d["n_max"], d["nw"])
            assert rel_err(a.chi, chi.detach().reshape(a.chi.shape).numpy()) < PARITY_RTOL
            chi.backward(batch.chi_grad[i].cpu().reshape(chi.shape))
            assert rel_err(batch.U_grad[i], U.grad.numpy()) < 1e-9, i
            assert rel_err(batch.e_grad[i], e_k.grad.numpy()) < 1e-9, i
            t_ref = np.fft.fftn(e_k.grad.numpy().reshape(tuple(d["dims"]) + e_k.shape[1:]), axes=(0, 1, 2))
            assert rel_err(batch.t_grad[i], t_ref.reshape(e_k.shape)) < 1e-9, i
    batch.close()
