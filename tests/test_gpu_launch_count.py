"""tprf_kernel_launches: one count per kernel launch of the library, the kernel
count of a batch graph at each of its launches, nothing for the launches a
graph capture records."""
import numpy as np
import pytest
import torch

from test_gpu_batch import _make

pytestmark = pytest.mark.gpu


def test_direct_launches_are_counted_once(cuda_lib):
    from tprf_gb300 import _native
    rng = np.random.default_rng(0)
    nb, dims, nw = 2, (4, 4, 1), 3
    nk = int(np.prod(dims))
    chi0 = torch.as_tensor(0.05 * (rng.standard_normal((2 * nw - 1, nk, nb ** 4))
                                   + 1j * rng.standard_normal((2 * nw - 1, nk, nb ** 4)))).cuda()
    U = torch.as_tensor(np.eye(nb * nb).reshape((nb,) * 4) + 0j).cuda()
    out = torch.empty_like(chi0)
    lib = cuda_lib
    lib.tprf_set_autotune(0)
    n0 = lib.tprf_kernel_launches()
    _native.check(lib.tprf_solve_rpa_PH(chi0.shape[0] * nk, nb, chi0.data_ptr(), U.data_ptr(), out.data_ptr(), None))
    torch.cuda.synchronize()
    assert lib.tprf_kernel_launches() - n0 == 1  # one RPA kernel
    n1 = lib.tprf_kernel_launches()
    _native.check(lib.tprf_fourier_wk_to_wr(chi0.shape[0], _native.dims3(dims), nb ** 4, chi0.data_ptr(),
                                            out.data_ptr(), None))
    torch.cuda.synchronize()
    assert lib.tprf_kernel_launches() - n1 >= 1  # the lattice passes of a 4 x 4 mesh


def test_graph_kernels_are_counted_at_each_launch(cuda_lib):
    from tprf_gb300 import workloads
    from tprf_gb300.batch import BatchedRPA
    specs = workloads.batched_instances(4, seed=1)
    for d in specs:
        d["dims"] = (8, 8, 1)
        d["n_max"] = d["nw"] = 16
    lib = cuda_lib
    lib.tprf_set_autotune(0)  # no trial launches in the planning run
    n0 = lib.tprf_kernel_launches()
    batch = BatchedRPA(_make(specs), n_streams=2)  # plans eagerly, then captures
    torch.cuda.synchronize()
    n1 = lib.tprf_kernel_launches()
    batch.run()
    torch.cuda.synchronize()
    n2 = lib.tprf_kernel_launches()
    batch.run()
    torch.cuda.synchronize()
    n3 = lib.tprf_kernel_launches()
    per_run = n2 - n1
    # every instance runs Dyson, the chain and the RPA: at least 6 kernels each
    assert per_run >= 6 * len(specs)
    assert n3 - n2 == per_run
    # the eager planning run launches at most what one graph holds (the capture adds nothing)
    assert n1 - n0 <= per_run
    batch.close()
