"""The allocation-free lattice FFT, tprf_fourier_lattice_noalloc.

Some callers cannot let a library allocate device memory: applications that
give all device memory to their own pool allocator at start-up, or hosts
working within a fixed device-memory budget. For them the library offers one
entry point whose FFT tables sit in a static device array of the library
image instead of cudaMalloc'ed memory. These tests call it through the C ABI
and compare it with the regular entry points on two calls in a row (the second
call must not be affected by what the first left in the shared array), and
check that a request larger than the static array is refused before any work.
This file is collected last so that a failure here stops a -x run only after
every other test has run.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import PARITY_RTOL, rel_err

pytestmark = pytest.mark.gpu


def _call_regular(lib, native, forward, x, dims):
    out = torch.empty_like(x)
    fn = lib.tprf_fourier_wk_to_wr if forward else lib.tprf_fourier_wr_to_wk
    native.check(fn(x.shape[0], native.dims3(dims), x.shape[2], x.data_ptr(), out.data_ptr(), None))
    return out


def _call_noalloc(lib, native, forward, x, dims):
    out = torch.empty_like(x)
    native.check(lib.tprf_fourier_lattice_noalloc(1 if forward else 0, x.shape[0], native.dims3(dims), x.shape[2],
                                                  x.data_ptr(), out.data_ptr(), None), "fourier_lattice_noalloc")
    return out


@pytest.fixture(params=["df64", "fp64"])
def arithmetic(request, cuda_lib):
    """Both element types of the transform: double-float (default) and native FP64."""
    assert cuda_lib.tprf_set_arithmetic({"df64": 0, "fp64": 1}[request.param]) == 0
    yield request.param
    cuda_lib.tprf_set_arithmetic(0)


def _oracle(forward, x, dims):
    import oracle as O
    return O.fourier_wk_to_wr(x, dims) if forward else O.fourier_wr_to_wk(x, dims)


def test_noalloc_matches_regular_entry_points_twice_in_a_row(cuda_lib, arithmetic):
    from tprf_gb300 import _native
    rng = np.random.default_rng(5)
    cases = [((16, 16, 1), True), ((6, 10, 7), False), ((16, 16, 1), False), ((11, 4, 3), True)]
    for dims, forward in cases:
        nk = int(np.prod(dims))
        xh = rng.standard_normal((3, nk, 4)) + 1j * rng.standard_normal((3, nk, 4))
        x = torch.as_tensor(xh).cuda()
        ref = _call_regular(cuda_lib, _native, forward, x, dims)
        first = _call_noalloc(cuda_lib, _native, forward, x, dims)
        second = _call_noalloc(cuda_lib, _native, forward, x, dims)
        torch.cuda.synchronize()
        assert rel_err(first, ref) < PARITY_RTOL
        assert rel_err(second, ref) < PARITY_RTOL
        assert rel_err(first, _oracle(forward, xh, dims)) < PARITY_RTOL
        assert rel_err(second, _oracle(forward, xh, dims)) < PARITY_RTOL


def test_noalloc_allocates_no_device_memory(cuda_lib, arithmetic):
    """On mesh lengths no earlier call has planned (the regular entry points would
    allocate tables for them), two calls in a row leave the device's free memory
    and torch's reserve unchanged, and agree with the oracle."""
    from tprf_gb300 import _native
    rng = np.random.default_rng(17)
    warm = torch.zeros((1, 8, 1), dtype=torch.complex128, device="cuda")
    _call_noalloc(cuda_lib, _native, True, warm, (8, 1, 1))  # the device code is loaded
    dims = (23, 29, 1) if arithmetic == "df64" else (31, 37, 1)  # primes nothing else in the suite uses
    nk = int(np.prod(dims))
    xh = rng.standard_normal((2, nk, 3)) + 1j * rng.standard_normal((2, nk, 3))
    x = torch.as_tensor(xh).cuda()
    outs = [torch.empty_like(x) for _ in range(2)]
    torch.cuda.synchronize()
    free0, reserved0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_reserved()
    for out in outs:
        _native.check(cuda_lib.tprf_fourier_lattice_noalloc(1, 2, _native.dims3(dims), 3, x.data_ptr(),
                                                            out.data_ptr(), None), "fourier_lattice_noalloc")
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_reserved() == reserved0
    for out in outs:
        assert rel_err(out, _oracle(True, xh, dims)) < PARITY_RTOL


def test_noalloc_rejects_tables_beyond_the_static_array(cuda_lib):
    from tprf_gb300 import _native
    fake = ctypes.c_void_p(0x1000)  # never dereferenced: the size check comes first
    dims = (12000, 11999, 11998)    # 3 x 36 x ~12000 bytes of tables > 1 MiB
    st = cuda_lib.tprf_fourier_lattice_noalloc(1, 1, _native.dims3(dims), 1, fake, fake, None)
    assert st == -1
    assert "static scratch" in cuda_lib.tprf_last_error().decode()
    # one mesh length whose columns do not fit one CTA's shared memory (tables
    # 36 x 13000 bytes would fit the array)
    st = cuda_lib.tprf_fourier_lattice_noalloc(1, 1, _native.dims3((13000, 1, 1)), 1, fake, fake, None)
    assert st == -2
    assert "too long for one CTA" in cuda_lib.tprf_last_error().decode()
