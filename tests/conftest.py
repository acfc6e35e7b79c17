import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# Relative parity bar of the CUDA path against the FP64 oracle: max-abs error
# over the whole tensor divided by the tensor's max-abs value.
PARITY_RTOL = 1e-10


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built tprf_gb300 library")


@pytest.fixture(scope="session")
def cuda_lib():
    """The CUDA library, built if needed; skips only when no GPU is present."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tprf_gb300.build import build_library
    build_library()
    from tprf_gb300 import _native
    return _native.lib()


def rel_err(a, b):
    import numpy as np
    a = a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)
    b = b.detach().cpu().numpy() if hasattr(b, "detach") else np.asarray(b)
    den = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / den)
