"""FP64 CPU oracle for the imaginary-time bubble + RPA path.

TEST INFRASTRUCTURE ONLY. This package is the checker that the CUDA path is
compared against. Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` may import it; the library package
``tprf_gb300`` never does, and never falls back to it.

Pinning status: the reference (TPRF 3.2 on TRIQS 3.2) cannot be built or
imported on this machine, so the oracle is a restatement of the cited
reference files. It is pinned against the known answers that the reference's
own tests use (analytic Lindhard bubble, the 1D density-of-states integral,
the Fazekas RPA closed forms, the matrix-RPA identities, round trips), stored
as fixtures under ``tests/golden/``. The TRIQS ``fit_tail`` least-squares
moment fit is third-party arithmetic that is not vendored; the oracle's
restatement of it is **parity unpinned** (see ``tail_fit_matrix``).
"""
from .tprf_oracle import *  # noqa: F401,F403
