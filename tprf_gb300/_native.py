"""ctypes binding of the C ABI in ``include/tprf_gb300.h``.

The CUDA library is the only compute path: if it is missing or cannot be
loaded, every call raises. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libtprf_gb300.so")
_lock = threading.Lock()
_lib = None

c_int, c_long, c_double, c_void_p, c_size_t = ctypes.c_int, ctypes.c_long, ctypes.c_double, ctypes.c_void_p, ctypes.c_size_t
c_int3 = ctypes.c_int * 3


class Instance(ctypes.Structure):
    """C layout of tprf_instance (include/tprf_gb300.h)."""
    _fields_ = [("beta", ctypes.c_double), ("mu", ctypes.c_double), ("n_iw", ctypes.c_int), ("n_tau", ctypes.c_int),
                ("nw", ctypes.c_int), ("nb", ctypes.c_int), ("dims", ctypes.c_int * 3), ("e_k", ctypes.c_void_p),
                ("U", ctypes.c_void_p), ("chi", ctypes.c_void_p)]


class GradInstance(ctypes.Structure):
    """C layout of tprf_grad_instance (include/tprf_gb300.h)."""
    _fields_ = [("inst", Instance), ("chi0", ctypes.c_void_p), ("chi_grad", ctypes.c_void_p),
                ("U_grad", ctypes.c_void_p), ("e_grad", ctypes.c_void_p), ("t_grad", ctypes.c_void_p)]


# name -> (restype, argtypes); mirrors include/tprf_gb300.h
SIGNATURES = {
    "tprf_status_string": (ctypes.c_char_p, [c_int]),
    "tprf_last_error": (ctypes.c_char_p, []),
    "tprf_version": (ctypes.c_char_p, []),
    "tprf_set_sync_checks": (None, [c_int]),
    "tprf_check_device_status": (c_int, [c_void_p]),
    "tprf_kernel_launches": (ctypes.c_ulonglong, []),
    "tprf_set_device_wait_limit_ns": (c_int, [ctypes.c_longlong]),
    "tprf_set_arithmetic": (c_int, [c_int]),
    "tprf_get_arithmetic": (c_int, []),
    "tprf_measure_fp64_tflops": (c_int, [ctypes.POINTER(c_double), c_void_p, c_size_t, c_void_p]),
    "tprf_tail_fit_matrix": (c_int, [c_double, c_int, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                                     ctypes.POINTER(c_int), ctypes.POINTER(c_double)]),
    "tprf_vandermonde_inverse8": (None, [ctypes.POINTER(c_double)]),
    "tprf_fit_derivative_rows": (None, [ctypes.POINTER(c_double)]),
    "tprf_lattice_dyson_g_wk": (c_int, [c_double, c_int, c_long, c_int, c_double, c_void_p, c_void_p, c_int,
                                        c_void_p, c_void_p]),
    "tprf_fourier_wk_to_wr": (c_int, [c_long, c_int3, c_long, c_void_p, c_void_p, c_void_p]),
    "tprf_fourier_wr_to_wk": (c_int, [c_long, c_int3, c_long, c_void_p, c_void_p, c_void_p]),
    "tprf_fourier_lattice_noalloc": (c_int, [c_int, c_long, c_int3, c_long, c_void_p, c_void_p, c_void_p]),
    "tprf_fourier_wr_to_tr": (c_int, [c_double, c_int, c_int, c_long, c_long, c_void_p, c_void_p, c_void_p,
                                      c_void_p]),
    "tprf_chi0_tr_from_grt_PH": (c_int, [c_int, c_int3, c_int, c_void_p, c_void_p, c_void_p]),
    "tprf_chi0_wr_from_grt_PH": (c_int, [c_double, c_int, c_int, c_int3, c_int, c_void_p, c_void_p, c_void_p]),
    "tprf_chi0_w0r_from_grt_PH": (c_int, [c_double, c_int, c_int3, c_int, c_void_p, c_void_p, c_void_p]),
    "tprf_chi_wr_from_chi_tr": (c_int, [c_double, c_int, c_int, c_long, c_long, c_void_p, c_void_p, c_void_p]),
    "tprf_chi_w0r_from_chi_tr": (c_int, [c_double, c_int, c_long, c_long, c_void_p, c_void_p, c_void_p]),
    "tprf_solve_rpa_PH": (c_int, [c_long, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tprf_solve_rpa_PH_wk": (c_int, [c_int, c_int3, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tprf_imtime_bubble_rpa_to_host_workspace_bytes": (c_size_t, [c_int, c_int, c_int, c_int3, c_int, c_int, c_int]),
    "tprf_imtime_bubble_rpa_to_host": (c_int, [c_double, c_int, c_int, c_int, c_int3, c_int, c_void_p, c_void_p,
                                               c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p, c_size_t,
                                               c_void_p]),
    "tprf_imtime_bubble_rpa_to_host_async": (c_int, [c_double, c_int, c_int, c_int, c_int3, c_int, c_void_p,
                                                     c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p,
                                                     c_size_t, c_void_p]),
    "tprf_imtime_bubble_rpa_to_host_join": (c_int, [c_void_p]),
    "tprf_imtime_bubble_rpa_to_host_last_d2h_bytes": (c_size_t, []),
    "tprf_imtime_bubble_rpa_to_host_last_stats": (c_int, [ctypes.POINTER(c_double), c_int]),
    "tprf_set_host_fill": (c_int, [c_int]),
    "tprf_set_host_fill_fraction": (c_int, [c_double]),
    "tprf_lindhard_chi00_workspace_bytes": (c_size_t, [c_long, c_int]),
    "tprf_lindhard_chi00": (c_int, [c_long, c_int3, c_int, c_void_p, c_double, c_double, c_int, c_void_p, c_void_p,
                                    c_size_t, c_void_p]),
    "tprf_gw_dynamic_sigma": (c_int, [c_long, c_long, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tprf_dynamical_screened_interaction_W": (c_int, [c_long, c_long, c_int, c_void_p, c_void_p, c_int, c_void_p,
                                                      c_void_p]),
    "tprf_split_into_dynamic_wk_and_constant_k": (c_int, [c_double, c_int, c_long, c_long, c_void_p, c_void_p,
                                                          c_void_p, c_void_p]),
    "tprf_fourier_tr_to_wr": (c_int, [c_double, c_int, c_int, c_long, c_long, c_void_p, c_void_p, c_void_p]),
    "tprf_chi_tr_from_chi_wr": (c_int, [c_double, c_int, c_int, c_long, c_long, c_void_p, c_void_p, c_void_p,
                                        c_void_p]),
    "tprf_tail_fit_matrix_stat": (c_int, [c_double, c_int, c_int, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                                          c_void_p, c_void_p]),
    "tprf_solve_rpa_PH_to_host_workspace_bytes": (c_size_t, [c_long, c_int, c_int]),
    "tprf_solve_rpa_PH_to_host": (c_int, [c_long, c_int, c_void_p, c_void_p, c_void_p, c_long, c_void_p, c_size_t,
                                          c_void_p]),
    "tprf_solve_rpa_PH_adjoint": (c_int, [c_long, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                          c_void_p]),
    "tprf_chi_wr_from_chi_tr_adjoint": (c_int, [c_double, c_int, c_int, c_long, c_long, c_void_p, c_void_p,
                                                c_void_p]),
    "tprf_chi0_tr_from_grt_PH_adjoint": (c_int, [c_int, c_int3, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tprf_chi0_wr_from_grt_PH_adjoint": (c_int, [c_double, c_int, c_int, c_int3, c_int, c_void_p, c_void_p, c_void_p,
                                                 c_void_p]),
    "tprf_fourier_wr_to_tr_adjoint": (c_int, [c_double, c_int, c_int, c_long, c_long, c_void_p, c_int, c_void_p,
                                              c_void_p]),
    "tprf_lattice_dyson_g_wk_adjoint": (c_int, [c_int, c_long, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tprf_batch_workspace_bytes": (c_size_t, [ctypes.POINTER(Instance), c_int, c_int]),
    "tprf_batch_create": (c_int, [ctypes.POINTER(Instance), c_int, c_int, c_void_p, c_size_t,
                                  ctypes.POINTER(c_void_p)]),
    "tprf_batch_run": (c_int, [c_void_p, c_void_p]),
    "tprf_batch_size": (c_int, [c_void_p]),
    "tprf_batch_destroy": (c_int, [c_void_p]),
    "tprf_set_autotune": (c_int, [c_int]),
    "tprf_get_autotune": (c_int, []),
    "tprf_autotune_entries": (c_int, []),
    "tprf_autotune_clear": (None, []),
    "tprf_autotune_save": (c_int, [ctypes.c_char_p]),
    "tprf_autotune_load": (c_int, [ctypes.c_char_p]),
    "tprf_batch_grad_workspace_bytes": (c_size_t, [ctypes.POINTER(GradInstance), c_int, c_int]),
    "tprf_batch_grad_create": (c_int, [ctypes.POINTER(GradInstance), c_int, c_int, c_void_p, c_size_t,
                                       ctypes.POINTER(c_void_p)]),
    "tprf_batch_backward": (c_int, [c_void_p, c_void_p]),
    "tprf_imtime_bubble_workspace_bytes": (c_size_t, [c_int, c_int, c_int3, c_int]),
    "tprf_imtime_bubble_chi0_wk": (c_int, [c_double, c_int, c_int, c_int, c_int3, c_int, c_void_p, c_void_p,
                                           c_void_p, c_void_p, c_size_t, c_void_p]),
    "tprf_imtime_bubble_chi0_wk_timed": (c_int, [c_double, c_int, c_int, c_int, c_int3, c_int, c_void_p, c_void_p,
                                                 c_void_p, c_void_p, c_size_t, ctypes.POINTER(c_void_p), c_void_p]),
}


class TprfError(RuntimeError):
    """Raised when a tprf_gb300 entry point returns a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


def library_path() -> str:
    return _LIB_PATH


def lib():
    """Load (once) and return the CUDA library; raise if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_LIB_PATH):
                raise RuntimeError(
                    f"tprf_gb300 CUDA library not found at {_LIB_PATH}; build it with "
                    "tprf_gb300.build.build_library() (there is no CPU fallback)")
            import torch  # noqa: F401  (load torch's CUDA runtime first so both share it)
            handle = ctypes.CDLL(_LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
    return _lib


def check(status: int, what: str = "") -> None:
    if status != 0:
        l = lib()
        msg = l.tprf_last_error().decode() or l.tprf_status_string(status).decode()
        raise TprfError(status, f"{what}: {msg}" if what else msg)


def dims3(dims) -> ctypes.Array:
    d = list(dims) + [1] * (3 - len(dims))
    return c_int3(*[int(x) for x in d[:3]])
