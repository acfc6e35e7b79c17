"""tprf_gb300: GB300-native imaginary-time bubble + RPA path of TRIQS/TPRF.

The compute path is the CUDA library ``_lib/libtprf_gb300.so`` (C ABI in
``include/tprf_gb300.h``); this package mirrors the reference's Python entry
points on top of it. There is no CPU fallback.
"""
from .gf import Gf
from .mesh import MeshBrZone, MeshCycLat, MeshImFreq, MeshImTime, MeshProduct
from .lattice import (chi0_tr_from_grt_PH, chi0_w0r_from_grt_PH, chi0_wr_from_grt_PH, chi_tr_from_chi_wr,
                      chi_w0r_from_chi_tr, chi_wk_from_chi_wr, chi_wr_from_chi_tr, chi_wr_from_chi_wk, fourier_tr_to_wr,
                      fourier_wk_to_wr, fourier_wr_to_tr, fourier_wr_to_wk, lattice_dyson_g0_wk, lattice_dyson_g_wk,
                      lindhard_chi00, solve_rpa_PH, split_into_dynamic_wk_and_constant_k)
from .gw import bubble_PI_wk, dynamical_screened_interaction_W, gw_dynamic_sigma
from .lattice_utils import imtime_bubble_chi0_wk
from ._native import TprfError

__version__ = "0.1.0"
