"""CPU tests of the C-ABI library: it loads, exports what include/tprf_gb300.h
declares, and its host-only logic (argument checks, tail-fit definition,
Vandermonde table) agrees with the oracle. No kernel is launched."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from tprf_gb300.build import build_library
    build_library()
    from tprf_gb300 import _native
    return _native.lib()


def declared_functions():
    text = open(os.path.join(ROOT, "include", "tprf_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tprf_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    from tprf_gb300 import _native
    names = declared_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), f"{name} declared but not exported"
        assert name in _native.SIGNATURES, f"{name} has no ctypes signature"


def test_status_strings(lib):
    assert lib.tprf_version().decode() == "0.1.0"
    assert lib.tprf_status_string(0).decode() == "ok"
    assert "tail" in lib.tprf_status_string(-4).decode()
    assert "double-float range" in lib.tprf_status_string(-9).decode()


def test_tail_fit_matrix_matches_oracle(lib):
    for beta, n_max in [(10.0, 64), (20.0, 256), (40.0, 512), (5.0, 32), (0.544, 20), (2.0, 3)]:
        nf, nm = ctypes.c_int(), ctypes.c_int()
        assert lib.tprf_tail_fit_matrix(beta, n_max, 0, ctypes.byref(nf), ctypes.byref(nm), None, None) == 0
        rows = (ctypes.c_int * nf.value)()
        F = (ctypes.c_double * (2 * nf.value * nm.value))()
        assert lib.tprf_tail_fit_matrix(beta, n_max, nf.value * nm.value, ctypes.byref(nf), ctypes.byref(nm),
                                        rows, F) == 0
        idx, Fo, _ = O.tail_fit_matrix(beta, n_max)
        assert np.array_equal(np.array(rows[:]), idx)
        Fc = np.frombuffer(F, dtype=np.complex128).reshape(nm.value, nf.value)
        assert np.abs(Fc - Fo).max() <= 1e-10 * np.abs(Fo).max()


def test_bosonic_tail_fit_matrix_matches_oracle(lib):
    """The bosonic mesh's fit (chi_tr_from_chi_wr) follows the same definition in both."""
    for beta, nw in [(10.0, 64), (20.0, 256), (5.0, 33), (40.0, 128), (2.0, 12)]:
        nf, nm = ctypes.c_int(), ctypes.c_int()
        assert lib.tprf_tail_fit_matrix_stat(beta, nw, 0, 0, ctypes.byref(nf), ctypes.byref(nm), None, None) == 0
        rows = (ctypes.c_int * nf.value)()
        F = (ctypes.c_double * (2 * nf.value * nm.value))()
        assert lib.tprf_tail_fit_matrix_stat(beta, nw, 0, nf.value * nm.value, ctypes.byref(nf), ctypes.byref(nm),
                                             rows, F) == 0
        idx, Fo, _ = O.tail_fit_matrix(beta, nw, "Boson")
        assert np.array_equal(np.array(rows[:]), idx)
        assert 0 not in idx - (nw - 1)  # iw = 0 is never a fit point
        Fc = np.frombuffer(F, dtype=np.complex128).reshape(nm.value, nf.value)
        assert np.abs(Fc - Fo).max() <= 1e-10 * np.abs(Fo).max()


def test_vandermonde_inverse_bitwise(lib):
    v = (ctypes.c_double * 64)()
    lib.tprf_vandermonde_inverse8(v)
    assert np.array_equal(np.array(v[:]).reshape(8, 8), O.vandermonde_inverse(8))


def test_fit_derivative_rows_bitwise(lib):
    """The kernels' fit_derivatives constants are the oracle's (the reference's table rows)."""
    v = (ctypes.c_double * 16)()
    lib.tprf_fit_derivative_rows(v)
    assert np.array_equal(np.array(v[:]).reshape(2, 8), O.FIT_DERIVATIVE_ROWS)


def test_argument_errors_are_reported_without_a_gpu(lib):
    from tprf_gb300 import _native
    fake = ctypes.c_void_p(0x1000)
    # time mesh shorter than twice the frequency mesh (fourier_matsubara.cpp:128-131)
    st = lib.tprf_fourier_wr_to_tr(1.0, 10, 15, 4, 1, fake, None, fake, None)
    assert st == -3 and "twice" in lib.tprf_last_error().decode()
    st = lib.tprf_chi_wr_from_chi_tr(1.0, 21, 11, 4, 1, fake, fake, None)
    assert st == -3
    assert lib.tprf_solve_rpa_PH(0, 2, fake, fake, fake, None) == -1
    assert lib.tprf_lattice_dyson_g_wk(-1.0, 4, 4, 2, 0.0, fake, None, 0, fake, None) == -1
    assert lib.tprf_fourier_wk_to_wr(1, _native.dims3((0, 1, 1)), 1, fake, fake, None) == -1
    assert lib.tprf_imtime_bubble_chi0_wk(1.0, 4, 25, 2, _native.dims3((2, 2, 1)), 2, fake, None, fake, fake, 16,
                                          None) == -7
    with pytest.raises(_native.TprfError):
        _native.check(lib.tprf_solve_rpa_PH(0, 2, fake, fake, fake, None), "solve_rpa_PH")
    # streamed RPA: a workspace smaller than one chunk is rejected before any CUDA call
    assert lib.tprf_solve_rpa_PH_to_host_workspace_bytes(10, 3, 2) == 2 * 10 * 81 * 16 + 256
    assert lib.tprf_solve_rpa_PH_to_host(100, 3, fake, fake, fake, 10, fake, 1000, None) == -1
    assert "chunk" in lib.tprf_last_error().decode()
    # a fixed link / host split outside [0, 1] (checked before the device is touched)
    for f in (-0.1, 1.5, float("nan")):
        assert lib.tprf_set_host_fill_fraction(f) == -1
    assert "[0, 1]" in lib.tprf_last_error().decode()


def test_workspace_size(lib):
    from tprf_gb300 import _native
    n = lib.tprf_imtime_bubble_workspace_bytes(256, -1, _native.dims3((32, 32, 32)), 3)
    # G(iv, r), G(tau, r) and its double-float copy, the real-input test words, alignment
    expect = (512 + 2 * 1537) * 32768 * 9 * 16 + 512
    assert n == expect


def test_meshes():
    from tprf_gb300.mesh import MeshBrZone, MeshImFreq, MeshImTime, MeshProduct
    wf = MeshImFreq(10.0, "Fermion", 64)
    wb = MeshImFreq(10.0, "Boson", 64)
    assert len(wf) == 128 and len(wb) == 127
    np.testing.assert_allclose(wf.values(), O.fermionic_iw(10.0, 64))
    np.testing.assert_allclose(wb.values(), O.bosonic_iw(10.0, 64))
    np.testing.assert_allclose(MeshImTime(10.0, "Fermion", 385).values(), O.tau_points(10.0, 385))
    k = MeshBrZone(dims=(4, 2))
    assert k.dims == (4, 2, 1) and len(k) == 8
    np.testing.assert_allclose(k.values(), O.kpoints((4, 2, 1)))
    assert len(MeshProduct(wf, k)) == 128 * 8


def test_autotune_wisdom_file_round_trip(lib, tmp_path):
    """Wisdom files (host-only): load, count, save, reload; malformed files are refused."""
    from tprf_gb300 import tuning
    from tprf_gb300._native import TprfError
    tuning.clear_wisdom()
    src = tmp_path / "w.txt"
    src.write_text("# comment\nsm103x152/tau_to_w/0/1536/256/0/13 4\nsm103x152/rpa_group/0/3 8\n")
    tuning.load_wisdom(src)
    assert tuning.wisdom_entries() == 2
    out = tmp_path / "out.txt"
    tuning.save_wisdom(out)
    lines = [ln for ln in out.read_text().splitlines() if not ln.startswith("#")]
    assert sorted(lines) == ["sm103x152/rpa_group/0/3 8", "sm103x152/tau_to_w/0/1536/256/0/13 4"]
    tuning.clear_wisdom()
    assert tuning.wisdom_entries() == 0
    tuning.load_wisdom(out)
    assert tuning.wisdom_entries() == 2
    bad = tmp_path / "bad.txt"
    bad.write_text("only_a_key\n")
    with pytest.raises(TprfError, match="malformed line 1"):
        tuning.load_wisdom(bad)
    with pytest.raises(TprfError, match="cannot read"):
        tuning.load_wisdom(tmp_path / "missing.txt")
    assert lib.tprf_set_autotune(2) != 0
    assert not tuning.autotune_enabled()
    tuning.clear_wisdom()


def test_tuned_block_loads_and_writes_back_the_wisdom(lib, tmp_path):
    """tuning.tuned(path): loads the file, turns measure mode on for the block and
    back off after it, and writes every choice back (host-only)."""
    from tprf_gb300 import tuning
    tuning.clear_wisdom()
    tuning.set_autotune(False)
    path = tmp_path / "w.txt"
    path.write_text("sm103x152/rpa_group/0/3 9\n")
    with tuning.tuned(path):
        assert tuning.autotune_enabled()
        assert tuning.wisdom_entries() == 1
    assert not tuning.autotune_enabled()
    assert "sm103x152/rpa_group/0/3 9" in path.read_text().splitlines()
    tuning.clear_wisdom()
    with tuning.tuned(tmp_path / "new.txt", measure=False):  # no file yet: nothing loaded
        assert not tuning.autotune_enabled() and tuning.wisdom_entries() == 0
    assert (tmp_path / "new.txt").exists()
