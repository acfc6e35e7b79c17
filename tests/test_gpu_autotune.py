"""Autotuner (tprf_set_autotune): measure mode picks launch shapes on the first
call of each shape, records them as wisdom, and leaves every result unchanged."""
import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _chain(d):
    import tprf_gb300 as T
    from tprf_gb300.tight_binding import ek_tensor
    e_k = T.Gf(mesh=T.MeshBrZone(dims=d["dims"]), data=ek_tensor(d["hoppings"], d["dims"], device="cuda"))
    g0 = T.lattice_dyson_g0_wk(d["mu"], e_k, T.MeshImFreq(d["beta"], "Fermion", d["n_max"]))
    chi0 = T.imtime_bubble_chi0_wk(g0, nw=d["nw"], verbose=False)
    chi = T.solve_rpa_PH(chi0, d["U"])
    torch.cuda.synchronize()
    return chi0.data.clone(), chi.data.clone()


def test_measure_mode_records_wisdom_and_keeps_results(cuda_lib, tmp_path):
    from tprf_gb300 import tuning, workloads
    cases = [workloads.config("cfg0", dims=(8, 8, 1), n_max=40, nw=12),
             workloads.config("cfg1", dims=(6, 6, 4), n_max=24, nw=8)]  # nb = 3: the RPA group kernel
    tuning.set_autotune(False)
    tuning.clear_wisdom()
    ref = [_chain(d) for d in cases]
    try:
        tuning.set_autotune(True)
        tuned = [_chain(d) for d in cases]
        n = tuning.wisdom_entries()
        assert n >= 4, n  # iv -> tau, fused bubble + tau -> iw (x2 shapes), RPA group kernel
        path = tmp_path / "wisdom.txt"
        tuning.save_wisdom(path)
        text = path.read_text()
        for kernel in ("/nu_to_tau/", "/tau_to_w/", "/rpa_group/"):
            assert kernel in text, text
        again = [_chain(d) for d in cases]  # wisdom hits: no new entries
        assert tuning.wisdom_entries() == n
        tuning.set_autotune(False)
        tuning.clear_wisdom()
        tuning.load_wisdom(path)
        loaded = [_chain(d) for d in cases]
        for (c0, c), runs in zip(ref, zip(tuned, again, loaded)):
            for t0, t in runs:
                assert rel_err(t0, c0) < 1e-13 and rel_err(t, c) < 1e-13
    finally:
        tuning.set_autotune(False)
        tuning.clear_wisdom()


def _device_prefix():
    p = torch.cuda.get_device_properties(0)
    return f"sm{p.major}{p.minor}x{p.multi_processor_count}"


def test_every_rpa_group_size_gives_the_same_chi(cuda_lib, tmp_path):
    """The RPA group kernel with 8, 9, 16 and 32 lanes per point (forced through
    wisdom files) gives the same chi, in double-float and in FP64 arithmetic,
    including points re-solved in FP64 (a near-singular subset)."""
    from tprf_gb300 import _native, tuning
    from tprf_gb300.workloads import kanamori_spin_vertex
    nb, n = 3, 20000
    rng = np.random.default_rng(7)
    chi0 = 0.2 * (rng.standard_normal((n, nb ** 4)) + 1j * rng.standard_normal((n, nb ** 4)))
    U = kanamori_spin_vertex(nb, 2.3, 0.4)
    Ug = U.reshape(nb, nb, nb, nb).transpose(0, 1, 3, 2).reshape(nb * nb, nb * nb)
    # points 0..99: chi0 = (I - eps) Ug^-1 grouped, so I - chi0 Ug is nearly singular
    inv = np.linalg.inv(Ug)
    for i in range(100):
        m = (np.eye(nb * nb) - 1e-3 * rng.standard_normal((nb * nb, nb * nb))) @ inv
        chi0[i] = m.reshape(nb, nb, nb, nb).transpose(0, 1, 3, 2).reshape(-1)
    x = torch.as_tensor(chi0, device="cuda").contiguous()
    u = torch.as_tensor(U, dtype=torch.complex128, device="cuda").contiguous()
    lib = cuda_lib
    out = {}
    try:
        for arith in (0, 1):
            _native.check(lib.tprf_set_arithmetic(arith))
            for lanes in (8, 9, 16, 32):
                tuning.set_autotune(False)
                tuning.clear_wisdom()
                w = tmp_path / f"w{lanes}.txt"
                w.write_text(f"{_device_prefix()}/rpa_group/{arith}/{nb} {lanes}\n")
                tuning.load_wisdom(w)
                chi = torch.empty_like(x)
                _native.check(lib.tprf_solve_rpa_PH(n, nb, x.data_ptr(), u.data_ptr(), chi.data_ptr(), None))
                torch.cuda.synchronize()
                out[(arith, lanes)] = chi.cpu().numpy()
    finally:
        lib.tprf_set_arithmetic(0)
        tuning.clear_wisdom()
    ref = out[(1, 8)]
    for key, chi in out.items():
        assert rel_err(chi, ref) < 1e-11, key
        assert rel_err(chi, out[(key[0], 8)]) < 1e-14, key



@pytest.mark.parametrize("dims,n_target", [((32, 32, 4), 9), ((16, 8, 1), 81), ((8, 8, 2), 1), ((4, 8, 1), 5)])
def test_tma_plane_pass_matches_the_plain_pass_and_numpy(cuda_lib, tmp_path, dims, n_target):
    """The TMA-staged plane pass of the lattice FFT (forced through wisdom with
    each tile size it accepts) gives the plain pass's transform, in place and out
    of place, both directions, against numpy."""
    from tprf_gb300 import _native, tuning
    rng = np.random.default_rng(3)
    n_w, nk = 3, int(np.prod(dims))
    x = rng.standard_normal((n_w, nk, n_target)) + 1j * rng.standard_normal((n_w, nk, n_target))
    xd = torch.as_tensor(x, device="cuda").contiguous()
    nontriv = [d for d in dims if d > 1]
    n1, n2 = nontriv[-2], nontriv[-1]
    lib = cuda_lib
    ref_f = np.fft.fftn(x.reshape((n_w,) + dims + (n_target,)), axes=(1, 2, 3)).reshape(x.shape) / nk
    ref_b = np.fft.ifftn(x.reshape((n_w,) + dims + (n_target,)), axes=(1, 2, 3)).reshape(x.shape) * nk
    try:
        for nt in (0, 1, 2, 4, 8, 16):
            tuning.set_autotune(False)
            tuning.clear_wisdom()
            w = tmp_path / f"p{nt}.txt"
            w.write_text(f"{_device_prefix()}/lattice_plane_tma/0/{n1}/{n2}/{n_target} {nt}\n")
            tuning.load_wisdom(w)
            for fn, ref in ((lib.tprf_fourier_wk_to_wr, ref_f), (lib.tprf_fourier_wr_to_wk, ref_b)):
                out = torch.empty_like(xd)
                _native.check(fn(n_w, _native.dims3(dims), n_target, xd.data_ptr(), out.data_ptr(), None))
                inplace = xd.clone()
                _native.check(fn(n_w, _native.dims3(dims), n_target, inplace.data_ptr(), inplace.data_ptr(), None))
                torch.cuda.synchronize()
                assert rel_err(out, ref) < 1e-13, (nt, fn)
                assert rel_err(inplace, ref) < 1e-13, (nt, fn)
    finally:
        tuning.clear_wisdom()


def test_tma_plane_wait_that_runs_out_is_reported(cuda_lib, tmp_path):
    """A wait of the TMA-staged plane pass on its tile copies that runs out (limit
    0 ns: every wait gives up at its first check) sets the device error word, read
    back as a timeout; the blocks let their copies in flight land before leaving,
    so the context stays usable and the next call, with the default limit, is
    correct."""
    from tprf_gb300 import _native, tuning
    dims, n_target, n_w = (16, 8, 1), 81, 2
    rng = np.random.default_rng(9)
    x = rng.standard_normal((n_w, 128, n_target)) + 1j * rng.standard_normal((n_w, 128, n_target))
    xd = torch.as_tensor(x, device="cuda").contiguous()
    ref = np.fft.fftn(x.reshape((n_w,) + dims + (n_target,)), axes=(1, 2, 3)).reshape(x.shape) / 128
    lib = cuda_lib
    try:
        tuning.set_autotune(False)
        tuning.clear_wisdom()
        w = tmp_path / "tma.txt"
        w.write_text(f"{_device_prefix()}/lattice_plane_tma/0/16/8/{n_target} 1\n")
        tuning.load_wisdom(w)
        out = torch.empty_like(xd)
        _native.check(lib.tprf_set_device_wait_limit_ns(0))
        _native.check(lib.tprf_fourier_wk_to_wr(n_w, _native.dims3(dims), n_target, xd.data_ptr(), out.data_ptr(),
                                                None))
        torch.cuda.synchronize()
        st = lib.tprf_check_device_status(None)
        assert st != 0 and "timed out" in lib.tprf_last_error().decode()
        _native.check(lib.tprf_set_device_wait_limit_ns(200_000_000))
        _native.check(lib.tprf_fourier_wk_to_wr(n_w, _native.dims3(dims), n_target, xd.data_ptr(), out.data_ptr(),
                                                None))
        torch.cuda.synchronize()
        assert lib.tprf_check_device_status(None) == 0
        assert rel_err(out, ref) < 1e-13
    finally:
        lib.tprf_set_device_wait_limit_ns(200_000_000)
        tuning.clear_wisdom()


def test_every_fft_radix_order_gives_the_same_chain(cuda_lib, tmp_path):
    """The radix orders the autotuner chooses among for the Matsubara transforms
    (forced one after the other through wisdom files rewritten from a measure-mode
    run) give the same chi0, against the oracle. L = 3072 = 2^10 3 has four
    distinct orders: 8 8 8 2 3, 4 4 4 4 4 3, 3 8 8 8 2, 2 8 8 8 3."""
    import oracle as O
    import tprf_gb300 as T
    from conftest import PARITY_RTOL
    from tprf_gb300 import tuning
    dims, beta, n_max, nw = (4, 4, 1), 30.0, 512, 24
    hop = {(1, 0): np.array([[-1.0, 0.3], [0.3, -0.7]]), (0, 1): np.array([[-0.8, 0.1], [0.1, -1.0]])}
    hop.update({(-R[0], -R[1]): t.T for R, t in list(hop.items())})
    ek = O.ek_from_hoppings(hop, dims)
    ref = O.imtime_bubble_chi0_wk(O.lattice_dyson_g0_wk(0.0, ek, beta, n_max), beta, dims, nw=nw)
    g0 = T.lattice_dyson_g0_wk(0.0, T.Gf(mesh=T.MeshBrZone(dims=dims), data=ek), T.MeshImFreq(beta, "Fermion", n_max))
    try:
        tuning.clear_wisdom()
        tuning.set_autotune(True)
        T.imtime_bubble_chi0_wk(g0, nw=nw, verbose=False)
        tuning.set_autotune(False)
        path = tmp_path / "measured.txt"
        tuning.save_wisdom(path)
        lines = path.read_text().splitlines()
        assert any("/tau_to_w_radix/" in ln for ln in lines) and any("/nu_to_tau_radix/" in ln for ln in lines)
        outs = []
        for v in range(4):
            forced = [ln.split()[0] + f" {v}" if "_radix/" in ln else ln for ln in lines]
            w = tmp_path / f"radix{v}.txt"
            w.write_text("\n".join(forced) + "\n")
            tuning.clear_wisdom()
            tuning.load_wisdom(w)
            chi0 = T.imtime_bubble_chi0_wk(g0, nw=nw, verbose=False).data
            torch.cuda.synchronize()
            assert rel_err(chi0, ref) < PARITY_RTOL, v
            outs.append(chi0.clone())
        for v in range(1, 4):
            assert rel_err(outs[v], outs[0]) < 1e-13, v
    finally:
        tuning.set_autotune(False)
        tuning.clear_wisdom()
