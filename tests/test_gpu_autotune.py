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
