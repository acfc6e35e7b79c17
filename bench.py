"""Benchmark of the imaginary-time bubble + RPA path on GB300.

One step = the whole path on the 3-orbital cubic workload (32^3 k, beta = 20,
256 fermionic / 256 bosonic Matsubara frequencies, 9 x 9 Kanamori vertex):
Dyson G0(iv, k) -> k->r -> iv->tau -> bubble fused with tau->iw -> r->q ->
RPA. The metric is (q, iw) points per second: (2 nw - 1) * N_k per step.

  value : device-resident inputs, preallocated buffers, C-ABI calls.
  e2e   : the public Python API (lattice_dyson_g0_wk, imtime_bubble_chi0_wk,
          solve_rpa_PH) from a pinned host e(k) to chi(iw, q) copied back
          into pinned host memory, both copies inside the timed region.

``--impl reference`` times the CPU implementation of the same path (the FP64
restatement of the reference, run on all host cores) on a bounded sample of
the same workload. With torchrun (N > 1) every rank runs an independent
replica (the path has no cross-instance exchange): weak scaling.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "RPA \u03c7(q,i\u03bd) points/s on 1 GB300 at \u22641e-10 rel err vs plain GPU path; % HBM peak"
UNIT = "points/s"
C16 = 16  # bytes per complex128


# ---------------------------------------------------------------------------
# algorithmic traffic and flops per stage: one read of each input and one write
# of each output, in the representation the stage hands on. On the real path
# (real hoppings: G(tau, r) real, G(-iv) = G(iv)^dagger, chi0(-w) from chi0(w))
# iv -> tau reads the frequencies v >= 0 and writes real G(tau, r) (8 bytes per
# element), the bubble writes the frequencies w >= 0 and r -> q reads those and
# writes all 2 nw - 1. On a three-dimensional mesh whose last two axes are
# powers of two, the bubble writes only the canonical orbital columns
# abcd <= dcba ((nb^4 + nb^2) / 2 of nb^4; compact_columns) and r -> q reads those.

def compact_columns(dims, nb, n_tau, nw, real=True):
    """Canonical orbital columns the bubble hands to r -> q on this workload (the
    library's compact path), or None where the full columns are used."""
    pow2 = lambda n: n >= 2 and n & (n - 1) == 0  # noqa: E731
    nc = (nb ** 4 + nb ** 2) // 2
    if (real and nw >= 2 and all(d > 1 for d in dims) and pow2(dims[1]) and pow2(dims[2])
            and max(dims[1], dims[2]) <= 256 and nw * nc <= (n_tau - 18) * nb * nb):
        return nc
    return None


def stage_model(nb, nk, n_nu, n_tau, nw, real=True, nc=None):
    nb2, nb4, nwt = nb * nb, nb ** 4, 2 * nw - 1
    L = n_tau - 1
    fft_flops = lambda n: 5.0 * n * math.log2(n) if n > 1 else 0.0  # noqa: E731
    g_tau = (8 if real else C16) * nb2 * nk * n_tau
    w_out = nw if real else nwt
    cols = nc or nb4  # the columns of chi0(w, r) the bubble writes
    return {
        "dyson": dict(bytes=C16 * nb2 * (n_nu + 1) * nk, flops=n_nu * nk * 8.0 * nb ** 3),
        "fft_k_to_r": dict(bytes=2 * C16 * nb2 * n_nu * nk, flops=n_nu * nb2 * fft_flops(nk)),
        "nu_to_tau": dict(bytes=C16 * nb2 * nk * (n_nu // 2 if real else n_nu) + g_tau,
                          flops=nk * nb2 * fft_flops(L)),
        "bubble_tau_to_w": dict(bytes=g_tau + C16 * cols * nk * w_out, flops=nk * nb4 * (6.0 * n_tau + fft_flops(L))),
        "fft_r_to_q": dict(bytes=C16 * nk * (cols * w_out + nb4 * nwt), flops=nwt * nb4 * fft_flops(nk)),
        "rpa": dict(bytes=2 * C16 * nb4 * nwt * nk, flops=nwt * nk * 8.0 * (nb2 ** 3 * 2 + nb2 ** 3 / 3.0)),
    }


# ---------------------------------------------------------------------------
# clocks sampled during the timed region

class ClockSampler:
    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# distributed helpers (replicas)

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value: float, world: int, device=None) -> float:
    """Max of a per-rank float over all ranks (identity for one rank)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int, device=None):
    if world > 1:
        import torch.distributed as dist
        if device is not None and device.type == "cuda":
            dist.barrier(device_ids=[device.index])
        else:
            dist.barrier()


# ---------------------------------------------------------------------------
# host placement of the end-to-end leg (NUMA nodes of the pinned buffer, the GPU
# and the library's host-fill threads), read from /proc and /sys

def _cpulist(text):
    out = []
    for part in text.strip().split(","):
        if "-" in part:
            a, b = part.split("-")
            out.extend(range(int(a), int(b) + 1))
        elif part:
            out.append(int(part))
    return out


def numa_nodes():
    base = "/sys/devices/system/node"
    nodes = {}
    try:
        for name in sorted(os.listdir(base)):
            if name.startswith("node") and name[4:].isdigit():
                with open(os.path.join(base, name, "cpulist")) as f:
                    cpus = _cpulist(f.read())
                if cpus:
                    nodes[int(name[4:])] = cpus
    except OSError:
        pass
    return nodes


def buffer_numa_pages(ptr):
    """{node: pages} of the mapping that holds host address `ptr` (/proc/self/numa_maps)."""
    start = None
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                lo, hi = (int(x, 16) for x in line.split()[0].split("-"))
                if lo <= ptr < hi:
                    start = lo
                    break
        if start is None:
            return {}
        with open("/proc/self/numa_maps") as f:
            for line in f:
                fields = line.split()
                if int(fields[0], 16) == start:
                    return {int(k[1:]): int(v) for k, v in (x.split("=") for x in fields[2:] if x[:1] == "N" and "=" in x)}
    except (OSError, ValueError):
        pass
    return {}


def thread_cpus(comm):
    """Last CPU of each thread of this process named `comm`."""
    cpus = []
    try:
        for tid in os.listdir("/proc/self/task"):
            try:
                with open(f"/proc/self/task/{tid}/comm") as f:
                    if f.read().strip() != comm:
                        continue
                with open(f"/proc/self/task/{tid}/stat") as f:
                    stat = f.read()
                cpus.append(int(stat[stat.rindex(")") + 2:].split()[36]))
            except (OSError, ValueError, IndexError):
                continue
    except OSError:
        pass
    return sorted(cpus)


def gpu_numa_node(dev_index):
    import torch
    p = torch.cuda.get_device_properties(dev_index)
    bus = f"{p.pci_domain_id:04x}:{p.pci_bus_id:02x}:{p.pci_device_id:02x}.0"
    try:
        with open(f"/sys/bus/pci/devices/{bus}/numa_node") as f:
            return int(f.read().strip())
    except (OSError, ValueError):
        return None


def host_placement(ptr, dev_index):
    nodes = numa_nodes()
    node_of = {c: n for n, cs in nodes.items() for c in cs}
    fill = thread_cpus("tprf-host-fill")
    allowed = sorted(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else []
    return {"pinned_buffer_pages_by_node": buffer_numa_pages(ptr), "gpu_pci_numa_node": gpu_numa_node(dev_index),
            "cpus_allowed": len(allowed), "cpus_allowed_by_node": {n: sum(1 for c in allowed if node_of.get(c) == n)
                                                                   for n in nodes},
            "fill_thread_cpus": fill, "fill_thread_nodes": sorted({node_of.get(c) for c in fill} - {None})}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle on a bounded sample of the workload

def cpu_sample_seconds(cfg, frac_seed=0, scale=1.0):
    """Extrapolated seconds for one full step of the oracle, from timed slices.

    Each stage is timed on a slice (a few frequencies, r points, columns or
    (w, q) points) and scaled linearly by the slice fraction.
    """
    import numpy as np
    import oracle as O
    dims, beta, mu, n_max, nw = cfg["dims"], cfg["beta"], cfg["mu"], cfg["n_max"], cfg["nw"]
    ek = O.ek_from_hoppings(cfg["hoppings"], dims)
    nk, nb = ek.shape[0], ek.shape[-1]
    n_nu, n_tau = 2 * n_max, 6 * n_max + 1
    nwt = 2 * nw - 1
    rng = np.random.default_rng(frac_seed)
    t = {}
    # Dyson on a few frequencies
    s_nu = max(1, int(4 * scale))
    t0 = time.perf_counter()
    g_part = np.linalg.inv((O.fermionic_iw(beta, n_max)[:s_nu] + mu)[:, None, None, None] * np.eye(nb) - ek[None])
    t["dyson"] = (time.perf_counter() - t0) * n_nu / s_nu
    # k -> r on the same frequencies
    t0 = time.perf_counter()
    g_r = O.fourier_wk_to_wr(g_part, dims)
    t["fft_k_to_r"] = (time.perf_counter() - t0) * n_nu / s_nu
    # iv -> tau on a slice of columns (G(iv, r) for all frequencies of a few columns)
    s_col = max(16, int(256 * scale))
    g_cols = O.lattice_dyson_g0_wk(mu, ek[:s_col // (nb * nb) + 1], beta, n_max).reshape(n_nu, -1)[:, :s_col]
    t0 = time.perf_counter()
    g_t = O.fourier_wr_to_tr(g_cols[:, :, None], beta, n_tau)
    t["nu_to_tau"] = (time.perf_counter() - t0) * (nk * nb * nb) / s_col
    # bubble + tau -> w for a few r points
    s_r = max(1, int(2 * scale))
    gt = rng.standard_normal((n_tau, 2, nb, nb)) + 0j
    t0 = time.perf_counter()
    for _ in range(s_r):
        chi_t = np.einsum("tda,tbc->tabcd", gt[:, 0], gt[::-1, 1]).reshape(n_tau, -1)
        O.chi_wr_from_chi_tr(chi_t, beta, nw)
    t["bubble_tau_to_w"] = (time.perf_counter() - t0) * nk / s_r
    # r -> q for a few (w, element) slices
    s_w = max(1, int(8 * scale))
    x = rng.standard_normal((s_w, nk, 1)) + 0j
    t0 = time.perf_counter()
    O.fourier_wr_to_wk(x, dims)
    t["fft_r_to_q"] = (time.perf_counter() - t0) * nwt * nb ** 4 / s_w
    # RPA on a slice of points
    s_p = max(64, int(4096 * scale))
    c0 = 0.05 * (rng.standard_normal((s_p, nb, nb, nb, nb)) + 1j * rng.standard_normal((s_p, nb, nb, nb, nb)))
    t0 = time.perf_counter()
    O.solve_rpa_PH(c0, cfg["U"])
    t["rpa"] = (time.perf_counter() - t0) * nwt * nk / s_p
    del g_r, g_t
    return sum(t.values()), t


def _cpu_worker(args):
    key, seed, scale = args
    from tprf_gb300 import workloads
    return cpu_sample_seconds(workloads.config(key), seed, scale)[0]


def cpu_throughput(cfg_key, procs: int, scale=1.0, pool=None):
    """(points/s, cores, seconds of wall time) of the oracle on `procs` host processes.

    Every process times one slice-sampled full step (``cpu_sample_seconds``);
    with several processes they run concurrently on separate cores, as the
    reference's OpenMP loops over r and w do, and the throughput adds up.
    """
    from tprf_gb300 import workloads
    cfg = workloads.config(cfg_key)
    points = (2 * cfg["nw"] - 1) * int(math.prod(cfg["dims"]))
    t0 = time.perf_counter()
    if procs <= 1 or pool is None:
        sec, _ = cpu_sample_seconds(cfg, 0, scale)
        return points / sec, 1, time.perf_counter() - t0
    secs = pool.map(_cpu_worker, [(cfg_key, i, scale) for i in range(procs)])
    wall = time.perf_counter() - t0
    return procs * points / statistics.mean(secs), procs, wall


# ---------------------------------------------------------------------------
# GPU arm

def setup_autotune(lib, args):
    """Measure mode of the library's autotuner unless --no-autotune: the first
    (warm-up) call of each shape times the candidate launch shapes."""
    from tprf_gb300._native import check
    lib.tprf_set_autotune(0 if args.no_autotune else 1)
    if getattr(args, "load_wisdom", None):
        check(lib.tprf_autotune_load(args.load_wisdom.encode()), "autotune_load")


def save_wisdom(lib, args):
    from tprf_gb300._native import check
    if getattr(args, "save_wisdom", None):
        check(lib.tprf_autotune_save(args.save_wisdom.encode()), "autotune_save")


def autotune_info(lib, args):
    """The autotuner's mode and its choices ("wisdom": kernel/shape key -> value;
    the *_radix keys name the FFT radix order, see fft_variants)."""
    import tempfile
    save_wisdom(lib, args)
    wisdom = {}
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "wisdom.txt")
        if lib.tprf_autotune_save(path.encode()) == 0 and os.path.exists(path):
            for ln in open(path):
                parts = ln.split()
                if len(parts) == 2:
                    wisdom[parts[0].split("/", 1)[-1]] = int(parts[1])
    return {"mode": "fixed heuristics" if args.no_autotune else "measure (tuned during warm-up)",
            "wisdom_entries": int(lib.tprf_autotune_entries()), "wisdom": wisdom}


def lattice_passes(dims) -> int:
    """Kernel launches of one lattice FFT over `dims`: the two fastest non-trivial axes
    share one pass when both are powers of two (at most 256, plane at most 4096 points),
    every other non-trivial axis takes one."""
    nontriv = [d for d in dims if d > 1]
    if len(nontriv) >= 2:
        a, b = nontriv[-2], nontriv[-1]
        pow2 = lambda n: n & (n - 1) == 0  # noqa: E731
        if pow2(a) and pow2(b) and max(a, b) <= 256 and a * b <= 4096:
            return len(nontriv) - 1
    return len(nontriv)


def run_gpu(args):
    import numpy as np
    import torch

    import tprf_gb300 as T
    from tprf_gb300 import _native, workloads
    from tprf_gb300._native import check, dims3
    from tprf_gb300.tight_binding import ek_tensor

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    lib = _native.lib()
    setup_autotune(lib, args)
    cfg = workloads.config(args.config)
    dims, beta, mu, n_max, nw = cfg["dims"], cfg["beta"], cfg["mu"], cfg["n_max"], cfg["nw"]
    nk = int(math.prod(dims))
    e_k = ek_tensor(cfg["hoppings"], dims, device=dev)
    nb = e_k.shape[-1]
    nb2, nb4 = nb * nb, nb ** 4
    n_nu, n_tau, nwt = 2 * n_max, 6 * n_max + 1, 2 * nw - 1
    points = nwt * nk
    U = torch.as_tensor(cfg["U"], dtype=torch.complex128, device=dev).contiguous()
    g_wk = torch.empty(n_nu, nk, nb, nb, dtype=torch.complex128, device=dev)
    chi0 = torch.empty(nwt, nk, nb4, dtype=torch.complex128, device=dev)
    chi = torch.empty_like(chi0)
    d3 = dims3(dims)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    lib.tprf_set_sync_checks(0)
    # Dyson, k->r passes, Hermitian test, iv->tau, bubble + tau->iw, r->q passes (the
    # last one also stores the negative frequencies of a real bubble), RPA
    launches_per_step = 1 + lattice_passes(dims) + 1 + 1 + 1 + lattice_passes(dims) + 1

    ws_bytes = lib.tprf_imtime_bubble_workspace_bytes(n_max, n_tau, d3, nb)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    stages = ["dyson", "fft_k_to_r", "nu_to_tau", "bubble_tau_to_w", "fft_r_to_q", "rpa"]
    no_events = (ctypes.c_void_p * 5)()

    def step(ev=None, out=None):
        # Dyson, then the bubble chain through its own entry point (k->r, iv->tau,
        # bubble + tau->iw, r->q; stage events recorded by the library), then the RPA
        out = chi if out is None else out
        if ev is not None:
            ev[0][0].record(stream)
        check(lib.tprf_lattice_dyson_g_wk(beta, n_max, nk, nb, mu, e_k.data_ptr(), None, 0, g_wk.data_ptr(), sh))
        check(lib.tprf_imtime_bubble_chi0_wk_timed(beta, n_max, n_tau, nw, d3, nb, g_wk.data_ptr(), None,
                                                   chi0.data_ptr(), ws.data_ptr(), ws_bytes,
                                                   ev[1] if ev is not None else no_events, sh))
        check(lib.tprf_solve_rpa_PH_wk(nw, d3, nb, chi0.data_ptr(), U.data_ptr(), out.data_ptr(), sh))
        if ev is not None:
            ev[0][6].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    check(lib.tprf_check_device_status(sh), "warm-up")
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(7)] for _ in range(args.steps)]
    for row in evs:  # torch creates an event's handle at its first record
        for e in row:
            e.record(stream)
    torch.cuda.synchronize()
    handles = [(ctypes.c_void_p * 5)(*[row[i].cuda_event for i in range(1, 6)]) for row in evs]
    assert all(h for row in handles for h in row)
    clocks = ClockSampler(local)
    barrier(world, dev)
    torch.cuda.synchronize()
    with clocks:
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        l0 = lib.tprf_kernel_launches()
        t_start.record(stream)
        for k in range(args.steps):
            step((evs[k], handles[k]))
        t_end.record(stream)
        launches = lib.tprf_kernel_launches() - l0
        torch.cuda.synchronize()
    barrier(world, dev)
    check(lib.tprf_check_device_status(sh), "timed steps")
    elapsed_ms = t_start.elapsed_time(t_end)
    elapsed_ms = max_over_ranks(elapsed_ms, world, dev)
    ms_per_step = elapsed_ms / args.steps
    stage_ms = {s: statistics.mean(evs[k][i].elapsed_time(evs[k][i + 1]) for k in range(args.steps))
                for i, s in enumerate(stages)}
    value = world * points / (ms_per_step / 1e3)

    # ---- the metric's accuracy clause: one more step with every stage in native
    # FP64 (the plain GPU path: no double-float stage, every (w, q) point solved on
    # its own), compared with the benched step's chi over the whole tensor
    accuracy = None
    if not args.no_accuracy:
        # chi_ref beside chi and chi0 when the device has room; otherwise the FP64
        # chain's chi0 replaces the benched one and its RPA (the point form, which in
        # the FP64 mode equals the mesh form bit for bit) is solved and compared in
        # chunks of frequencies
        whole = torch.cuda.mem_get_info(dev)[0] > chi.numel() * C16 + (4 << 30)
        chi_ref = torch.empty_like(chi) if whole else None
        chunk = 32
        num = den = 0.0
        mode0, tune0 = lib.tprf_get_arithmetic(), lib.tprf_get_autotune()
        lib.tprf_set_autotune(0)
        check(lib.tprf_set_arithmetic(1))
        try:
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a0.record(stream)
            if whole:
                step(out=chi_ref)
            else:
                check(lib.tprf_lattice_dyson_g_wk(beta, n_max, nk, nb, mu, e_k.data_ptr(), None, 0, g_wk.data_ptr(),
                                                  sh))
                check(lib.tprf_imtime_bubble_chi0_wk(beta, n_max, n_tau, nw, d3, nb, g_wk.data_ptr(), None,
                                                     chi0.data_ptr(), ws.data_ptr(), ws_bytes, sh))
                part = torch.empty((chunk,) + tuple(chi.shape[1:]), dtype=chi.dtype, device=dev)
                for a in range(0, nwt, chunk):
                    b = min(nwt, a + chunk)
                    check(lib.tprf_solve_rpa_PH((b - a) * nk, nb, chi0[a:b].data_ptr(), U.data_ptr(),
                                                part.data_ptr(), sh))
                    num = max(num, float((chi[a:b] - part[: b - a]).abs().max()))
                    den = max(den, float(part[: b - a].abs().max()))
                del part
            a1.record(stream)
            torch.cuda.synchronize()
            check(lib.tprf_check_device_status(sh), "FP64 step")
        finally:
            lib.tprf_set_arithmetic(mode0)
            lib.tprf_set_autotune(tune0)
        fp64_ms = a0.elapsed_time(a1)
        if whole:
            for a in range(0, nwt, 32):  # chunks of frequencies bound the temporaries
                b = min(nwt, a + 32)
                num = max(num, float((chi[a:b] - chi_ref[a:b]).abs().max()))
                den = max(den, float(chi_ref[a:b].abs().max()))
        accuracy = {"max_rel_err_vs_fp64": num / den, "bar": 1e-10,
                    "definition": "max |chi - chi_fp64| / max |chi_fp64| over the whole (iw, q, orbital) tensor",
                    "arithmetic": {0: "df64", 1: "fp64", 2: "df64_all"}[mode0],
                    "arithmetic_detail": "double-float (FP32 pairs) in the lattice FFTs, iv->tau, bubble + tau->iw, "
                                         "the Dyson inversion and the nb >= 3 RPA (points with a conditioning "
                                         "estimate above 100 re-solved in FP64); tail fits and fit_derivatives "
                                         "samples in FP64" if mode0 == 0 else "see tprf_set_arithmetic",
                    "fp64_path": {"value": world * points / (fp64_ms / 1e3), "unit": UNIT, "ms_per_step": fp64_ms,
                                  "timing": "one step" if whole else "the step with the RPA and the comparison in "
                                                                    "chunks of 32 frequencies (chi_ref did not fit)"}}
        # how ill-conditioned the RPA is: chi = A^-1 chi0 with A = I - chi0 U amplifies a
        # relative change of chi0 by up to ~kappa(A), so two FP64 implementations of the
        # chain (chi0 ~1e-15 apart) agree on chi only to ~kappa x 1e-15. Measured on the
        # static slice w = 0, where the RPA is closest to an instability; chi0 holds the
        # FP64 step's chi0 here.
        grouped = torch.swapaxes(chi0[nw - 1].reshape((nk,) + (nb,) * 4), -1, -2).reshape(nk, nb2, nb2)
        A = torch.eye(nb2, dtype=chi0.dtype, device=dev) - grouped @ torch.swapaxes(U, -1, -2).reshape(nb2, nb2)
        kappa = torch.linalg.cond(A)
        accuracy["rpa_condition_w0"] = {
            "kappa_max": float(kappa.max()), "kappa_median": float(kappa.median()),
            "q_points_kappa_over_1e4": int((kappa > 1e4).sum()),
            "fp64_agreement_floor": float(kappa.max()) * 1e-15,
            "meaning": "2-norm condition number of I - chi0 U over q at w = 0; kappa x 1e-15 is the level at "
                       "which two FP64 implementations of the chain agree on chi"}
        del chi_ref, grouped, A, kappa
        torch.cuda.empty_cache()

    # ---- end to end through the public API, host buffers in and out
    e2e = None
    if not args.no_e2e:
        ek_host = e_k.cpu().pin_memory()
        # two pinned outputs used in turn where host memory allows: a pipelined call's chi
        # (its copies and host fill running behind the next call) must not be the next
        # call's output; with one (a chi too large to pin twice) the calls share it
        chi_bytes = nwt * nk * nb ** 4 * C16
        try:
            host_bytes = os.sysconf("SC_PHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
        except (ValueError, OSError):
            host_bytes = 0
        n_out = 2 if 2 * chi_bytes <= 0.3 * host_bytes else 1
        out_hosts = [torch.empty((nwt, nk) + (nb,) * 4, dtype=torch.complex128, pin_memory=True)
                     for _ in range(n_out)]
        out_host = out_hosts[0]
        turn = [0]
        wmesh = T.MeshImFreq(beta, "Fermion", n_max)
        kmesh = T.MeshBrZone(dims=dims)
        del g_wk, ws, chi0, chi
        torch.cuda.empty_cache()
        from tprf_gb300.lattice_utils import imtime_bubble_rpa_wk, join_host_copies
        block = max(1, -(-nw // 16))
        # a ring slot for every block of the frequencies w >= 0 (real bubble): the
        # solves never wait for the call's own copies, which drain behind the next
        # call's chain
        slots = min(32, -(-nw // block))
        fws = torch.empty(lib.tprf_imtime_bubble_rpa_to_host_workspace_bytes(n_max, n_tau, nw, d3, nb, block, slots),
                          dtype=torch.uint8, device=dev)
        chi0_buf = torch.empty((nwt, nk) + (nb,) * 4, dtype=torch.complex128, device=dev)

        def e2e_step(wait):
            # the public API: Dyson, then the bubble chain and the RPA in one call with chi
            # copied to the pinned host buffer in frequency blocks while later blocks solve
            ekd = ek_host.to(dev, non_blocking=True)
            g = T.lattice_dyson_g0_wk(mu, T.Gf(mesh=kmesh, data=ekd), wmesh)
            out = out_hosts[turn[0] % n_out]
            turn[0] += 1
            imtime_bubble_rpa_wk(g, cfg["U"], nw, out=out, block_freqs=block, slots=slots, chi0=chi0_buf,
                                 workspace=fws, wait=wait)
            del g

        def e2e_run(n, wait):
            # every step copies its e(k) in and its whole chi out; the run ends when the
            # last chi is on the host
            torch.cuda.synchronize()
            barrier(world, dev)
            t0 = time.perf_counter()
            for _ in range(n):
                e2e_step(wait)
            join_host_copies()
            torch.cuda.synchronize()
            return max_over_ranks((time.perf_counter() - t0) / n, world, dev)

        def host_record():
            # the library's record of the last call: its device-to-host copies and the
            # host threads' fill of the negative frequencies
            st = (ctypes.c_double * 10)()
            check(lib.tprf_imtime_bubble_rpa_to_host_last_stats(st, 10), "last_stats")
            return {"d2h_gb": round(st[0] / 1e9, 3), "d2h_copy_ms": round(st[1], 2),
                    "d2h_gbs": round(st[0] / (st[1] * 1e6), 1) if st[1] > 0 else None,
                    "copy_span_ms": round(st[2], 2), "fill_span_ms": round(st[3], 2),
                    "fill_job_ms": round(st[4], 1), "fill_cpus": int(st[5]), "copies": int(st[6]),
                    "fill_threads": int(st[7]), "real_path": bool(st[8]),
                    "blocks_with_negative_rows_over_link": round(st[9], 3)}

        # the run ends when the last step's chi is on the host: that drain (one call's
        # copies and fill behind its compute) is part of the time, spread over 10 steps
        e2e_steps = 10
        # pipelined: a step's chi copy (bound by the device-to-host link) runs behind the
        # next step's chain; device errors are read once, after the run
        lib.tprf_set_sync_checks(0)
        e2e_step(False)
        e2e_s = e2e_run(e2e_steps, False)
        check(lib.tprf_check_device_status(sh), "e2e steps")
        rec_pipelined = host_record()
        placement = host_placement(out_host.data_ptr(), local)
        # one call at a time: each returns when its chi is on the host
        lib.tprf_set_sync_checks(1)
        serial_s = e2e_run(max(1, min(args.steps, 2)), True)
        rec_serial = host_record()
        # the link alone: one 4 GiB device-to-host copy into the same pinned buffer
        probe = torch.empty(1 << 29, dtype=torch.float64, device=dev)
        dst = out_host.view(torch.float64).reshape(-1)[: probe.numel()]
        l0, l1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        dst.copy_(probe, non_blocking=True)
        l0.record(stream)
        dst.copy_(probe, non_blocking=True)
        l1.record(stream)
        torch.cuda.synchronize()
        link_gbs = probe.numel() * 8 / (l0.elapsed_time(l1) * 1e6)
        del probe, fws, chi0_buf
        torch.cuda.empty_cache()
        # the bytes that crossed to the host: the frequencies w >= 0 when the host fills
        # chi(-w, q) = conj(chi(w, -q)) (real bubble, real U), else all of chi
        d2h = int(lib.tprf_imtime_bubble_rpa_to_host_last_d2h_bytes())
        e2e = {"value": world * points / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(ek_host.numel() * C16),
               "d2h_bytes_per_step": d2h, "result_bytes_per_step": int(out_host.numel() * C16),
               "path": "lattice_dyson_g0_wk -> imtime_bubble_rpa_wk(wait=False) (chain + RPA, chi to pinned host "
                       "memory, the copies of a step overlapping the next step's chain; host threads fill "
                       "chi(-w, q) = conj(chi(w, -q)) when only w >= 0 crossed)",
               "steps": e2e_steps, "ms_per_step": e2e_s * 1e3, "block_freqs": block, "ring_slots": slots,
               "host_outputs": n_out,
               "serial": {"value": world * points / serial_s, "ms_per_step": serial_s * 1e3,
                          "path": "imtime_bubble_rpa_wk(wait=True): each call returns with chi on the host",
                          "host_side_last_step": rec_serial},
               "host_side_last_step": rec_pipelined, "d2h_link_gbs_4gib_copy": round(link_gbs, 1),
               "placement": placement}

    # ---- roofline of the dominant kernel
    real = all(not np.any(np.imag(np.asarray(h))) for h in cfg["hoppings"].values())
    model = stage_model(nb, nk, n_nu, n_tau, nw, real=real, nc=compact_columns(dims, nb, n_tau, nw, real=real))
    top = max(stage_ms, key=stage_ms.get)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    achieved = model[top]["bytes"] / (stage_ms[top] * 1e-3) / 1e9
    fp64_peak_tflops = measure_fp64_peak(lib, dev)
    per_stage = {s: {"ms": round(stage_ms[s], 3), "share": round(stage_ms[s] / sum(stage_ms.values()), 4),
                     "hbm_gbs": round(model[s]["bytes"] / (stage_ms[s] * 1e-3) / 1e9, 1),
                     "hbm_frac": round(model[s]["bytes"] / (stage_ms[s] * 1e-3) / 1e9 / hbm_peak, 4),
                     "fp64_tflops": round(model[s]["flops"] / (stage_ms[s] * 1e-3) / 1e12, 3)}
                 for s in stages}
    traffic, traffic_src = stage_traffic(dims, nb, n_max, nw)
    for s in stages:
        if s in traffic:
            per_stage[s]["traffic"] = round(traffic[s])
            per_stage[s]["traffic_over_algorithmic"] = round(traffic[s] / model[s]["bytes"], 3)
    roofline = {"bound": "hbm", "kernel": top, "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                "frac": round(achieved / hbm_peak, 4), "peak_source": peak_src,
                "algorithmic_bytes": model[top]["bytes"],
                "traffic": round(traffic[top]) if top in traffic else None, "traffic_source": traffic_src,
                # algorithmic FP64 flops of the stage / time, against this GPU's native FP64 rate:
                # above 1 where the butterflies run in double-float on the FP32 pipe
                "fp64": {"achieved_tflops": per_stage[top]["fp64_tflops"], "peak_tflops": fp64_peak_tflops,
                         "frac": round(per_stage[top]["fp64_tflops"] / fp64_peak_tflops, 4),
                         "meaning": "algorithmic FP64-equivalent flops / time vs the native FP64 FMA rate"},
                "stages": per_stage}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128", "data": "synthetic (seeded tight-binding model)",
        "config": {"workload": cfg["name"], "dims": list(dims), "nb": nb, "beta": beta, "n_max": n_max, "nw": nw,
                   "n_tau": n_tau, "points_per_step": points, "vertex": cfg.get("vertex_label"),
                   "l2": f"inputs larger than L2 (G(tau,r) {n_tau * nk * nb2 * C16 / 1e9:.2f} GB, "
                         f"chi {points * nb4 * C16 / 1e9:.2f} GB per step)",
                   "parallelism": f"replicas x{world}"},
        "e2e": e2e,
        "accuracy": accuracy,
        # counted by the library (tprf_kernel_launches) over the timed steps; the
        # expected count is launches_per_step per step
        "gpu_launches": int(launches), "gpu_launches_expected": launches_per_step * args.steps,
        "roofline": roofline,
        "clocks": clocks.summary(),
        "autotune": autotune_info(lib, args),
    }
    if not args.no_batched:
        # the 512 uneven instances, forward and with gradients, after the buffers
        # above are released
        try:
            del chi0, chi, g_wk, ws  # still held when the e2e leg did not run
        except NameError:
            pass
        torch.cuda.empty_cache()
        line["batched"] = batched_leg(args, dev, lib, world)
    if rank == 0 and not args.no_cpu_baseline:
        v, cores, wall = cpu_throughput(args.config, 1, scale=40)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"FP64 oracle, every stage timed on a slice and scaled to one full step "
                                          f"({wall:.1f} s of CPU work)"}
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def batched_leg(args, dev, lib, world, steps=3):
    """The 512 uneven instances (the batched configuration) inside the default run:
    forward graph alone and forward + backward graphs per step (gradients of
    L = sum_i sum |chi_i|^2 with respect to every instance's U, e(k) and t(R)),
    and the plain single-instance paths over all 512 instances (public API per
    instance; tprf_gb300.autodiff forward + backward per instance) beside them."""
    import numpy as np
    import torch

    import tprf_gb300 as T
    from tprf_gb300 import workloads
    from tprf_gb300._native import check
    from tprf_gb300.autodiff import HoppingModel, chi_rpa
    from tprf_gb300.batch import BatchedRPAGrad, RPAInstance
    from tprf_gb300.tight_binding import ek_tensor

    specs = workloads.batched_instances(512, seed=0)
    insts = [RPAInstance(e_k=ek_tensor(d["hoppings"], d["dims"], device=dev), U=d["U"], dims=d["dims"],
                         beta=d["beta"], mu=d["mu"], n_max=d["n_max"], nw=d["nw"]) for d in specs]
    lib.tprf_set_sync_checks(0)
    t_setup = time.perf_counter()
    batch = BatchedRPAGrad(insts, n_streams=args.streams, device=dev)
    setup_s = time.perf_counter() - t_setup
    points = batch.points
    stream = torch.cuda.current_stream()

    def timed(fn, n):
        fn()
        torch.cuda.synchronize()
        barrier(world, dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = lib.tprf_kernel_launches()
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        launched[fn.__name__] = int(lib.tprf_kernel_launches() - l0)
        torch.cuda.synchronize()
        return max_over_ranks(e0.elapsed_time(e1) / n, world, dev)

    launched = {}

    def step():
        batch.forward()
        torch.mul(batch.chi_flat, 2.0, out=batch.chi_grad_flat)  # dL/d conj(chi) of sum |chi|^2
        batch.backward()

    fwd_ms = timed(batch.forward, steps)
    grad_ms = timed(step, steps)
    check(lib.tprf_check_device_status(stream.cuda_stream), "batched graphs")
    batch.close()
    del batch
    torch.cuda.empty_cache()
    # the plain single-instance paths, one instance after the other, every instance
    lib.tprf_set_sync_checks(1)

    def plain_forward():
        for a in insts:
            g0 = T.lattice_dyson_g0_wk(a.mu, T.Gf(mesh=T.MeshBrZone(dims=a.dims), data=a.e_k),
                                       T.MeshImFreq(a.beta, "Fermion", a.n_max))
            T.solve_rpa_PH(T.imtime_bubble_chi0_wk(g0, nw=a.nw, verbose=False), a.U)

    models = []
    for d in specs:
        nb = d["nb"]
        models.append(HoppingModel(base=d["hoppings"], patterns=[{(1, 0): np.eye(nb), (-1, 0): np.eye(nb)}],
                                   dims=d["dims"], beta=d["beta"], mu=d["mu"], n_max=d["n_max"], nw=d["nw"]))
    Us = [torch.as_tensor(d["U"], dtype=torch.complex128, device=dev) for d in specs]
    theta0 = torch.zeros(1, dtype=torch.float64, device=dev)

    def plain_grad():
        for m, U in zip(models, Us):
            th = theta0.clone().requires_grad_(True)
            u = U.clone().requires_grad_(True)
            (chi_rpa(th, u, m).abs() ** 2).sum().backward()

    def wall(fn):
        fn()  # plans
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return max_over_ranks(time.perf_counter() - t0, world, dev)

    plain_fwd_s = wall(plain_forward)
    plain_grad_s = wall(plain_grad)
    lib.tprf_set_sync_checks(0)
    nb_counts = {nb: sum(1 for a in insts if a.nb == nb) for nb in (1, 2)}
    fwd_v, grad_v = world * points / (fwd_ms / 1e3), world * points / (grad_ms / 1e3)
    pf_v, pg_v = world * points / plain_fwd_s, world * points / plain_grad_s
    return {
        "workload": "batched_512_square_lattice_instances", "instances": len(insts), "nb_counts": nb_counts,
        "k_meshes": "{8,16,24,32,48}^2", "beta": "U[5,40]", "n_max": "7-smooth nearest 12.8 beta in [32,512]",
        "points_per_step": points, "unit": UNIT, "steps": steps, "streams": args.streams,
        "launch": "forward graph (+ backward graph) per step", "graph_setup_s": round(setup_s, 2),
        "forward": {"value": fwd_v, "ms_per_step": fwd_ms, "gpu_launches": launched["forward"]},
        "forward_plus_gradient": {"value": grad_v, "ms_per_step": grad_ms, "loss": "sum_i sum |chi_i|^2",
                                  "gradients": "dL/dU, dL/de(k), dL/dt(R) of every instance",
                                  "gpu_launches": launched["step"]},
        "plain_single_instance": {
            "instances_timed": len(insts),
            "forward": {"value": pf_v, "s_per_pass": plain_fwd_s,
                        "path": "lattice_dyson_g0_wk -> imtime_bubble_chi0_wk -> solve_rpa_PH per instance"},
            "forward_plus_gradient": {"value": pg_v, "s_per_pass": plain_grad_s,
                                      "path": "tprf_gb300.autodiff.chi_rpa forward + backward per instance"}},
        "speedup_vs_plain_single_instance": {"forward": fwd_v / pf_v, "forward_plus_gradient": grad_v / pg_v},
    }


def run_gpu_batched(args):
    """cfg2: 512 uneven instances (1-band / 2-orbital square lattices, k in
    {8..48}^2, beta in [5, 40], n_max with beta) through tprf_batch_run, one
    graph launch per step; the plain single-instance API path on the same
    instances is timed beside it."""
    import numpy as np
    import torch

    import tprf_gb300 as T
    from tprf_gb300 import _native, workloads
    from tprf_gb300.batch import BatchedRPA, RPAInstance
    from tprf_gb300.tight_binding import ek_tensor

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    lib = _native.lib()
    setup_autotune(lib, args)
    specs = workloads.batched_instances(512, seed=0)
    insts = [RPAInstance(e_k=ek_tensor(d["hoppings"], d["dims"], device=dev), U=d["U"], dims=d["dims"],
                         beta=d["beta"], mu=d["mu"], n_max=d["n_max"], nw=d["nw"]) for d in specs]
    lib.tprf_set_sync_checks(0)
    batch = BatchedRPA(insts, n_streams=args.streams, device=dev)
    points = batch.points
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        batch.run()
    torch.cuda.synchronize()
    check = _native.check
    check(lib.tprf_check_device_status(stream.cuda_stream), "warm-up")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    barrier(world, dev)
    torch.cuda.synchronize()
    with clocks:
        l0 = lib.tprf_kernel_launches()
        e0.record(stream)
        for _ in range(args.steps):
            batch.run()
        e1.record(stream)
        launches = lib.tprf_kernel_launches() - l0
        torch.cuda.synchronize()
    barrier(world, dev)
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, dev)
    value = world * points / (ms / 1e3)
    # the plain single-instance path: the reference's loop, one instance after the other, public API
    lib.tprf_set_sync_checks(1)
    n_plain = min(len(insts), 128)
    plain_pts = sum(a.points for a in insts[:n_plain])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for a in insts[:n_plain]:
        g0 = T.lattice_dyson_g0_wk(a.mu, T.Gf(mesh=T.MeshBrZone(dims=a.dims), data=a.e_k),
                                   T.MeshImFreq(a.beta, "Fermion", a.n_max))
        T.solve_rpa_PH(T.imtime_bubble_chi0_wk(g0, nw=a.nw, verbose=False), a.U)
    torch.cuda.synchronize()
    plain = plain_pts / (time.perf_counter() - t0)
    nb_counts = {nb: sum(1 for a in insts if a.nb == nb) for nb in (1, 2)}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (seeded tight-binding models)",
        "config": {"workload": "batched_512_square_lattice_instances", "instances": len(insts),
                   "nb_counts": nb_counts, "k_meshes": "{8,16,24,32,48}^2", "beta": "U[5,40]",
                   "n_max": "7-smooth nearest 12.8 beta in [32,512]", "points_per_step": points,
                   "streams": args.streams, "launch": "one CUDA graph launch per step",
                   "parallelism": f"replicas x{world}"},
        "plain_single_instance": {"value": plain, "unit": UNIT, "instances_timed": n_plain,
                                  "path": "lattice_dyson_g0_wk -> imtime_bubble_chi0_wk -> solve_rpa_PH per instance"},
        "speedup_vs_plain_single_instance": value / plain,
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "autotune": autotune_info(lib, args),
    }
    batch.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_gpu_batched_grad(args):
    """cfg2 with gradients: the 512 uneven instances of cfg2, forward graph then
    backward graph (tprf_batch_grad_*) per step, giving chi of every instance and
    the gradient of L = sum_i sum |chi_i|^2 with respect to every instance's U,
    e(k) and hoppings t(R). The plain single-instance differentiable path
    (tprf_gb300.autodiff, one instance after the other) is timed beside it."""
    import numpy as np
    import torch

    from tprf_gb300 import _native, workloads
    from tprf_gb300.autodiff import HoppingModel, chi_rpa
    from tprf_gb300.batch import BatchedRPAGrad, RPAInstance
    from tprf_gb300.tight_binding import ek_tensor

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    lib = _native.lib()
    setup_autotune(lib, args)
    specs = workloads.batched_instances(512, seed=0)
    insts = [RPAInstance(e_k=ek_tensor(d["hoppings"], d["dims"], device=dev), U=d["U"], dims=d["dims"],
                         beta=d["beta"], mu=d["mu"], n_max=d["n_max"], nw=d["nw"]) for d in specs]
    lib.tprf_set_sync_checks(0)
    batch = BatchedRPAGrad(insts, n_streams=args.streams, device=dev)
    points = batch.points
    stream = torch.cuda.current_stream()

    def step():
        batch.forward()
        torch.mul(batch.chi_flat, 2.0, out=batch.chi_grad_flat)  # dL/d conj(chi) of sum |chi|^2
        batch.backward()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    _native.check(lib.tprf_check_device_status(stream.cuda_stream), "warm-up")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    barrier(world, dev)
    torch.cuda.synchronize()
    with clocks:
        l0 = lib.tprf_kernel_launches()
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        launches = lib.tprf_kernel_launches() - l0
        torch.cuda.synchronize()
    barrier(world, dev)
    _native.check(lib.tprf_check_device_status(stream.cuda_stream), "timed steps")
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, dev)
    value = world * points / (ms / 1e3)
    # forward graph alone
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        batch.forward()
    e1.record(stream)
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1) / args.steps
    # the plain single-instance differentiable path, one instance after the other
    lib.tprf_set_sync_checks(1)
    n_plain = min(len(insts), 64)
    plain_pts = sum(a.points for a in insts[:n_plain])
    models = []
    for d in specs[:n_plain]:
        nb = d["nb"]
        pat = {(1, 0): np.eye(nb), (-1, 0): np.eye(nb)}
        models.append(HoppingModel(base=d["hoppings"], patterns=[pat], dims=d["dims"], beta=d["beta"], mu=d["mu"],
                                   n_max=d["n_max"], nw=d["nw"]))
    Us = [torch.as_tensor(d["U"], dtype=torch.complex128, device=dev) for d in specs[:n_plain]]
    theta0 = torch.zeros(1, dtype=torch.float64, device=dev)

    def plain_pass():
        for m, U in zip(models, Us):
            th = theta0.clone().requires_grad_(True)
            u = U.clone().requires_grad_(True)
            (chi_rpa(th, u, m).abs() ** 2).sum().backward()

    plain_pass()  # plans
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain_pass()
    torch.cuda.synchronize()
    plain = plain_pts / (time.perf_counter() - t0)
    line = {
        "metric": "RPA chi(q,iw) + dL/dU, dL/de(k), dL/dt(R) points/s (complex128)", "value": value, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded tight-binding models)",
        "config": {"workload": "batched_512_square_lattice_instances_with_gradients", "instances": len(insts),
                   "points_per_step": points, "loss": "sum_i sum |chi_i|^2", "streams": args.streams,
                   "launch": "forward graph + backward graph per step", "parallelism": f"replicas x{world}"},
        "forward_only": {"value": world * points / (fwd_ms / 1e3), "unit": UNIT, "ms_per_step": fwd_ms},
        "plain_single_instance": {"value": plain, "unit": UNIT, "instances_timed": n_plain,
                                  "path": "tprf_gb300.autodiff.chi_rpa forward + backward per instance"},
        "speedup_vs_plain_single_instance": value / plain,
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "autotune": autotune_info(lib, args),
    }
    batch.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_gpu_grad(args):
    """cfg3: chi(q, iw) plus the gradient of Re Tr chi(q=(pi,pi), iw=0) + sum |chi|^2
    with respect to U and 8 hopping amplitudes, through tprf_gb300.autodiff (forward
    kernels, then the hand-written adjoint kernels). One step = forward + backward.
    The forward pass alone is timed beside it."""
    import torch

    from tprf_gb300 import _native
    from tprf_gb300.autodiff import chi_rpa
    from tprf_gb300.workloads import cfg3_loss, cfg3_model

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    lib = _native.lib()
    setup_autotune(lib, args)
    lib.tprf_set_sync_checks(0)
    model, theta0, U0 = cfg3_model()
    nk = int(math.prod(model.dims))
    points = (2 * model.nw - 1) * nk
    theta_h = torch.as_tensor(theta0, dtype=torch.float64).pin_memory()
    U_h = torch.as_tensor(U0, dtype=torch.complex128).pin_memory()
    grads_h = torch.empty(len(theta0) + 2 * U0.size, dtype=torch.float64, pin_memory=True)
    loss_h = torch.empty(1, dtype=torch.float64, pin_memory=True)
    stream = torch.cuda.current_stream()

    def step(backward=True):
        theta = theta_h.to(dev, non_blocking=True).requires_grad_(backward)
        U = U_h.to(dev, non_blocking=True).requires_grad_(backward)
        L = cfg3_loss(chi_rpa(theta, U, model))
        if backward:
            L.backward()
            g = torch.cat([theta.grad, torch.view_as_real(U.grad).reshape(-1)])
            grads_h.copy_(g, non_blocking=True)
        loss_h.copy_(L.detach().reshape(1), non_blocking=True)

    def timed(backward):
        for _ in range(args.warmup):
            step(backward)
        torch.cuda.synchronize()
        barrier(world, dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        l0 = lib.tprf_kernel_launches()
        e0.record(stream)
        for _ in range(args.steps):
            step(backward)
        e1.record(stream)
        n_launch = lib.tprf_kernel_launches() - l0
        torch.cuda.synchronize()
        wall = (time.perf_counter() - t0) / args.steps
        return (max_over_ranks(e0.elapsed_time(e1) / args.steps, world, dev), max_over_ranks(wall, world, dev),
                n_launch)

    fwd_ms, _, _ = timed(False)
    clocks = ClockSampler(local)
    with clocks:
        ms, wall_s, launches = timed(True)
    _native.check(lib.tprf_check_device_status(stream.cuda_stream), "timed steps")
    nb = model.patterns[0][(1, 0)].shape[0]
    line = {
        "metric": "RPA chi(q,iw) + dL/dU, dL/dt(R) points/s (complex128)", "value": world * points / (ms / 1e3),
        "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (seeded 2-orbital square lattice, 8 seeded hopping patterns)",
        "config": {"workload": "grad_2orb_square_32x32", "dims": list(model.dims), "nb": nb, "beta": model.beta,
                   "n_max": model.n_max, "nw": model.nw, "points_per_step": points,
                   "loss": "Re Tr chi(q=(pi,pi), iw=0) + sum |chi|^2", "parameters": "U [2,2,2,2] complex, 8 real t(R) amplitudes",
                   "parallelism": f"replicas x{world}"},
        "forward_only": {"value": world * points / (fwd_ms / 1e3), "unit": UNIT, "ms_per_step": fwd_ms},
        "e2e": {"value": world * points / wall_s, "unit": UNIT,
                "h2d_bytes_per_step": int(theta_h.numel() * 8 + U_h.numel() * 16),
                "d2h_bytes_per_step": int(grads_h.numel() * 8 + 8)},
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "autotune": autotune_info(lib, args),
    }
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure_fp64_peak(lib, dev) -> float:
    """Live FP64 FMA throughput of this GPU (TFLOP/s), the denominator of the FP64 fractions."""
    import ctypes

    import torch
    from tprf_gb300._native import check
    scratch = torch.empty(2048 * 256, dtype=torch.float64, device=dev)
    out = ctypes.c_double(0.0)
    check(lib.tprf_measure_fp64_tflops(ctypes.byref(out), scratch.data_ptr(), scratch.numel() * 8,
                                       torch.cuda.current_stream().cuda_stream), "measure_fp64_tflops")
    return round(out.value, 3)


# ---------------------------------------------------------------------------
# DRAM traffic per stage, from an ncu launch capture
#
# The table in profiles/ is written by
#   python bench.py --traffic-from-ncu <capture.csv> --config <the captured workload> --traffic-out <table>
# from a one-pass capture (dram__bytes_read.sum, dram__bytes_write.sum and
# gpu__time_duration.sum of every launch, --print-units base). It records a hash of
# the CUDA sources; the bench reports `traffic` only while the sources still hash
# the same, scaled from the captured mesh to the benched one by the number of k
# points (every stage streams its (frequency, r or k) columns, so its DRAM bytes
# grow in proportion at fixed frequencies and orbitals).

TRAFFIC_TABLE = os.path.join(ROOT, "profiles", "traffic_cubic3orb_32x32x32.txt")
STAGES = ("dyson", "fft_k_to_r", "nu_to_tau", "bubble_tau_to_w", "fft_r_to_q", "rpa")


# the translation units that define or launch the forward chain's kernels (the
# headers count too); the host-copy, batch, GW, Lindhard and nb <= 2 RPA units
# do not change those kernels' traffic
CHAIN_SOURCES = ("dyson.cu", "fft_lattice.cu", "matsubara.cu", "pipeline.cu", "plans.cu", "rpa_warp.cu", "tune.cu")


def kernel_sources_hash() -> str:
    """sha256 (first 16 hex digits) of the CUDA sources the chain's kernels are built from."""
    import hashlib
    h = hashlib.sha256()
    d = os.path.join(ROOT, "tprf_gb300", "csrc")
    for name in sorted(os.listdir(d)):
        if name in CHAIN_SOURCES or name.endswith((".cuh", ".hpp", ".h")):
            h.update(name.encode())
            with open(os.path.join(d, name), "rb") as f:
                h.update(f.read())
    return h.hexdigest()[:16]


def stage_of_kernel(name: str):
    """The path stage a kernel of the forward chain belongs to (None: not one)."""
    import re
    n = name.split("(")[0]
    if "dyson_kernel" in n and "adjoint" not in n:
        return "dyson"
    m = re.search(r"lattice_(?:axis|plane|plane_tma)_kernel<(\w+)", n)
    if m:  # first template argument FWD: the k -> r direction
        return "fft_k_to_r" if m.group(1) in ("1", "true") else "fft_r_to_q"
    if "hermitian_check_kernel" in n or re.search(r"nu_to_tau_kernel\b", n):
        return "nu_to_tau"
    if re.search(r"tau_to_w_kernel\b", n):
        return "bubble_tau_to_w"
    if re.search(r"rpa_(?:pair|warp|lu|lu_pair)_kernel\b", n):
        return "rpa"
    return None


def write_traffic_table(args):
    """Per-stage DRAM bytes of one launch (median over the capture's launches of each
    kernel, summed over the stage's kernels: each runs once per step) from
    `ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum
    --print-units base --csv`."""
    import csv
    import re
    from tprf_gb300 import workloads
    cfg = workloads.config(args.config)
    launches = {}
    with open(args.traffic_from_ncu, newline="") as f:
        rows = [r for r in csv.reader(f) if len(r) > 5]
    start = next(i for i, r in enumerate(rows) if "Kernel Name" in r and "Metric Value" in r)
    head, rows = rows[start], rows[start:]
    col = {k: head.index(k) for k in ("ID", "Kernel Name", "Metric Name", "Metric Unit", "Metric Value")}
    scale = {"byte": 1.0, "ns": 1e-6, "nsecond": 1e-6, "us": 1e-3, "usecond": 1e-3, "ms": 1.0, "msecond": 1.0}
    for r in rows[1:]:
        unit = r[col["Metric Unit"]]
        if unit not in scale:
            raise SystemExit(f"unexpected unit {unit!r}: capture with --print-units base")
        rec = launches.setdefault(r[col["ID"]], {"kernel": r[col["Kernel Name"]].split("(")[0]})
        rec[r[col["Metric Name"]]] = float(r[col["Metric Value"]].replace(",", "")) * scale[unit]
    per_kernel = {}
    for rec in launches.values():
        if stage_of_kernel(rec["kernel"]) and "dram__bytes_read.sum" in rec:
            per_kernel.setdefault(rec["kernel"], []).append(rec)
    nk = int(math.prod(cfg["dims"]))
    lines = ["# DRAM traffic per stage of one step (bytes per launch, median over the captured launches of each",
             "# kernel, summed over the stage's kernels), from one ncu launch capture.",
             f"workload {cfg['name']}", f"dims {' '.join(str(d) for d in cfg['dims'])}",
             f"nb {int(cfg['U'].shape[0])}", f"n_max {cfg['n_max']}", f"nw {cfg['nw']}", f"nk {nk}",
             f"sources {kernel_sources_hash()}", "# kernel launches read_bytes write_bytes ms stage"]
    stage_sum = {s: [0.0, 0.0, 0.0] for s in STAGES}
    for k in sorted(per_kernel, key=lambda k: STAGES.index(stage_of_kernel(k))):
        recs = per_kernel[k]
        rd = statistics.median(x["dram__bytes_read.sum"] for x in recs)
        wr = statistics.median(x["dram__bytes_write.sum"] for x in recs)
        ms = statistics.median(x.get("gpu__time_duration.sum", 0.0) for x in recs)
        s = stage_of_kernel(k)
        stage_sum[s][0] += rd
        stage_sum[s][1] += wr
        stage_sum[s][2] += ms
        short = re.search(r"\w+_kernel(?:<.*>)?", k).group(0).replace(" ", "")
        lines.append(f"kernel {short} {len(recs)} {rd:.0f} {wr:.0f} {ms:.4f} {s}")
    lines.append("# stage read_bytes write_bytes ms")
    for s in STAGES:
        lines.append(f"stage {s} {stage_sum[s][0]:.0f} {stage_sum[s][1]:.0f} {stage_sum[s][2]:.4f}")
    text = "\n".join(lines) + "\n"
    if args.traffic_out:
        with open(args.traffic_out, "w") as f:
            f.write(text)
    print(text, end="")


def stage_traffic(dims, nb, n_max, nw, path=TRAFFIC_TABLE):
    """({stage: DRAM bytes per launch at this mesh}, provenance) from the committed
    table, or ({}, reason) when it is absent, for other frequencies or orbitals, or
    captured from other kernel sources."""
    try:
        with open(path) as f:
            rows = [ln.split() for ln in f if ln.strip() and not ln.startswith("#")]
    except OSError:
        return {}, {"traffic": None, "reason": f"no table at {os.path.relpath(path, ROOT)}"}
    meta = {r[0]: r[1:] for r in rows if r[0] not in ("kernel", "stage")}
    src = {"table": os.path.relpath(path, ROOT), "captured_on": meta["workload"][0]}
    if meta["sources"][0] != kernel_sources_hash():
        return {}, dict(src, traffic=None, reason="stale: the CUDA sources changed since the capture")
    if (int(meta["nb"][0]), int(meta["n_max"][0]), int(meta["nw"][0])) != (nb, n_max, nw):
        return {}, dict(src, traffic=None, reason="captured at other frequencies or orbitals")
    ratio = int(math.prod(dims)) / int(meta["nk"][0])
    out = {r[1]: (float(r[2]) + float(r[3])) * ratio for r in rows if r[0] == "stage"}
    return out, dict(src, scale_by_k_points=ratio)


# ---------------------------------------------------------------------------
# reference arm: the CPU implementation on the host cores

def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    os.environ["OMP_NUM_THREADS"] = "1"
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    procs = max(1, os.cpu_count() or 1)
    vals, walls = [], []
    with mp.get_context("spawn").Pool(procs) as pool:
        for _ in range(args.warmup):
            cpu_throughput(args.config, procs, scale=10, pool=pool)
        for _ in range(args.steps):
            v, cores, wall = cpu_throughput(args.config, procs, scale=10, pool=pool)
            vals.append(v)
            walls.append(wall)
    from tprf_gb300 import workloads
    cfg = workloads.config(args.config)
    nb = int(cfg["U"].shape[0])
    value = statistics.mean(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(walls), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded tight-binding model)",
        "config": {"workload": cfg["name"], "dims": list(cfg["dims"]), "nb": nb, "beta": cfg["beta"],
                   "n_max": cfg["n_max"], "nw": cfg["nw"], "n_tau": 6 * cfg["n_max"] + 1,
                   "points_per_step": (2 * cfg["nw"] - 1) * int(math.prod(cfg["dims"])),
                   "vertex": cfg.get("vertex_label"), "parallelism": "host cores"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                         "sample": "FP64 restatement of the reference (numpy), one process per host core, each "
                                   "timing every stage on a slice (~2 s) and scaling it to one full step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="cfg1")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP64 comparison step (profiling runs)")
    ap.add_argument("--no-batched", action="store_true", help="skip the 512-instance batched leg of the default run")
    ap.add_argument("--streams", type=int, default=32, help="concurrent streams of the batched graph (cfg2)")
    ap.add_argument("--grad", action="store_true", help="cfg2: forward + gradient graphs per step")
    ap.add_argument("--no-autotune", action="store_true", help="fixed launch-shape heuristics instead of measure mode")
    ap.add_argument("--load-wisdom", metavar="PATH", help="autotuner choices to load before the run (profiling runs "
                                                          "with --no-autotune: the tuned shapes, no trial launches)")
    ap.add_argument("--save-wisdom", metavar="PATH", help="write the autotuner's choices after the run")
    ap.add_argument("--traffic-from-ncu", metavar="CSV", help="write the per-stage DRAM traffic table of an ncu "
                                                              "launch capture (see traffic_table) and exit")
    ap.add_argument("--traffic-out", metavar="PATH", help="with --traffic-from-ncu: the table's path")
    args = ap.parse_args()
    if args.traffic_from_ncu:
        write_traffic_table(args)
        return
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "cfg2" and args.grad:
        run_gpu_batched_grad(args)
    elif args.config == "cfg2":
        run_gpu_batched(args)
    elif args.config == "cfg3":
        run_gpu_grad(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
