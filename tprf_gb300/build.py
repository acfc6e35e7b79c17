"""Build the tprf_gb300 CUDA library in-tree (``tprf_gb300/_lib/libtprf_gb300.so``).

Each translation unit under ``csrc/`` is compiled by nvcc for sm_103a only, in
parallel, then linked into one shared library that exposes the C ABI declared
in ``include/tprf_gb300.h``. No torch headers are involved: the library is
plain CUDA + C++, loaded from Python with ctypes.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libtprf_gb300.so")
CXX_DIR = os.path.join(HERE, "cxx")
CXX_LIB_PATH = os.path.join(LIB_DIR, "libtprf_gb300_cxx.so")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH_FLAGS + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
    "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"),
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the tprf_gb300 CUDA library cannot be built")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def cuda_root() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _cxx() -> str:
    for cand in (os.environ.get("CXX"), shutil.which("g++"), shutil.which("c++")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("g++ not found: the C++ layer of tprf_gb300 cannot be built")


def cxx_flags():
    """Compile and link flags of a C++ program using the TPRF-signature layer."""
    root = cuda_root()
    return (["-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(root, "include")],
            ["-L", LIB_DIR, "-ltprf_gb300_cxx", "-ltprf_gb300", "-L", os.path.join(root, "lib64"), "-lcudart",
             "-Wl,-rpath," + LIB_DIR, "-Wl,-rpath," + os.path.join(root, "lib64")])


def build_cxx_layer(verbose: bool = False, force: bool = False) -> str:
    """The C++ host layer with TPRF's signatures (include/triqs_tprf_gb300/triqs_tprf.hpp)
    over the C ABI: one g++ translation unit, linked against libtprf_gb300.so."""
    srcs = sorted(os.path.join(CXX_DIR, f) for f in os.listdir(CXX_DIR) if f.endswith(".cpp"))
    hdrs = [os.path.join(ROOT, "include", "tprf_gb300.h"), os.path.join(ROOT, "include", "triqs_tprf_gb300",
                                                                          "triqs_tprf.hpp")]
    if not (force or _stale(CXX_LIB_PATH, srcs + hdrs + [LIB_PATH])):
        return CXX_LIB_PATH
    cflags, _ = cxx_flags()
    root = cuda_root()
    tmp = CXX_LIB_PATH + ".tmp"
    cmd = [_cxx(), *cflags, "-fPIC", "-shared", "-Wall", "-o", tmp, *srcs, "-L", LIB_DIR, "-ltprf_gb300",
           "-L", os.path.join(root, "lib64"), "-lcudart", "-Wl,-rpath," + LIB_DIR,
           "-Wl,-rpath," + os.path.join(root, "lib64")]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"g++ failed for the C++ layer:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, CXX_LIB_PATH)
    return CXX_LIB_PATH


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(verbose: bool = False, force: bool = False, jobs: int | None = None) -> str:
    """Compile (if needed) and return the path of libtprf_gb300.so."""
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp"))]
    headers.append(os.path.join(ROOT, "include", "tprf_gb300.h"))
    srcs = sources()
    objs = []
    cmds = []
    for src in srcs:
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmds.append([nvcc, *NVCC_FLAGS, "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}:\n{res.stdout}\n{res.stderr}")
        if verbose and res.stderr.strip():
            print(res.stderr, file=sys.stderr)

    if cmds:
        with ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
            list(ex.map(run, cmds))
    if force or cmds or _stale(LIB_PATH, objs):
        tmp = LIB_PATH + ".tmp"
        cuda_lib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "lib64")
        run([nvcc, *ARCH_FLAGS, "-shared", "-cudart", "shared", "-Xlinker", "-rpath", "-Xlinker", cuda_lib,
             "-o", tmp, *objs])
        os.replace(tmp, LIB_PATH)
    build_cxx_layer(verbose=verbose, force=force)
    return LIB_PATH


if __name__ == "__main__":
    print(build_library(verbose=True, force="--force" in sys.argv))
