"""Build the in-tree shared library ``libspmv_gb300.so`` for sm_103a.

Every translation unit under ``csrc/`` is compiled by ``nvcc`` in parallel (one
``-gencode``, ``-lineinfo``) into ``_build/``, then linked next to this file.
Rebuilds only what changed.  No cmake, no pip: ``python -m
benchmark_spmv_using_csr_gb300.build`` or ``build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB_NAME = "libspmv_gb300.so"
LIB_PATH = os.path.join(HERE, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp,-O3",
                     "--expt-relaxed-constexpr", "-I" + INCLUDE]
# extra -D flags for experiments (e.g. SPMV_NVCC_DEFINES="-DSPMV_CACHE_MODE=1")
NVCC_FLAGS += os.environ.get("SPMV_NVCC_DEFINES", "").split()
LINK_FLAGS = ["-shared", "-Xcompiler", "-fopenmp", "-lgomp", "-ldl"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the SpMV library")


def _sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(nvcc: str, src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if _stale(obj, [src] + _headers()):
        cmd = [nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj]
        if src.endswith(".cpp"):  # host-only code; no FMA contraction on any host CPU
            cmd = [nvcc, "-x", "c++"] + NVCC_FLAGS[len(ARCH):] + ["-Xcompiler", "-ffp-contract=off",
                                                                 "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return obj


DRIVER_SRC = os.path.join(HERE, "driver", "spmv_main.cpp")
# the reference-style benchmark driver, one executable per value type (USE_DOUBLE)
DRIVERS = {"spmv": 1, "spmv_f32": 0}


def _build_drivers(nvcc: str, verbose: bool) -> None:
    incs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    for name, use_double in DRIVERS.items():
        exe = os.path.join(HERE, name)
        if not _stale(exe, [DRIVER_SRC, LIB_PATH] + incs):
            continue
        cmd = [nvcc, "-x", "c++", "-O3", "-std=c++17", "-Xcompiler", "-fopenmp",
               f"-DUSE_DOUBLE={use_double}", "-I" + INCLUDE, DRIVER_SRC, "-o", exe + ".tmp",
               "-L" + HERE, "-lspmv_gb300", "-lgomp", "-Xlinker", "-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")
        os.replace(exe + ".tmp", exe)


def build(verbose: bool = False) -> str:
    """Compile and link the library and the benchmark driver; returns the library's path."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, verbose), srcs))
    if _stale(LIB_PATH, objs):
        cmd = [nvcc] + ARCH + LINK_FLAGS + objs + ["-o", LIB_PATH + ".tmp"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB_PATH + ".tmp", LIB_PATH)
    _build_drivers(nvcc, verbose)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
