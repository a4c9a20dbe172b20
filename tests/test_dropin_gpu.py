"""The reference-style C++ caller (tests/dropin/caller.cpp) compiled unchanged against
include/bhsparse_spmv_cuda.h, for FP64 (USE_DOUBLE=1) and FP32 (USE_DOUBLE=0), linked with
libspmv_gb300.so and run on the GPU: the 6x6 known answer and an integer-valued random
matrix checked by exact equality, as spmv_cuda/main.cu does."""
import os
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def binaries(tmp_path_factory, cuda_ok):
    from benchmark_spmv_using_csr_gb300.build import LIB_PATH, build
    build()
    out = tmp_path_factory.mktemp("dropin")
    libdir = os.path.dirname(LIB_PATH)
    bins = {}
    for use_double in (1, 0):
        exe = out / f"spmv_{use_double}"
        cmd = ["g++", "-O2", f"-DUSE_DOUBLE={use_double}", "-I", os.path.join(ROOT, "include"),
               os.path.join(ROOT, "tests", "dropin", "caller.cpp"), "-o", str(exe),
               "-L", libdir, "-lspmv_gb300", f"-Wl,-rpath,{libdir}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        bins[use_double] = str(exe)
    return bins


@pytest.mark.parametrize("use_double", [1, 0])
def test_known_answer_mode(binaries, use_double):
    r = subprocess.run([binaries[use_double], "0"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASS!" in r.stdout and "6, 39, 21, 0, 12, 42" in r.stdout


@pytest.mark.parametrize("use_double", [1, 0])
def test_benchmark_mode(binaries, use_double):
    r = subprocess.run([binaries[use_double], "rand", "300000", "7"], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASS!" in r.stdout and "Bandwidth" in r.stdout


def test_unchanged_caller_gets_a_tuned_schedule(binaries):
    """The reference-style caller never sets a schedule; prepare_mem chooses one with the
    library's learned network (or its sweep fallback) when a network file ships with the
    library, which BHSP_LOG_SCHEDULE makes visible without touching the caller."""
    from benchmark_spmv_using_csr_gb300.build import LIB_PATH
    have_net = os.path.exists(os.path.join(os.path.dirname(LIB_PATH), "tuner_data",
                                           "gb300_f64_tuner.bin"))
    env = dict(os.environ, BHSP_LOG_SCHEDULE="1")
    r = subprocess.run([binaries[1], "rand", "200000", "3"], capture_output=True, text=True,
                       timeout=300, env=env)
    assert r.returncode == 0 and "PASS!" in r.stdout, r.stdout + r.stderr
    lines = [ln for ln in r.stderr.splitlines() if ln.startswith("bhsp: m=200000")]
    assert lines, r.stderr
    if have_net:
        assert "the learned network" in lines[0] or "the autotune sweep" in lines[0], lines[0]
    else:
        assert "the fixed default" in lines[0], lines[0]
