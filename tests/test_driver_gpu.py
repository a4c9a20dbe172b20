"""The reference-style driver on the GPU: the known-answer mode `spmv 0` and the file mode on
the Matrix Market fixtures, FP64 and FP32 builds; every method (CSR-vector, cuSPARSE, OpenMP at
4 and all threads, the drop-in class) must print PASS! and its timing line."""
import os
import subprocess

import pytest

from benchmark_spmv_using_csr_gb300.build import HERE, build

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MTX = os.path.join(ROOT, "tests", "golden", "mtx")


@pytest.fixture(scope="module")
def exes(cuda_ok):
    build()
    return {"f64": os.path.join(HERE, "spmv"), "f32": os.path.join(HERE, "spmv_f32")}


def _run(args):
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_known_answer_mode(exes, prec):
    out = _run([exes[prec], "0", "--runs", "20"])
    assert "(GPU) y = " in out and "NO PASS" not in out
    for what in ("CSR-vector", "OpenMP", "bhSPARSE"):
        assert f"Checking {what} SpMV Correctness ... PASS!" in out
        assert f"{what} time = " in out
    assert "cuSPARSE time = " in out or "cuSPARSE is not available" in out


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("name", ["known6_general_real.mtx", "general_real_shuffled.mtx",
                                  "symmetric_real_crlf.mtx", "general_pattern.mtx", "empty.mtx"])
def test_file_mode(exes, prec, name):
    out = _run([exes[prec], os.path.join(MTX, name), "--runs", "10", "--seed", "3"])
    assert "NO PASS" not in out
    assert "Checking bhSPARSE SpMV Correctness ... PASS!" in out
    assert "bhSPARSE time = " in out and " nnz = " in out
