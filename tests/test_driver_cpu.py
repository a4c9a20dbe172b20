"""The reference-style driver (benchmark_spmv_using_csr_gb300/driver/spmv_main.cpp) on CPU: usage
and the file-mode failures the reference reports before touching a GPU (spmv_cuda/main.cu:582-604)."""
import os
import subprocess

import pytest

from benchmark_spmv_using_csr_gb300.build import HERE, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MTX = os.path.join(ROOT, "tests", "golden", "mtx")


@pytest.fixture(scope="module")
def spmv():
    build()
    exe = os.path.join(HERE, "spmv")
    assert os.access(exe, os.X_OK)
    return exe


def test_usage(spmv):
    r = subprocess.run([spmv], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stdout


@pytest.mark.parametrize("name,status,message", [
    ("err_complex.mtx", -3, "Sorry, data type 'COMPLEX' is not supported."),
    ("err_banner_prefix.mtx", -2, "Could not process Matrix Market banner."),
    ("err_index.mtx", -6, "status -6"),
])
def test_file_failures(spmv, name, status, message):
    r = subprocess.run([spmv, os.path.join(MTX, name)], capture_output=True, text=True, timeout=60)
    assert r.returncode == status & 0xFF
    assert message in r.stdout
    assert "PRECISION = 64-bit Double Precision" in r.stdout and "RUN SpMV 200 times" in r.stdout
