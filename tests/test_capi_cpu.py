"""CPU tests of the C ABI boundary: the library loads, exports every symbol that
include/*.h declares, and rejects bad arguments without touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT

import benchmark_spmv_using_csr_gb300 as sp
from benchmark_spmv_using_csr_gb300._lib import SIGNATURES, lib


def _declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(inc, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for mt in re.finditer(r"\b(bhsp_[a-z0-9_]+)\s*\(", src):
            names.add(mt.group(1))
    return names


def test_library_exports_every_declared_symbol():
    L = lib()
    declared = _declared_symbols()
    assert len(declared) >= 30
    missing = [n for n in sorted(declared) if not hasattr(L, n)]
    assert not missing, missing
    # the Python binding covers the whole declared surface
    assert declared <= set(SIGNATURES), sorted(declared - set(SIGNATURES))


def test_version_string():
    assert "sm_103a" in sp.version()


def test_create_rejects_unknown_value_type():
    h = ctypes.c_void_p()
    assert lib().bhsp_create(ctypes.byref(h), 9) == sp.BHSPARSE_UNSUPPORTED_VALUE_TYPE
    assert lib().bhsp_create(None, 0) == sp.BHSPARSE_INVALID_ARGUMENT


def test_config_validation_without_gpu():
    s = sp.BhsparseSpmvCuda(sp.VALUE_F64)
    assert s.get_config() == sp.DEFAULT_CONFIG
    assert s.set_config(12, 1, 4) == sp.BHSPARSE_INVALID_ARGUMENT
    assert s.set_config(16, 2, 4, 0) == sp.BHSPARSE_SUCCESS
    assert s.get_config() == (16, 2, 4, 0)
    assert s.set_config(8, 0, 0, -1) == sp.BHSPARSE_SUCCESS
    assert s.get_config() == (8,) + sp.DEFAULT_CONFIG[1:]
    assert s.set_config(8, 1, 6) == sp.BHSPARSE_INVALID_ARGUMENT
    assert s.set_config(8, 1, 4, 1) == sp.BHSPARSE_INVALID_ARGUMENT
    assert s.set_config(16, 4, 8, 3) == sp.BHSPARSE_SUCCESS  # 8 warps x 3 FP64 slots fit
    b = sp.BhsparseSpmvCuda(sp.VALUE_MIXED_BF16)  # BF16 storage defaults to the staged ring
    assert b.get_config() == sp.DEFAULT_CONFIG[:3] + (2,)
    assert b.set_config(8, 0, 0, -1) == sp.BHSPARSE_SUCCESS and b.get_config() == (8, 8, 4, 2)
    assert b.set_config(16, 8, 4, 0) == sp.BHSPARSE_SUCCESS and b.get_config() == (16, 8, 4, 0)
    # 8 warps x 3 slots of 32 x 32 FP64 runs exceed 227 KB of shared memory
    assert s.set_config(32, 4, 8, 3) == sp.BHSPARSE_INVALID_ARGUMENT
    s.close()


def test_plan_queries_reject_a_null_plan():
    L = lib()
    n = ctypes.c_int()
    assert L.bhsp_plan_chunk_form(None, ctypes.byref(n), ctypes.byref(n)) == sp.BHSPARSE_INVALID_ARGUMENT
    assert L.bhsp_plan_gather_path(None, ctypes.byref(n), ctypes.byref(n),
                                   ctypes.byref(n)) == sp.BHSPARSE_INVALID_ARGUMENT
    assert L.bhsp_plan_tiles(None, None, None, None) == sp.BHSPARSE_INVALID_ARGUMENT
    assert L.bhsp_plan_set_variant(None, 1, 0) == sp.BHSPARSE_INVALID_ARGUMENT
    assert L.bhsp_batch_set_variant(None, 0, 1) == sp.BHSPARSE_INVALID_ARGUMENT
    assert L.bhsp_plan_set_grid(None, 1) == sp.BHSPARSE_INVALID_ARGUMENT


def test_run_before_prepare_is_an_error():
    s = sp.BhsparseSpmvCuda(sp.VALUE_F32)
    assert s.run_benchmark() == sp.BHSPARSE_NOT_PREPARED
    assert s.get_y() == sp.BHSPARSE_NOT_PREPARED
    assert "prepare_mem" in s.last_error
    s.close()


def test_prepare_rejects_bad_sizes_before_any_cuda_call():
    s = sp.BhsparseSpmvCuda(sp.VALUE_F64)
    y = np.zeros(4)
    rp = np.array([0, 1, 2, 3, 4], np.int32)
    assert s.prepare_mem(-1, 4, 4, rp, rp[:4], np.ones(4), np.ones(4), y) == sp.BHSPARSE_INVALID_ARGUMENT
    assert s.prepare_mem(4, 0, 4, rp, rp[:4], np.ones(4), np.ones(0), y) == sp.BHSPARSE_INVALID_ARGUMENT
    with pytest.raises(TypeError):
        s.prepare_mem(4, 4, 4, rp, rp[:4], np.ones(4), np.ones(4), np.zeros(4, np.float32))
    s.close()


def test_host_dtype_mapping():
    assert sp.host_dtype(sp.VALUE_F64) == np.float64
    assert sp.host_dtype(sp.VALUE_F32) == np.float32
    assert sp.host_dtype(sp.VALUE_MIXED_F32) == np.float64
    assert sp.host_dtype(sp.VALUE_MIXED_BF16) == np.float64


def test_dropin_header_compiles_as_plain_cxx(tmp_path):
    """A reference-style caller compiles against include/bhsparse_spmv_cuda.h with g++."""
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    src = tmp_path / "caller.cpp"
    src.write_text(
        '#include "bhsparse_spmv_cuda.h"\n'
        "int main() {\n"
        "  bhsparse_spmv_cuda *b = new bhsparse_spmv_cuda();\n"
        "  int rp[2] = {0, 1}, ci[1] = {0}; value_type v[1] = {2}, x[1] = {3}, y[1] = {0};\n"
        "  (void)rp; (void)ci; (void)v; (void)x; (void)y;\n"
        "  bhsparse_timer t; t.start(); double ms = t.stop(); (void)ms;\n"
        "  delete b; return NUM_RUN == 200 ? 0 : 1;\n"
        "}\n")
    cuda_inc = "/usr/local/cuda/include"
    r = subprocess.run(["g++", "-std=c++11", "-I", os.path.join(ROOT, "include"), "-I", cuda_inc,
                        "-c", str(src), "-o", str(tmp_path / "caller.o")], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
