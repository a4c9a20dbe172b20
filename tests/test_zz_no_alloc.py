"""The allocation-free entry point bhsp_spmv_f64_noalloc, called through the C ABI.

Some callers cannot allocate device memory: a host framework that owns every device byte through
its own caching allocator, a real-time loop that cannot block in cudaMalloc / cudaFree, a process
whose device footprint is fixed after start-up.  For them the library offers one FP64 entry point
whose scratch lives in a fixed 2 MiB device array.  These tests check that its y matches the
existing plan entry point (bhsp_plan_execute) within the FP64 tolerance used everywhere else
(componentwise 1e-12 relative to (|A|.|x|)_i), on two calls in a row, and that it rejects
matrices beyond its limit.  The file sorts last so that a failure here comes after every other
test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import oracle
from conftest import TOL_F64

import benchmark_spmv_using_csr_gb300 as sp
from benchmark_spmv_using_csr_gb300 import gen
from benchmark_spmv_using_csr_gb300._lib import lib

pytestmark = pytest.mark.gpu


def _noalloc(rp, ci, val, x, y, m, n, nnz, validate=0):
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    return lib().bhsp_spmv_f64_noalloc(
        ctypes.c_void_p(rp.data_ptr()), ctypes.c_void_p(ci.data_ptr()),
        ctypes.c_void_p(val.data_ptr()), ctypes.c_void_p(x.data_ptr()),
        ctypes.c_void_p(y.data_ptr()), m, n, nnz, validate, ctypes.c_void_p(stream))


@pytest.mark.parametrize("kind", ["powerlaw", "stencil27", "powerlaw_large"])
def test_noalloc_matches_plan_on_two_calls(cuda_ok, kind):
    """powerlaw_large (about 21 M non-zeros) has more workers than one wave, so its tile kernel
    is the persistent one, with the work queue in the fixed scratch."""
    import torch
    a = {"powerlaw": lambda: gen.powerlaw(300_000, seed=21),
         "stencil27": lambda: gen.stencil3d(40, 37, 33, seed=22),
         "powerlaw_large": lambda: gen.powerlaw(1_500_000, seed=24)}[kind]()
    rp, ci = torch.from_numpy(a.row_ptr).cuda(), torch.from_numpy(a.col).cuda()
    val = torch.from_numpy(a.val).cuda()
    plan = sp.Plan(sp.VALUE_F64, a.m, a.n, rp, ci)
    for call, seed in enumerate((31, 32)):  # two calls in a row, new x each time
        x_np = gen.uniform(a.n, seed)
        x = torch.from_numpy(x_np).cuda()
        y_ref = torch.full((a.m,), float("nan"), dtype=torch.float64, device="cuda")
        plan.execute(val, x, y_ref)
        plan.check()
        y = torch.full((a.m,), float("nan"), dtype=torch.float64, device="cuda")
        assert _noalloc(rp, ci, val, x, y, a.m, a.n, a.nnz) == sp.BHSPARSE_SUCCESS, call
        y_np, y_ref_np = y.cpu().numpy(), y_ref.cpu().numpy()
        scale = oracle.csr_absrow(a.row_ptr, a.col, a.val, x_np)
        assert oracle.componentwise_error(y_np, y_ref_np, scale) <= TOL_F64, call
        ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, x_np)
        assert oracle.componentwise_error(y_np, ystar, scale) <= TOL_F64, call
    plan.close()


def test_noalloc_rejects_too_large_and_invalid(cuda_ok):
    import torch
    a = gen.stencil2d(16, 16)
    rp, ci = torch.from_numpy(a.row_ptr).cuda(), torch.from_numpy(a.col).cuda()
    val = torch.from_numpy(a.val).cuda()
    x = torch.ones(a.n, dtype=torch.float64, device="cuda")
    y = torch.zeros(a.m, dtype=torch.float64, device="cuda")
    # beyond the fixed scratch: refused before any work touches the (small) buffers
    rc = _noalloc(rp, ci, val, x, y, a.m, a.n, 400_000_000)
    assert rc == sp.BHSPARSE_NOALLOC_TOO_LARGE
    # an out-of-range column index is caught when validation is asked for
    bad = ci.clone()
    bad[5] = a.n + 3
    assert _noalloc(rp, bad, val, x, y, a.m, a.n, a.nnz, validate=1) == sp.BHSPARSE_INVALID_CSR
    # and the valid matrix still runs, validated, right after
    assert _noalloc(rp, ci, val, x, y, a.m, a.n, a.nnz, validate=1) == sp.BHSPARSE_SUCCESS
    yr = oracle.csr_serial(a.row_ptr, a.col, a.val, np.ones(a.n))
    scale = oracle.csr_absrow(a.row_ptr, a.col, a.val, np.ones(a.n))
    assert oracle.componentwise_error(y.cpu().numpy(), yr, scale) <= TOL_F64


@pytest.mark.parametrize("validate", [0, 1])
def test_noalloc_allocates_no_device_memory(cuda_ok, validate):
    """After a warm-up call (which loads the kernels' module), further calls leave the driver's
    free device memory unchanged, with and without the CSR validation pass."""
    import torch
    a = gen.powerlaw(200_000, seed=23)
    rp, ci = torch.from_numpy(a.row_ptr).cuda(), torch.from_numpy(a.col).cuda()
    val = torch.from_numpy(a.val).cuda()
    x = torch.from_numpy(gen.uniform(a.n, 33)).cuda()
    y = torch.zeros(a.m, dtype=torch.float64, device="cuda")
    for _ in range(2):
        assert _noalloc(rp, ci, val, x, y, a.m, a.n, a.nnz, validate) == sp.BHSPARSE_SUCCESS
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        assert _noalloc(rp, ci, val, x, y, a.m, a.n, a.nnz, validate) == sp.BHSPARSE_SUCCESS
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
