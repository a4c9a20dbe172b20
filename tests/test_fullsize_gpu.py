"""Parity of y at the benchmark's full sizes, through the C ABI, against the oracle.

The reference checks its GPU result against the serial loop over the whole matrix
(spmv_cuda/main.cu:789-806).  These tests do the same on each benchmark matrix:

* power-law m = n = 4,194,304 (59 M non-zeros), 27-point stencil 160^3 (109 M) and 5-point
  Laplacian 256^2, real-valued: FP64 <= 1e-12 and FP32 <= 1e-5 componentwise relative to
  (|A|.|x|)_i against the FP64 compensated (Dot2) oracle; the mixed forms <= 1e-6 normwise,
  BF16 storage against the oracle on the BF16-rounded values and FP32 x;
* integer-valued data on the power-law and 27-point structures: FP64 and FP32 y bit for bit
  equal to the serial loop (every partial sum is an exact integer below 2^24);
* the 512-matrix batched workload at 1 and 8 right-hand sides: every matrix and right-hand
  side within 1e-6 normwise of the FP64 oracle.
"""
import numpy as np
import pytest

import oracle
from conftest import TOL_F32, TOL_F64, TOL_MIXED_NORMWISE

import benchmark_spmv_using_csr_gb300 as sp
from benchmark_spmv_using_csr_gb300 import batch, gen

pytestmark = pytest.mark.gpu

WORKLOADS = ["powerlaw_4m", "stencil27_160", "stencil5_256"]
# FP64 schedules: the handle's own choice (None), the bench picks on the two large matrices,
# and a TMA-staged one
FP64_SCHEDULES = [None, (8, 8, 4, 0), (32, 4, 4, 0), (16, 4, 4, 2)]


@pytest.fixture(scope="module", params=WORKLOADS)
def workload(request):
    a = gen.WORKLOADS[request.param]()
    x = gen.uniform(a.n, 7)
    ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, x)
    scale = oracle.csr_absrow(a.row_ptr, a.col, a.val, x)
    return request.param, a, x, ystar, scale


def run_handle(vt, a, val, x, cfg=None):
    dt = sp.host_dtype(vt)
    s = sp.BhsparseSpmvCuda(vt)
    if cfg is not None:
        assert s.set_config(*cfg) == 0, s.last_error
    assert s.init_platform() == 0, s.last_error
    y = np.full(a.m, np.nan, dt)
    assert s.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, val.astype(dt), x.astype(dt), y) == 0, \
        s.last_error
    for _ in range(2):  # a repeated call must give the same y
        assert s.run_benchmark() == 0, s.last_error
    assert s.get_y() == 0, s.last_error
    s.free_mem()
    s.close()
    return y


def test_fullsize_fp64(cuda_ok, workload):
    name, a, x, ystar, scale = workload
    for cfg in FP64_SCHEDULES:
        y = run_handle(sp.VALUE_F64, a, a.val, x, cfg)
        err = oracle.componentwise_error(y, ystar, scale)
        assert err <= TOL_F64, (name, cfg, err)


def test_fullsize_fp32(cuda_ok, workload):
    name, a, x, _, _ = workload
    v32, x32 = a.val.astype(np.float32), x.astype(np.float32)
    v64, x64 = v32.astype(np.float64), x32.astype(np.float64)
    ystar = oracle.csr_dot2(a.row_ptr, a.col, v64, x64)
    scale = oracle.csr_absrow(a.row_ptr, a.col, v64, x64)
    for cfg in (None, (16, 8, 4, 0)):
        y = run_handle(sp.VALUE_F32, a, v32, x32, cfg)
        err = oracle.componentwise_error(y, ystar, scale)
        assert err <= TOL_F32, (name, cfg, err)


def bf16_round(v):
    m, e = np.frexp(np.asarray(v, np.float64))
    return np.ldexp(np.round(m * 256.0), e - 8)


def test_fullsize_mixed_f32(cuda_ok, workload):
    name, a, x, ystar, _ = workload
    for cfg in (None, (32, 4, 4, 0)):
        y = run_handle(sp.VALUE_MIXED_F32, a, a.val, x, cfg)
        err = oracle.normwise_error(y, ystar)
        assert err <= TOL_MIXED_NORMWISE, (name, cfg, err)


def test_fullsize_mixed_bf16(cuda_ok, workload):
    name, a, x, _, _ = workload
    ystar_b = oracle.csr_dot2(a.row_ptr, a.col, bf16_round(a.val),
                              x.astype(np.float32).astype(np.float64))
    for cfg in (None, (16, 8, 4, 2)):
        y = run_handle(sp.VALUE_MIXED_BF16, a, a.val, x, cfg)
        err = oracle.normwise_error(y, ystar_b)
        assert err <= TOL_MIXED_NORMWISE, (name, cfg, err)


@pytest.mark.parametrize("name", ["powerlaw_4m", "stencil27_160"])
def test_fullsize_integer_bit_exact(cuda_ok, name):
    a = gen.WORKLOADS[name]()
    val = gen.uniform_int(a.nnz, 41, 10) - 4.0
    x = gen.uniform_int(a.n, 42, 10) - 4.0
    yr = oracle.csr_serial(a.row_ptr, a.col, val, x)
    assert np.abs(yr).max() < 2 ** 24
    for vt in (sp.VALUE_F64, sp.VALUE_F32):
        y = run_handle(vt, a, val, x)
        bad = int(np.count_nonzero(y.astype(np.float64) != yr))
        assert bad == 0, (name, vt, bad)


@pytest.fixture(scope="module")
def batch512():
    return gen.batch_workload(512)


@pytest.mark.parametrize("k", [1, 8])
def test_fullsize_batched_each_matrix(cuda_ok, batch512, k):
    import torch
    mats = batch512
    b = batch.Batch(mats, k=k)
    x_np = gen.uniform(b.n * k, 3).reshape(b.n, k)
    x = torch.from_numpy(x_np.astype(np.float32)).cuda()
    y = torch.full((b.m, k), float("nan"), dtype=torch.float32, device="cuda")
    b.execute(x, y, use_graph=True)
    b.check()
    ys = b.split(y.cpu().numpy())
    no = b.cat["n_off"]
    worst = 0.0
    for i, a in enumerate(mats):
        for j in range(k):
            ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, x_np[no[i]:no[i + 1], j].copy())
            if np.linalg.norm(ystar) == 0:
                assert not np.any(ys[i][:, j]), (i, j)
                continue
            err = oracle.normwise_error(ys[i][:, j].astype(np.float64), ystar)
            worst = max(worst, err)
            assert err <= TOL_MIXED_NORMWISE, (i, a.name, j, err)
    b.close()
    assert worst > 0.0
