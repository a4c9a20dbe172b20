"""The comparators of include/spmv_compare.h on the GPU: the CSR-vector kernel at every vector
width and cuSPARSE's generic SpMV, exact on integer-valued data against the serial loop and
within the FP64 / FP32 tolerances on real data."""
import numpy as np
import pytest
import torch

import oracle
from conftest import TOL_F32, TOL_F64

import benchmark_spmv_using_csr_gb300 as sp
from benchmark_spmv_using_csr_gb300 import compare, gen

pytestmark = pytest.mark.gpu


def _dev(a, x, dt):
    return (torch.from_numpy(a.row_ptr).cuda(), torch.from_numpy(a.col).cuda(),
            torch.from_numpy(a.val.astype(dt)).cuda(), torch.from_numpy(x.astype(dt)).cuda(),
            torch.zeros(max(a.m, 1), dtype=torch.float64 if dt == np.float64 else torch.float32,
                        device="cuda"))


def test_vector_width_rule():
    assert [compare.vector_width(100, k) for k in (0, 200, 300, 800, 1600, 1700)] == \
        [2, 2, 4, 8, 16, 32]


@pytest.mark.parametrize("vt,dt", [(sp.VALUE_F64, np.float64), (sp.VALUE_F32, np.float32)])
def test_integer_exact(cuda_ok, vt, dt):
    a = gen.mixed_rows(20000, 15000, dense_row=77, mean_len=9.0, empty_frac=0.05, seed=3)
    val = gen.uniform_int(a.nnz, 4, 10)
    x = gen.uniform_int(a.n, 5, 10)
    a.val = val
    yr = oracle.csr_serial(a.row_ptr, a.col, val, x)
    rp, col, v, xd, y = _dev(a, x, dt)
    for tpv in (0, 2, 4, 8, 16, 32):
        y.zero_()
        compare.csr_vector(vt, rp, col, v, xd, y, tpv)
        torch.cuda.synchronize()
        assert np.array_equal(y[:a.m].cpu().numpy().astype(np.float64), yr), tpv
    try:
        cs = compare.Cusparse(vt, rp, col, v, xd, y)
    except RuntimeError as e:
        pytest.skip(f"cuSPARSE unavailable: {e}")
    y.zero_()
    cs.run()
    torch.cuda.synchronize()
    cs.close()
    assert np.array_equal(y[:a.m].cpu().numpy().astype(np.float64), yr)


@pytest.mark.parametrize("vt,dt,tol", [(sp.VALUE_F64, np.float64, TOL_F64),
                                       (sp.VALUE_F32, np.float32, TOL_F32)])
def test_real_within_tolerance(cuda_ok, vt, dt, tol):
    a = gen.powerlaw(50000, seed=9)
    x = gen.uniform(a.n, 10)
    ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val.astype(dt).astype(np.float64),
                            x.astype(dt).astype(np.float64))
    scale = oracle.csr_absrow(a.row_ptr, a.col, a.val.astype(dt).astype(np.float64),
                              x.astype(dt).astype(np.float64))
    rp, col, v, xd, y = _dev(a, x, dt)
    compare.csr_vector(vt, rp, col, v, xd, y)
    torch.cuda.synchronize()
    assert oracle.componentwise_error(y.cpu().numpy().astype(np.float64), ystar, scale) <= tol
