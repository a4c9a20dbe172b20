"""Matrix Market matrices through the drop-in class: the reference driver's file mode
(spmv_cuda/main.cu:547-825) -- load, integer values 0..9 for val and x (main.cu:735-743),
y = A.x on the GPU, and the exact comparison with the serial CSR loop (main.cu:789-806)."""
import glob
import os

import numpy as np
import pytest

import oracle
import benchmark_spmv_using_csr_gb300 as sp
from benchmark_spmv_using_csr_gb300 import mtx

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
VALID = [f for f in sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "mtx", "*.mtx")))
         if not os.path.basename(f).startswith("err_")]


@pytest.mark.parametrize("vt", [sp.VALUE_F64, sp.VALUE_F32])
def test_mtx_files_exact(cuda_ok, vt):
    for i, path in enumerate(VALID):
        a = mtx.load(path)
        val, x = mtx.reference_values(a, seed=5 + i)
        yr = oracle.csr_serial(a.row_ptr, a.col, val, x)
        dt = sp.host_dtype(vt)
        h = sp.BhsparseSpmvCuda(vt)
        assert h.init_platform() == 0, h.last_error
        y = np.zeros(max(a.m, 1), dt)
        assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, val.astype(dt), x.astype(dt),
                             y) == 0, h.last_error
        assert h.run_benchmark() == 0, h.last_error
        assert h.get_y() == 0, h.last_error
        h.free_mem()
        h.close()
        assert np.array_equal(y[:a.m].astype(np.float64), yr), os.path.basename(path)


def test_mtx_file_real_values(cuda_ok, tmp_path):
    """A larger symmetric real file with its own values, FP64, against the compensated oracle."""
    rng = np.random.default_rng(3)
    m = 30000
    r = rng.integers(0, m, 200000)
    c = rng.integers(0, m, 200000)
    r, c = np.maximum(r, c), np.minimum(r, c)
    keep = np.unique(r * m + c, return_index=True)[1]
    r, c = r[keep], c[keep]
    v = rng.uniform(-1, 1, r.size)
    p = tmp_path / "sym.mtx"
    with open(p, "w") as fh:
        fh.write(f"%%MatrixMarket matrix coordinate real symmetric\n{m} {m} {r.size}\n")
        fh.writelines(f"{a + 1} {b + 1} {x:.17g}\n" for a, b, x in zip(r, c, v))
    a = mtx.load(str(p))
    x = rng.uniform(-1, 1, m)
    h = sp.BhsparseSpmvCuda(sp.VALUE_F64)
    assert h.init_platform() == 0
    y = np.zeros(m)
    assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val, x, y) == 0, h.last_error
    assert h.run_benchmark() == 0 and h.get_y() == 0
    h.free_mem()
    h.close()
    ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, x)
    scale = oracle.csr_absrow(a.row_ptr, a.col, a.val, x)
    assert oracle.componentwise_error(y, ystar, scale) <= 1e-12
