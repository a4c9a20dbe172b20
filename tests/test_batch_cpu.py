"""CPU tests of the batched form's host logic: block-diagonal concatenation."""
import numpy as np

import oracle
from benchmark_spmv_using_csr_gb300 import batch, gen


def test_concatenation_is_block_diagonal():
    mats = [gen.stencil2d(5, 7), gen.powerlaw(300, seed=3), gen.blockdiag(70, 70, 32),
            gen.density(50, 50, 0.05, seed=2)]
    cat = batch.concatenate(mats)
    assert cat["m"] == sum(a.m for a in mats) and cat["nnz"] == sum(a.nnz for a in mats)
    rp, col, val = cat["row_ptr"], cat["col"], cat["val"]
    assert rp[0] == 0 and rp[-1] == cat["nnz"] and np.all(np.diff(rp) >= 0)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(cat["n"])
    y = oracle.csr_serial(rp, col, val, x)
    for i, a in enumerate(mats):
        xs = x[cat["n_off"][i]:cat["n_off"][i + 1]]
        yi = oracle.csr_serial(a.row_ptr, a.col, a.val, xs)
        np.testing.assert_array_equal(y[cat["m_off"][i]:cat["m_off"][i + 1]], yi)


def test_batch_workload_sizes():
    mats = gen.batch_workload(count=40, seed=9)
    assert len(mats) == 40
    assert all(800 <= a.m <= 210_000 for a in mats)
    kinds = {a.name.split("_")[0] for a in mats}
    assert len(kinds) >= 4
