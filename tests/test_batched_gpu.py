"""GPU parity of the batched multi-RHS form (FP32 storage, compensated FP32 accumulation, FP64
carry records) through the C ABI: integer-valued data bit-exact against the serial loop, real
data within 1e-6 normwise of the FP64 compensated oracle on every matrix and right-hand side,
graph replay identical to direct launches, repeated calls stable."""
import numpy as np
import pytest

import oracle
from conftest import TOL_MIXED_NORMWISE

from benchmark_spmv_using_csr_gb300 import batch, gen

pytestmark = pytest.mark.gpu


def _mats(seed, count=24, integer=False):
    mats = gen.batch_workload(count=count, m_lo=100, m_hi=20_000, seed=seed)
    mats.append(gen.mixed_rows(3000, 3000, dense_row=17, mean_len=4, empty_frac=0.9, seed=seed))
    mats.append(gen.powerlaw(1, seed=1))  # a one-row matrix
    if integer:
        for i, a in enumerate(mats):
            a.val = gen.uniform_int(a.nnz, 100 + i, 10) - 4.0
    return mats


@pytest.mark.parametrize("k", [1, 2, 4, 8])
@pytest.mark.parametrize("cfg", [(16, 4, 4), (8, 1, 8), (32, 2, 4), (16, 2, 8), (8, 3, 4),
                                 (32, 1, 8)])
def test_batched_integer_bit_exact(cuda_ok, k, cfg):
    """Every persistent kernel: each non-zeros-per-lane and warps-per-CTA pair, and every kernel
    variant (the one-head form at k = 1; L2-only gathers on and off) forced with
    bhsp_batch_set_variant, through graph replay and direct launches."""
    import torch
    mats = _mats(7, integer=True)
    b = batch.Batch(mats, k=k, seg=cfg[0], tiles_per_worker=cfg[1], warps_per_cta=cfg[2])
    x_np = (gen.uniform_int(b.n * k, 5, 10) - 4.0).reshape(b.n, k)
    x = torch.from_numpy(x_np.astype(np.float32)).cuda()
    y = torch.full((b.m, k), float("nan"), dtype=torch.float32, device="cuda")
    cat = b.cat
    yr = [oracle.csr_serial(cat["row_ptr"], cat["col"], cat["val"], x_np[:, j].copy())
          for j in range(k)]
    variants = [(None, None)] + [(oh, l2) for oh in ((False, True) if k == 1 else (False,))
                                 for l2 in (False, True)]
    for oh, l2 in variants:
        b.set_variant(one_head=oh, l2_only=l2)
        info = b.info()
        if oh is not None:
            assert (info["one_head"], info["x_l2_only"]) == (oh, l2)
        for use_graph in (True, False):
            y.fill_(float("nan"))
            b.execute(x, y, use_graph=use_graph)
            b.check()
            yh = y.cpu().numpy().astype(np.float64)
            for j in range(k):
                np.testing.assert_array_equal(yh[:, j], yr[j], err_msg=str((oh, l2, use_graph, j)))
    if k > 1:
        with pytest.raises(RuntimeError):
            b.set_variant(one_head=True)
    b.close()


@pytest.mark.parametrize("k", [1, 8])
def test_batched_real_normwise_each_matrix(cuda_ok, k):
    import torch
    mats = _mats(11)
    b = batch.Batch(mats, k=k)
    x_np = gen.uniform(b.n * k, 3).reshape(b.n, k)
    x = torch.from_numpy(x_np.astype(np.float32)).cuda()
    y = torch.zeros((b.m, k), dtype=torch.float32, device="cuda")
    b.execute(x, y)
    b.check()
    ys = b.split(y.cpu().numpy())
    no = b.cat["n_off"]
    for i, a in enumerate(mats):
        for j in range(k):
            xs = x_np[no[i]:no[i + 1], j].copy()
            ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, xs)
            if np.linalg.norm(ystar) == 0:
                assert np.all(ys[i][:, j] == 0)
                continue
            assert oracle.normwise_error(ys[i][:, j], ystar) <= TOL_MIXED_NORMWISE, (a.name, j)
    b.close()


def test_graph_replay_equals_direct_and_is_stable(cuda_ok):
    import torch
    mats = _mats(13)
    b = batch.Batch(mats, k=4)
    x = torch.from_numpy(gen.uniform(b.n * 4, 8).reshape(b.n, 4).astype(np.float32)).cuda()
    y0 = torch.zeros((b.m, 4), dtype=torch.float32, device="cuda")
    b.execute(x, y0, use_graph=False)
    y1 = torch.full((b.m, 4), 3.0, dtype=torch.float32, device="cuda")
    for _ in range(3):
        b.execute(x, y1, use_graph=True)
    b.check()
    assert torch.equal(y0, y1)
    info = b.info()
    assert info["launches"] == 2 and info["grid"] >= 152
    b.close()


@pytest.mark.parametrize("k", [1, 8])
def test_batched_autotune_pick_is_correct_and_no_slower(cuda_ok, tmp_path, k):
    """The batched autotuner times every candidate schedule; its pick is the fastest of the
    table, so at least as fast as the default schedule (which is a candidate), gives y within
    the mixed form's tolerance, and a second call takes the cached table."""
    import torch
    from benchmark_spmv_using_csr_gb300 import tune
    mats = _mats(13, count=40)
    b0 = batch.Batch(mats, k=k)
    x_np = gen.uniform(b0.n * k, 4).reshape(b0.n, k)
    x = torch.from_numpy(x_np.astype(np.float32)).cuda()
    y = torch.zeros((b0.m, k), dtype=torch.float32, device="cuda")
    b0.close()
    cache = tune.TuneCache(str(tmp_path / "batch.json"))
    b, t = batch.tuned(mats, k, x, y, cache=cache, reps=3)
    cands = batch.tune_candidates()
    ms = np.array([t["table_ms"][",".join(map(str, c))] for c in cands])
    # the pick is a fastest entry (the table is rounded to 0.1 us, so ties can hide the order)
    assert np.all(ms > 0) and ms[cands.index(tuple(t["pick"]))] == ms.min()
    dflt = (32 if k == 4 else 16, 4, 4)
    assert dflt in cands and ms.min() <= ms[cands.index(dflt)]
    y.fill_(float("nan"))
    b.execute(x, y)
    b.check()
    ys = b.split(y.cpu().numpy())
    no = b.cat["n_off"]
    for i, a in enumerate(mats):
        for j in range(k):
            ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, x_np[no[i]:no[i + 1], j].copy())
            if np.linalg.norm(ystar) > 0:
                assert oracle.normwise_error(ys[i][:, j].astype(np.float64), ystar) <= TOL_MIXED_NORMWISE
    b.close()
    b2, t2 = batch.tuned(mats, k, x, y, cache=cache)
    assert t2["cached"] and t2["pick"] == t["pick"]
    b2.close()


def test_batched_variant_follows_the_columns(cuda_ok):
    """The batch's kernel variant comes from the same counts as a single matrix's plan: random
    columns gather from L2 only, stencils through L1; the one-head form only at k = 1."""
    dense_random = [gen.density(20_000, 20_000, 1e-3, seed=s) for s in range(4)]
    stencils = [gen.stencil3d(20, 20, 20, seed=s) for s in range(4)]
    b = batch.Batch(dense_random, k=1)
    assert b.info()["x_l2_only"]
    b.close()
    for k in (1, 2):
        b = batch.Batch(stencils, k=k)
        info = b.info()
        assert not info["x_l2_only"] and info["one_head"] == (k == 1)
        b.close()


@pytest.mark.parametrize("k", [2, 8])
def test_one_matrix_many_right_hand_sides(cuda_ok, k):
    """A batch of one matrix is the multi-RHS SpMV of that matrix: k right-hand sides in one
    persistent launch, exact on integer data."""
    import torch
    a = gen.stencil3d(30, 30, 30, seed=3)
    a.val = gen.uniform_int(a.nnz, 8, 10) - 4.0
    b = batch.Batch([a], k=k)
    x_np = (gen.uniform_int(a.n * k, 9, 10) - 4.0).reshape(a.n, k)
    x = torch.from_numpy(x_np.astype(np.float32)).cuda()
    y = torch.full((a.m, k), float("nan"), dtype=torch.float32, device="cuda")
    b.execute(x, y)
    b.check()
    yh = y.cpu().numpy().astype(np.float64)
    for j in range(k):
        np.testing.assert_array_equal(yh[:, j], oracle.csr_serial(a.row_ptr, a.col, a.val,
                                                                  x_np[:, j].copy()))
    b.close()
