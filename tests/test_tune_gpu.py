"""GPU tests of the tuning path through the C ABI: device features equal the host counts, the
autotuner times every candidate and its pick computes the same y."""
import numpy as np
import pytest

import oracle
from conftest import TOL_F64

import benchmark_spmv_using_csr_gb300 as sp
from benchmark_spmv_using_csr_gb300 import gen, tune

pytestmark = pytest.mark.gpu


def test_device_features_match_host(cuda_ok):
    import torch
    for a in (gen.powerlaw(200_000, seed=9), gen.stencil3d(30, 30, 30),
              gen.mixed_rows(100_000, 50_000, dense_row=3, mean_len=6, empty_frac=0.9, seed=1)):
        rp = torch.from_numpy(a.row_ptr).cuda()
        f_dev = tune.row_features(rp, a.n)
        f_host = tune.features_from_counts(a.m, a.n, tune.feature_counts(a.row_ptr))
        np.testing.assert_allclose(f_dev, f_host, rtol=1e-6, atol=1e-7)


def test_autotune_picks_a_correct_schedule(cuda_ok, tmp_path):
    import torch
    a = gen.powerlaw(300_000, seed=13)
    x = gen.uniform(a.n, 14)
    rp, ci = torch.from_numpy(a.row_ptr).cuda(), torch.from_numpy(a.col).cuda()
    val, xd = torch.from_numpy(a.val).cuda(), torch.from_numpy(x).cuda()
    y = torch.zeros(a.m, dtype=torch.float64, device="cuda")
    cache = tune.TuneCache(str(tmp_path / "cache.json"))
    ms, best = cache.tune(sp.VALUE_F64, rp, ci, val, xd, y, warmup=1, reps=3)
    assert ms.shape == (len(tune.candidates()),) and np.all(ms > 0)
    assert best == int(np.argmin(ms))
    assert cache.get(sp.VALUE_F64, tune.row_features(rp, a.n))[1] == best  # cached
    seg, tpw, warps, stages = tune.candidates()[best]
    p = sp.Plan(sp.VALUE_F64, a.m, a.n, rp, ci, seg=seg, tiles_per_worker=tpw, warps_per_cta=warps,
                stages=stages)
    y.fill_(float("nan"))
    p.execute(val, xd, y)
    p.check()
    scale = oracle.csr_absrow(a.row_ptr, a.col, a.val, x)
    err = oracle.componentwise_error(y.cpu().numpy(), oracle.csr_dot2(a.row_ptr, a.col, a.val, x), scale)
    assert err <= TOL_F64


@pytest.mark.parametrize("vt", [sp.VALUE_F64, sp.VALUE_MIXED_BF16])
def test_choose_schedule_on_device_buffers(cuda_ok, vt):
    """bhsp_choose_schedule picks for caller-held device buffers what prepare_mem picks for the
    same matrix through the handle, and a plan built with the pick computes the oracle's y."""
    import torch
    a = gen.stencil3d(60, 50, 40, seed=8)
    x = gen.uniform(a.n, 9)
    rp, ci = torch.from_numpy(a.row_ptr).cuda(), torch.from_numpy(a.col).cuda()
    v64 = torch.from_numpy(a.val).cuda()
    if vt == sp.VALUE_F64:
        val, xd = v64, torch.from_numpy(x).cuda()
    else:
        val, xd = v64.to(torch.bfloat16), torch.from_numpy(x).float().cuda()
    y = torch.zeros(a.m, dtype=xd.dtype, device="cuda")
    got = tune.choose_schedule(vt, rp, ci, val, xd, y)
    assert got["config"] in tune.candidates() or got["source"] == sp.SCHEDULE_DEFAULT
    h = sp.BhsparseSpmvCuda(vt)
    yh = np.zeros(a.m)
    assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val, x, yh) == 0, h.last_error
    src, conf = h.schedule_source()
    assert src == got["source"] and abs(conf - got["confidence"]) <= 1e-6
    if src == sp.SCHEDULE_LEARNED:  # the sweep's timing may differ run to run; the network not
        assert tuple(h.get_config()) == got["config"]
    h.close()
    none = tune.choose_schedule(vt, rp, ci, val, xd, y, tuner="")
    assert none["source"] == sp.SCHEDULE_DEFAULT and none["confidence"] == 0.0
    seg, tpw, warps, stages = got["config"]
    p = sp.Plan(vt, a.m, a.n, rp, ci, seg=seg, tiles_per_worker=tpw, warps_per_cta=warps,
                stages=stages)
    y.fill_(float("nan"))
    p.execute(val, xd, y)
    p.check()
    yy = y.double().cpu().numpy()
    if vt == sp.VALUE_F64:
        scale = oracle.csr_absrow(a.row_ptr, a.col, a.val, x)
        assert oracle.componentwise_error(yy, oracle.csr_dot2(a.row_ptr, a.col, a.val, x),
                                          scale) <= TOL_F64
    else:
        assert np.all(np.isfinite(yy))
    p.close()
