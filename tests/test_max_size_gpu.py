"""The largest matrix the C ABI accepts: nnz = BHSP_MAX_NNZ (2^31 - 4097), built on the device,
through the plan API for FP64 and FP32 at three schedules (direct S = 8 and S = 32, TMA-staged).

Every index computation near 2^31 runs here (tile boundaries, grid-stride loops over nnz,
tensor-map rows).  The check is size-independent and exact: integer values small enough that
every y_i is exact in FP32, compared with an int64 prefix-sum reference computed by torch.
About 45 GB of device memory."""
import numpy as np
import pytest
import torch

import benchmark_spmv_using_csr_gb300 as sp

pytestmark = pytest.mark.gpu

MAX_NNZ = 2147479551  # BHSP_MAX_NNZ of include/spmv_gb300.h
N = 1_000_003


@pytest.fixture(scope="module")
def big(cuda_ok):
    dev = "cuda"
    # ragged rows: lengths 1000..2200, every seventh row empty
    guess = MAX_NNZ // 1000 + 16
    i = torch.arange(guess, device=dev, dtype=torch.int64)
    lens = torch.where(i % 7 == 3, torch.zeros_like(i), 1000 + (i % 5) * 300)
    ends = torch.cumsum(lens, 0)
    m = int(torch.searchsorted(ends, torch.tensor([MAX_NNZ], device=dev)).item()) + 1
    rp = torch.zeros(m + 1, device=dev, dtype=torch.int64)
    rp[1:] = torch.clamp(ends[:m], max=MAX_NNZ)
    assert int(rp[-1]) == MAX_NNZ
    rp32 = rp.to(torch.int32)
    del i, lens, ends
    j = torch.arange(MAX_NNZ, device=dev, dtype=torch.int64)
    col = ((j * 7919) % N).to(torch.int32)
    vsmall = (j % 5).to(torch.uint8)  # values 0..4
    del j
    x_small = (torch.arange(N, device=dev, dtype=torch.int64) % 3).to(torch.uint8)  # 0..2
    # reference: y_i = sum over the row of val * x[col], exactly in int64
    prod = vsmall * x_small[col.long()]  # 0..8 as uint8
    cs = torch.zeros(MAX_NNZ + 1, device=dev, dtype=torch.int64)
    torch.cumsum(prod, 0, dtype=torch.int64, out=cs[1:])
    del prod
    y_ref = (cs[rp[1:]] - cs[rp[:-1]]).to(torch.float64)
    del cs, rp
    torch.cuda.empty_cache()
    yield {"m": m, "rp": rp32, "col": col, "vsmall": vsmall, "x_small": x_small, "y_ref": y_ref}
    torch.cuda.empty_cache()


@pytest.mark.parametrize("cfg", [(8, 16, 4, 0), (32, 4, 4, 0), (16, 4, 4, 2)])
def test_max_nnz_f64(big, cfg):
    val = big["vsmall"].to(torch.float64)
    x = big["x_small"].to(torch.float64)
    y = torch.full((big["m"],), -1.0, dtype=torch.float64, device="cuda")
    p = sp.Plan(sp.VALUE_F64, big["m"], N, big["rp"], big["col"], seg=cfg[0],
                tiles_per_worker=cfg[1], warps_per_cta=cfg[2], stages=cfg[3])
    p.execute(val, x, y)
    torch.cuda.synchronize()
    p.check()
    p.close()
    bad = int((y != big["y_ref"]).sum().item())
    del val
    torch.cuda.empty_cache()
    assert bad == 0


def test_max_nnz_f32(big):
    val = big["vsmall"].to(torch.float32)
    x = big["x_small"].to(torch.float32)
    y = torch.full((big["m"],), -1.0, dtype=torch.float32, device="cuda")
    p = sp.Plan(sp.VALUE_F32, big["m"], N, big["rp"], big["col"], seg=16, tiles_per_worker=8,
                warps_per_cta=4, stages=0)
    p.execute(val, x, y)
    torch.cuda.synchronize()
    p.check()
    p.close()
    assert int((y.double() != big["y_ref"]).sum().item()) == 0
    del val
    torch.cuda.empty_cache()


def test_above_max_rejected(cuda_ok):
    rp = torch.zeros(2, dtype=torch.int32, device="cuda")
    col = torch.zeros(32, dtype=torch.int32, device="cuda")
    with pytest.raises(sp.SpmvError):
        sp.Plan(sp.VALUE_F64, 1, 1, rp, col, nnz=MAX_NNZ + 1)
