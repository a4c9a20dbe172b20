"""Every tile kernel a plan can run, bit for bit against the serial loop.

A plan picks its tile kernel by value type, schedule (non-zeros per lane, tiles per worker, warps
per CTA, TMA stages) and variant (the one-head chunk form; x gathered from L2 only).  Its rules
choose the variant from the matrix, so a given matrix reaches only some kernels.  These tests
force every variant (bhsp_plan_set_variant) and both grids of the direct kernel (persistent and
static, bhsp_plan_set_grid) at every candidate schedule of the autotuner, in every value type, on
integer-valued matrices whose partial sums are exact in FP32: every form must then
equal the reference's serial CSR loop (spmv_cuda/main.cu:755-761) bit for bit.  The matrices mix
empty rows (dirty tiles), short rows (two row heads in one lane's chunk, which sends the one-head
form to its per-slot path), rows of 27 non-zeros, and a row longer than a worker (carry records
and their calibration); a second one is smaller than one tile.
"""
import numpy as np
import pytest

import oracle

import benchmark_spmv_using_csr_gb300 as sp
from benchmark_spmv_using_csr_gb300 import tune

pytestmark = pytest.mark.gpu

VARIANTS = [(False, False), (False, True), (True, False), (True, True)]


def mixed_rows(rng, m=4000, n=6000):
    lens = np.full(m, 27)
    lens[::50] = rng.integers(1, 4, lens[::50].size)
    lens[3::97] = 0
    lens[m // 3] = min(5000, n)
    rp = np.zeros(m + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    col = np.concatenate([np.sort(rng.choice(n, int(l), replace=False)) for l in lens]
                         ).astype(np.int32)
    return rp, col, n


def tiny(rng):
    lens = np.array([9, 0, 3, 30, 1, 0, 17])
    rp = np.zeros(lens.size + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    col = np.concatenate([np.sort(rng.choice(40, int(l), replace=False)) for l in lens]
                         ).astype(np.int32)
    return rp, col, 40


def device_arrays(torch, vt, val, x, m):
    if vt == sp.VALUE_F64:
        vd, xt = torch.from_numpy(val).cuda(), torch.float64
    elif vt == sp.VALUE_MIXED_BF16:
        vd, xt = torch.from_numpy(val).cuda().to(torch.bfloat16), torch.float32
    else:
        vd, xt = torch.from_numpy(val.astype(np.float32)).cuda(), torch.float32
    xd = torch.from_numpy(x).cuda().to(xt)
    yd = torch.full((max(m, 1),), float("nan"), dtype=xt, device="cuda")
    return vd, xd, yd


@pytest.mark.parametrize("vt", [sp.VALUE_F64, sp.VALUE_F32, sp.VALUE_MIXED_F32,
                                sp.VALUE_MIXED_BF16])
@pytest.mark.parametrize("shape", ["mixed_rows", "tiny"])
def test_every_schedule_and_variant_bit_exact(cuda_ok, vt, shape):
    import torch
    rng = np.random.default_rng(2024 + vt)
    rp, col, n = mixed_rows(rng) if shape == "mixed_rows" else tiny(rng)
    m = rp.size - 1
    val = rng.integers(-9, 10, col.size).astype(np.float64)
    x = rng.integers(-9, 10, n).astype(np.float64)
    yr = oracle.csr_serial(rp, col, val, x)
    assert np.abs(yr).max() < 2 ** 24
    rpd, cid = torch.from_numpy(rp).cuda(), torch.from_numpy(col).cuda()
    vd, xd, yd = device_arrays(torch, vt, val, x, m)
    ran = 0
    for cfg in tune.candidates():
        try:
            p = sp.Plan(vt, m, n, rpd, cid, seg=cfg[0], tiles_per_worker=cfg[1],
                        warps_per_cta=cfg[2], stages=cfg[3])
        except sp.SpmvError as e:
            # a staged ring that does not fit in shared memory for this value type
            assert cfg[3] > 0 and e.code == sp.BHSPARSE_INVALID_ARGUMENT, (cfg, e)
            continue
        for oh, l2 in VARIANTS:
            p.set_variant(one_head=oh, l2_only=l2)
            assert p.chunk_form()[1] == oh and p.gather_path()[2] == l2
            # both grids of the direct-load kernel: these matrices fit in one wave, so the rule
            # alone would only ever run the static one
            for persistent in ((False, True) if cfg[3] == 0 else (None,)):
                p.set_grid(persistent)
                for _ in range(2):  # a second launch finds the work queue at zero again
                    yd.fill_(float("nan"))
                    p.execute(vd, xd, yd)
                    p.check()
                    y = yd[:m].cpu().double().numpy()
                    bad = int(np.count_nonzero(y != yr))
                    assert bad == 0, (shape, vt, cfg, oh, l2, persistent, bad)
                ran += 1
        p.close()
    assert ran >= 4 * 24 * 2  # every direct schedule in every variant and both grids, and the
    # staged ones that fit


def test_set_variant_keeps_the_rule_with_minus_one(cuda_ok):
    import torch
    rng = np.random.default_rng(5)
    rp, col, n = mixed_rows(rng, m=600, n=900)
    p = sp.Plan(sp.VALUE_F64, rp.size - 1, n, torch.from_numpy(rp).cuda(),
                torch.from_numpy(col).cuda())
    rule = (p.chunk_form()[1], p.gather_path()[2])
    p.set_variant(one_head=not rule[0])
    assert (p.chunk_form()[1], p.gather_path()[2]) == (not rule[0], rule[1])
    p.set_variant(l2_only=not rule[1])
    assert (p.chunk_form()[1], p.gather_path()[2]) == (not rule[0], not rule[1])
    assert p._L.bhsp_plan_set_variant(p._p, 2, 0) == sp.BHSPARSE_INVALID_ARGUMENT
    assert p._L.bhsp_plan_set_variant(p._p, 0, -2) == sp.BHSPARSE_INVALID_ARGUMENT
    p.close()
