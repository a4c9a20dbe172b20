"""Seeded random matrices of awkward shapes through the plan API, every value type, a random
schedule and kernel variant per case, bit for bit against the serial loop.

Each case draws a row-length pattern that stresses one part of the path -- all rows empty but
one, a single row longer than many workers, alternating empty rows (dirty tiles everywhere),
power-law lengths, constant lengths at and around the chunk and tile sizes, far more columns
than rows or far more rows than columns -- and integer values whose partial sums are exact in
FP32, so every form (plain FP64 / FP32, compensated FP32 / BF16 storage) must equal the
reference's serial CSR loop (spmv_cuda/main.cu:755-761) exactly, whatever the schedule, kernel
variant and grid (persistent or static, drawn per case).
"""
import numpy as np
import pytest

import oracle

import benchmark_spmv_using_csr_gb300 as sp
from benchmark_spmv_using_csr_gb300 import tune

pytestmark = pytest.mark.gpu

VALUE_TYPES = [sp.VALUE_F64, sp.VALUE_F32, sp.VALUE_MIXED_F32, sp.VALUE_MIXED_BF16]
PATTERNS = ["one_row", "huge_row", "alternating_empty", "powerlaw", "constant", "wide", "tall"]


def lengths(rng, pattern):
    """(row lengths, n) for one pattern; every length is at most n."""
    if pattern == "one_row":
        m, n = int(rng.integers(1, 3000)), int(rng.integers(1, 5000))
        lens = np.zeros(m, np.int64)
        lens[rng.integers(0, m)] = rng.integers(1, n + 1)
    elif pattern == "huge_row":
        m, n = int(rng.integers(2, 400)), int(rng.integers(20000, 60000))
        lens = rng.integers(0, 5, m)
        lens[rng.integers(0, m)] = rng.integers(n // 2, n + 1)
    elif pattern == "alternating_empty":
        m, n = int(rng.integers(2, 8000)), int(rng.integers(1, 3000))
        lens = rng.integers(1, 40, m)
        lens[int(rng.integers(0, 2))::2] = 0
    elif pattern == "powerlaw":
        m, n = int(rng.integers(100, 20000)), int(rng.integers(100, 20000))
        lens = np.floor(rng.pareto(1.1, m) + 1).astype(np.int64)
        lens[rng.random(m) < 0.05] = 0
    elif pattern == "constant":
        m, n = int(rng.integers(1, 6000)), int(rng.integers(64, 3000))
        lens = np.full(m, int(rng.choice([1, 3, 4, 5, 7, 8, 9, 15, 16, 17, 31, 32, 33, 63])))
    elif pattern == "wide":
        m, n = int(rng.integers(1, 50)), int(rng.integers(50000, 200000))
        lens = rng.integers(0, 3000, m)
    else:  # tall
        m, n = int(rng.integers(20000, 80000)), int(rng.integers(1, 8))
        lens = rng.integers(0, n + 1, m)
    return np.minimum(lens, n), n


def csr(rng, pattern):
    lens, n = lengths(rng, pattern)
    rp = np.zeros(lens.size + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    col = (np.concatenate([np.sort(rng.choice(n, int(l), replace=False)) for l in lens if l])
           .astype(np.int32) if rp[-1] else np.zeros(0, np.int32))
    return rp, col, n


@pytest.mark.parametrize("vt", VALUE_TYPES)
def test_fuzz_bit_exact(cuda_ok, vt):
    import torch
    rng = np.random.default_rng(777 + vt)
    cands = tune.candidates()
    cases = 0
    for i in range(8 * len(PATTERNS)):
        pattern = PATTERNS[i % len(PATTERNS)]
        rp, col, n = csr(rng, pattern)
        m, nnz = rp.size - 1, int(rp[-1])
        val = rng.integers(-9, 10, nnz).astype(np.float64)
        x = rng.integers(-9, 10, n).astype(np.float64)
        yr = oracle.csr_serial(rp, col, val, x)
        if nnz and np.abs(yr).max() >= 2 ** 24:
            continue
        cfg = cands[int(rng.integers(0, len(cands)))]
        rpd = torch.from_numpy(rp).cuda()
        cid = torch.from_numpy(col).cuda() if nnz else torch.zeros(8, dtype=torch.int32,
                                                                      device="cuda")
        try:
            p = sp.Plan(vt, m, n, rpd, cid, nnz=nnz, seg=cfg[0], tiles_per_worker=cfg[1],
                        warps_per_cta=cfg[2], stages=cfg[3])
        except sp.SpmvError as e:  # a staged ring that does not fit for this value type
            assert cfg[3] > 0 and e.code == sp.BHSPARSE_INVALID_ARGUMENT, (cfg, e)
            continue
        oh, l2 = bool(rng.integers(0, 2)), bool(rng.integers(0, 2))
        p.set_variant(one_head=oh, l2_only=l2)
        p.set_grid(bool(rng.integers(0, 2)))
        if vt == sp.VALUE_F64:
            vd, xt = torch.from_numpy(val).cuda(), torch.float64
        elif vt == sp.VALUE_MIXED_BF16:
            vd, xt = torch.from_numpy(val).cuda().to(torch.bfloat16), torch.float32
        else:
            vd, xt = torch.from_numpy(val.astype(np.float32)).cuda(), torch.float32
        if not nnz:
            vd = torch.zeros(8, dtype=vd.dtype, device="cuda")
        xd = torch.from_numpy(x).cuda().to(xt)
        yd = torch.full((max(m, 1),), float("nan"), dtype=xt, device="cuda")
        for _ in range(2):  # a repeated call gives the same y
            p.execute(vd, xd, yd)
        p.check()
        p.close()
        y = yd[:m].cpu().double().numpy()
        bad = int(np.count_nonzero(y != yr))
        assert bad == 0, (i, pattern, m, n, nnz, cfg, oh, l2, bad)
        cases += 1
    assert cases >= 6 * len(PATTERNS)
