"""Build the learned tuner's dataset on a GB300: seeded synthetic matrices, their 16 row-length
features (computed on the device) and the autotuner's timing table for every candidate
schedule (plain FP32 form, median of 3 CUDA-event-timed runs after 1 warm-up).

Matrices: row counts log-uniform in [10,000, 8,000,000]; generator drawn from the batched
workload's mix (2D / 3D stencil, power-law rows, uniform density, block-diagonal 32x32) plus a
single-dense-row case and a 90 %-empty-rows case.  Uniform density is 1e-4 (capped so a matrix
stays under the non-zero budget); any matrix whose generator would exceed the budget
(NNZ_CAP) is drawn with proportionally fewer rows.  Indices [0, 2000) train, [2000, 2200) are
held out.

    python -m benchmark_spmv_using_csr_gb300.tuner_data.build_dataset [out.npz] [count]
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

M_LO, M_HI = 10_000, 8_000_000
NNZ_CAP = 24_000_000
KINDS = ("stencil2d", "stencil3d", "powerlaw", "density", "blockdiag", "dense_row", "empty90")
MEAN_LEN = {"stencil2d": 5, "stencil3d": 27, "powerlaw": 15, "blockdiag": 32, "dense_row": 8,
            "empty90": 1.5}
SEED = 55


def draw(i: int):
    from benchmark_spmv_using_csr_gb300 import gen
    u = gen.uniform(3, SEED * 1_000_003 + i, 0.0, 1.0)
    m = int(round(np.exp(np.log(M_LO) + u[0] * (np.log(M_HI) - np.log(M_LO)))))
    kind = KINDS[min(int(u[1] * len(KINDS)), len(KINDS) - 1)]
    seed = SEED * 7919 + i
    if kind == "density":
        dens = min(1e-4, NNZ_CAP / (float(m) * m))
        return kind, gen.density(m, m, dens, seed=seed)
    m = min(m, int(NNZ_CAP / MEAN_LEN[kind]))
    if kind == "dense_row":
        return kind, gen.mixed_rows(m, m, dense_row=int(u[2] * (m - 1)), mean_len=8, seed=seed)
    if kind == "empty90":
        return kind, gen.mixed_rows(m, m, mean_len=15, empty_frac=0.9, seed=seed)
    return kind, gen.batch_member(m, kind, seed)


def main(out: str, count: int = 2200) -> None:
    import torch

    import benchmark_spmv_using_csr_gb300 as sp
    from benchmark_spmv_using_csr_gb300 import tune
    k = len(tune.candidates())
    feats = np.zeros((count, tune.NUM_FEATURES), np.float32)
    ms = np.zeros((count, k), np.float32)
    meta = np.zeros((count, 3), np.int64)  # m, nnz, kind index
    start = 0
    if os.path.exists(out):  # resume
        d = np.load(out)
        done = int(d["done"])
        feats[:done], ms[:done], meta[:done] = d["features"][:done], d["ms"][:done], d["meta"][:done]
        start = done
    t0 = time.time()
    for i in range(start, count):
        kind, a = draw(i)
        rp, ci = torch.from_numpy(a.row_ptr).cuda(), torch.from_numpy(a.col).cuda()
        val = torch.from_numpy(a.val.astype(np.float32)).cuda()
        x = torch.from_numpy(np.ones(a.n, np.float32)).cuda()
        y = torch.zeros(a.m, dtype=torch.float32, device="cuda")
        feats[i] = tune.row_features(rp, a.n)
        ms[i], _ = tune.autotune(sp.VALUE_F32, rp, ci, val, x, y, warmup=1, reps=3)
        meta[i] = (a.m, a.nnz, KINDS.index(kind))
        del rp, ci, val, x, y
        if (i + 1) % 100 == 0 or i + 1 == count:
            np.savez(out, features=feats, ms=ms, meta=meta, done=i + 1, kinds=np.array(KINDS),
                     candidates=np.array(tune.candidates()), nnz_cap=NNZ_CAP)
            print(f"{i + 1}/{count} matrices, {time.time() - t0:.0f} s", flush=True)
            torch.cuda.empty_cache()


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(here, "gb300_fp32_timings.npz")
    main(out, int(sys.argv[2]) if len(sys.argv) > 2 else 2200)
