"""Build the learned tuner's datasets on a GB300: seeded synthetic matrices, their 16 row-length
features (computed on the device) and the autotuner's timing table for every candidate
schedule (median of 3 CUDA-event-timed runs after 1 warm-up, each after an L2-flushing write),
for each value type: plain FP64, plain FP32, mixed FP32 and mixed BF16 storage.  Each matrix
is generated once and timed in every value type; one timing file per value type
(gb300_<f64|f32|mixed_f32|mixed_bf16>_timings.npz).

Matrices 0-2199: row counts log-uniform in [10,000, 8,000,000]; generator drawn from the
batched workload's mix (2D / 3D stencil, power-law rows, uniform density, block-diagonal 32x32)
plus a single-dense-row case and a 90 %-empty-rows case.  Uniform density is 1e-4 (capped so a
matrix stays under the non-zero budget); any matrix whose generator would exceed the budget
(NNZ_CAP) is drawn with proportionally fewer rows.

Matrices 2200-2399, the large stratum: the same mix with a non-zero target log-uniform in
[24 M, 192 M] (rows = target / the kind's mean row length, at most 8,000,000), the size range of
the benchmark's power-law and 27-point matrices, which the first stratum's budget leaves out.
Their values are drawn on the device (timings do not depend on them), which saves two thirds
of the upload.

Splits (see train.split): train = [0, 2000) and [2200, 2380); held out = [2000, 2200) and
[2380, 2400).

    python -m benchmark_spmv_using_csr_gb300.tuner_data.build_dataset [out_dir] [count]
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


LARGE_START = 2200
LARGE_LO, LARGE_HI = 24_000_000, 192_000_000


def draw(i: int):
    from benchmark_spmv_using_csr_gb300 import gen
    u = gen.uniform(3, SEED * 1_000_003 + i, 0.0, 1.0)
    m = int(round(np.exp(np.log(M_LO) + u[0] * (np.log(M_HI) - np.log(M_LO)))))
    kind = KINDS[min(int(u[1] * len(KINDS)), len(KINDS) - 1)]
    seed = SEED * 7919 + i
    if i >= LARGE_START:
        target = float(np.exp(np.log(LARGE_LO) + u[0] * (np.log(LARGE_HI) - np.log(LARGE_LO))))
        if kind == "density":
            m = int(2_000_000 + u[2] * 6_000_000)
            return kind, gen.density(m, m, target / (float(m) * m), seed=seed)
        m = max(M_LO, min(M_HI, int(target / MEAN_LEN[kind])))
        if kind == "dense_row":
            return kind, gen.mixed_rows(m, m, dense_row=int(u[2] * (m - 1)), mean_len=8, seed=seed)
        if kind == "empty90":
            return kind, gen.mixed_rows(m, m, mean_len=15, empty_frac=0.9, seed=seed)
        return kind, gen.batch_member(m, kind, seed)
    if kind == "density":
        dens = min(1e-4, NNZ_CAP / (float(m) * m))
        return kind, gen.density(m, m, dens, seed=seed)
    m = min(m, int(NNZ_CAP / MEAN_LEN[kind]))
    if kind == "dense_row":
        return kind, gen.mixed_rows(m, m, dense_row=int(u[2] * (m - 1)), mean_len=8, seed=seed)
    if kind == "empty90":
        return kind, gen.mixed_rows(m, m, mean_len=15, empty_frac=0.9, seed=seed)
    return kind, gen.batch_member(m, kind, seed)


def _load(path: str, count: int, k: int):
    feats = np.zeros((count, 16), np.float32)
    ms = np.zeros((count, k), np.float32)
    meta = np.zeros((count, 3), np.int64)  # m, nnz, kind index
    done = 0
    if os.path.exists(path):  # resume
        d = np.load(path)
        if d["ms"].shape[1] == k:
            done = min(int(d["done"]), count)
            feats[:done], ms[:done], meta[:done] = (d["features"][:done], d["ms"][:done],
                                                    d["meta"][:done])
    return feats, ms, meta, done


def main(out_dir: str, count: int = 2400, value_types=None) -> None:
    import torch

    import benchmark_spmv_using_csr_gb300 as sp
    from benchmark_spmv_using_csr_gb300 import tune
    vts = list(sp.VALUE_NAMES) if value_types is None else list(value_types)
    cands = np.array(tune.candidates())
    k = len(cands)
    paths = {vt: os.path.join(out_dir, f"gb300_{sp.VALUE_NAMES[vt]}_timings.npz") for vt in vts}
    state = {vt: _load(paths[vt], count, k) for vt in vts}
    start = min(state[vt][3] for vt in vts)
    t0 = time.time()
    for i in range(start, count):
        kind, a = draw(i)
        rp, ci = torch.from_numpy(a.row_ptr).cuda(), torch.from_numpy(a.col).cuda()
        if i >= LARGE_START:  # values drawn on the device: timings do not depend on them
            g = torch.Generator(device="cuda")
            g.manual_seed(SEED * 7919 + i)
            v64 = torch.empty(a.nnz, dtype=torch.float64, device="cuda").uniform_(-1, 1,
                                                                                 generator=g)
        else:
            v64 = torch.from_numpy(a.val).cuda()
        f = tune.row_features(rp, a.n)
        for vt in vts:
            feats, ms, meta, done = state[vt]
            if i < done:
                continue
            if vt == sp.VALUE_F64:
                val, xt = v64, torch.float64
            elif vt == sp.VALUE_MIXED_BF16:
                val, xt = v64.to(torch.bfloat16), torch.float32
            else:
                val, xt = v64.float(), torch.float32
            x = torch.ones(a.n, dtype=xt, device="cuda")
            y = torch.zeros(a.m, dtype=xt, device="cuda")
            feats[i] = f
            ms[i], _ = tune.autotune(vt, rp, ci, val, x, y, warmup=1, reps=3)
            meta[i] = (a.m, a.nnz, KINDS.index(kind))
            del val, x, y
        del rp, ci, v64
        if (i + 1) % 100 == 0 or i + 1 == count:
            for vt in vts:
                feats, ms, meta, _ = state[vt]
                np.savez(paths[vt], features=feats, ms=ms, meta=meta, done=i + 1,
                         kinds=np.array(KINDS), candidates=cands, nnz_cap=NNZ_CAP, value_type=vt)
            print(f"{i + 1}/{count} matrices, {time.time() - t0:.0f} s", flush=True)
            torch.cuda.empty_cache()


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    out = sys.argv[1] if len(sys.argv) > 1 else here
    main(out, int(sys.argv[2]) if len(sys.argv) > 2 else 2400)
