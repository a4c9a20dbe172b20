"""Run a few SpMVs of one form on one benchmark matrix through the handle API and print their
times: a small, fixed command for timing checks and for profilers (ncu captures of one kernel
launch).

    python -m benchmark_spmv_using_csr_gb300.run_case --workload stencil27_160 \
        --form mixed_f32 [--config S TPW WARPS STAGES] [--steps 5] [--warmup 2]

Without --config the schedule is the one prepare_mem chooses.  Each step is the tile kernel
followed by the calibration kernel, with a 256 MiB write before it so that it starts with the
matrix out of L2; steps are timed with CUDA events.

    python -m benchmark_spmv_using_csr_gb300.run_case --batched K [--config S TPW WARPS 0]

runs the 512-matrix batched workload instead (FP32 storage, K = 1, 2, 4 or 8 right-hand sides),
one graph replay per step, at the given schedule or the batch's default; with --one-matrix, a
batch of the --workload matrix alone (its multi-right-hand-side SpMV).
"""
from __future__ import annotations

import argparse
import statistics

import numpy as np


def main() -> None:
    import torch

    import benchmark_spmv_using_csr_gb300 as sp
    from benchmark_spmv_using_csr_gb300 import gen
    forms = {v: k for k, v in sp.VALUE_NAMES.items()}
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--workload", choices=tuple(gen.WORKLOADS), default="powerlaw_4m")
    ap.add_argument("--form", choices=tuple(forms), default="f64")
    ap.add_argument("--config", type=int, nargs=4, default=None)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--batched", type=int, choices=(1, 2, 4, 8), default=None,
                    help="the 512-matrix batched workload at this many right-hand sides")
    ap.add_argument("--one-matrix", action="store_true",
                    help="with --batched: a batch of the --workload matrix alone")
    args = ap.parse_args()
    if args.batched:
        run_batched(args)
        return
    vt = forms[args.form]
    a = gen.WORKLOADS[args.workload]()
    x = gen.uniform(a.n, 7)
    dt = sp.host_dtype(vt)
    h = sp.BhsparseSpmvCuda(vt)
    if args.config:
        assert h.set_config(*args.config) == 0, h.last_error
    y = np.zeros(a.m, dt)
    assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val.astype(dt), x.astype(dt), y) == 0, \
        h.last_error
    stream = torch.cuda.Stream()
    flush = torch.empty(64 << 20, dtype=torch.int32, device="cuda")
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            assert h.run_phase(stream.cuda_stream, 3) == 0, h.last_error
        evs = []
        for i in range(args.steps):
            flush.fill_(i)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            assert h.run_phase(stream.cuda_stream, 3) == 0, h.last_error
            e1.record(stream)
            evs.append((e0, e1))
    torch.cuda.synchronize()
    assert h.check() == 0, h.last_error
    ms = [p.elapsed_time(q) for p, q in evs]
    src, conf = h.schedule_source()
    print(f"{args.workload} {args.form} m={a.m} nnz={a.nnz} schedule={h.get_config()} "
          f"(source {src}, confidence {conf:.3f}): median {statistics.median(ms):.4f} ms "
          f"over {args.steps} steps")
    h.close()


def run_batched(args) -> None:
    import torch

    from benchmark_spmv_using_csr_gb300 import batch, gen
    k = args.batched
    mats = [gen.WORKLOADS[args.workload]()] if args.one_matrix else gen.batch_workload(512)
    cfg = args.config[:3] if args.config else (0, 0, 0)
    b = batch.Batch(mats, k=k, seg=cfg[0], tiles_per_worker=cfg[1], warps_per_cta=cfg[2])
    x = torch.from_numpy(gen.uniform(b.n * k, 3).reshape(b.n, k).astype(np.float32)).cuda()
    y = torch.zeros((b.m, k), dtype=torch.float32, device="cuda")
    flush = torch.empty(64 << 20, dtype=torch.int32, device="cuda")
    for _ in range(args.warmup):
        b.execute(x, y)
    evs = []
    for i in range(args.steps):
        flush.fill_(i)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        b.execute(x, y)
        e1.record()
        evs.append((e0, e1))
    torch.cuda.synchronize()
    b.check()
    ms = statistics.median(p.elapsed_time(q) for p, q in evs)
    info = b.info()
    sched = tuple(args.config[:3]) if args.config else "default"
    print(f"batched k={k} matrices={len(mats)} nnz={b.nnz} schedule={sched} "
          f"variant=(one_head {info['one_head']}, l2_only {info['x_l2_only']}): median "
          f"{ms:.4f} ms over {args.steps} steps, {b.nnz * k / ms / 1e6:.1f} G nnz*k/s")
    b.close()


if __name__ == "__main__":
    main()
