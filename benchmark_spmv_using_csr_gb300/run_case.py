"""Run a few SpMVs of one form on one benchmark matrix through the handle API and print their
times: a small, fixed command for timing checks and for profilers (ncu captures of one kernel
launch).

    python -m benchmark_spmv_using_csr_gb300.run_case --workload stencil27_160 \
        --form mixed_f32 [--config S TPW WARPS STAGES] [--steps 5] [--warmup 2]

Without --config the schedule is the one prepare_mem chooses.  Each step is the tile kernel
followed by the calibration kernel, with a 256 MiB write before it so that it starts with the
matrix out of L2; steps are timed with CUDA events.
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
    args = ap.parse_args()
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


if __name__ == "__main__":
    main()
