#!/usr/bin/env python
"""Benchmark: plain FP64 speculative segmented-sum SpMV on one GB300 (per rank).

Workload (default ``powerlaw_4m``): m = n = 4,194,304, Zipf(2.1)-tailed row lengths
clipped to [1, 200,000], 5 % empty rows, about 59 M non-zeros, values and x uniform[-1, 1]
(seeded synthetic data, see benchmark_spmv_using_csr_gb300/gen.py).  One step = one
y = A.x through the library (the tile kernel + the calibration kernel).

Metric: SpMV HBM GB/s on the algorithmic bytes B = nnz*(s_val+4) + (m+1)*4 + n*s_x + m*s_y
(val + col_idx + row_ptr + x + y, each counted once).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload powerlaw_4m|stencil27_160|stencil5_256] [--no-forms]

* ``value``: B / (device time per step), inputs resident in HBM, L2 flushed (256 MiB
  write) before every timed step, CUDA events on the launching stream, max over ranks.
* ``e2e``: the same metric through the C ABI with host buffers, every step's x uploaded from
  pinned host memory and its y downloaded inside the timed region: bhsp_run_stream over the
  K steps (copies of neighbouring steps overlap each SpMV); ``e2e.per_call`` is the
  reference's per-call sequence bhsp_set_x / bhsp_run_benchmark / bhsp_get_y.
* ``sector_roofline`` (power-law matrix): L2 -> SM sectors per second against the random-gather
  probe's rate (323 G sectors/s), the unit that binds on that matrix.
* ``roofline``: the tile kernel alone (launched on its own between CUDA events, L2 flushed
  before each) against the measured HBM copy bandwidth.
* ``cpu_baseline``: the reference's serial CSR loop (spmv_cuda/main.cu:755-761) on one host
  core over whole-matrix passes, and its OpenMP loop at 4 and all threads: the reference's own
  loops compiled from its source (oracle/_ref) where they were built, else the ports in oracle/.
* ``--impl reference``: the reference's OpenMP CSR loop (spmv_cuda/main.cu:377-393, its own
  code from oracle/_ref, else the port) on all host cores, same workload / metric.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "SpMV HBM GB/s (% of peak), mixed/batched vs plain FP64 at stated rel. error"
UNIT = "GB/s"
FALLBACK_HBM_GBS = 6800.0
FLUSH_BYTES = 256 << 20
# 32-byte sectors per second the SMs take from L2 for random access, measured on GB300 by
# `python -m benchmark_spmv_using_csr_gb300.probes`: 64 M fully random 8-byte gathers into a
# 33.5 MB L2-resident vector, with their int32 column indices streamed beside them (one sector
# per gather + 1/8 sector of index each): 287 G gathers/s, the same through ld.global.nc,
# ld.global.cg and ld.global
SECTOR_PEAK_G = 323.0


def l2_sectors(a) -> int:
    """Algorithmic L2 -> SM sectors of one plain-FP64 SpMV: one per x gather (random columns)
    plus the val, col_idx and row_ptr streams in 32-byte sectors."""
    return int(a.nnz + (a.nnz * 12 + (a.m + 1) * 4 + 31) // 32)

WORKLOAD_TEXT = {
    "powerlaw_4m": "power-law m=n=4,194,304: row lengths floor(1.98*U^(-1/1.1)) clipped to "
                   "[1,200000] (Zipf 2.1 tail), 5% rows empty, distinct sorted uniform columns, "
                   "val and x uniform[-1,1]; plain FP64 (USE_DOUBLE=1)",
    "stencil27_160": "27-point stencil on a 160^3 grid, m=n=4,096,000, nnz=109,215,352, "
                     "weights 26/-1 x (1+U[-0.01,0.01]), x uniform[-1,1]; plain FP64",
    "stencil5_256": "5-point Laplacian on a 256^2 grid, m=n=65,536, nnz=326,656, values 4/-1 + "
                    "U[-1e-3,1e-3], x uniform[-1,1]; plain FP64",
}


def alg_bytes(m: int, n: int, nnz: int, s_v: int, s_x: int, s_y: int, k: int = 1) -> int:
    return nnz * (s_v + 4) + (m + 1) * 4 + n * k * s_x + m * k * s_y


def reference_formula_bytes(m: int, nnz: int, s_v: int) -> int:
    """spmv_cuda/main.cu:688 (counts x once per non-zero)."""
    return (m + 1 + nnz) * 4 + (2 * nnz + m) * s_v


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(kernel_workload: str):
    """Per-launch DRAM bytes of the tile kernel from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", f"{kernel_workload}.txt")
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_launch"):
                return int(float(line.split("=")[1].split()[0]))
    except Exception:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 100 ms while running."""

    FIELDS = ("uuid,clocks.sm,clocks.max.sm,power.draw,utilization.gpu,"
              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid: str | None):
        self.uuid = uuid
        self.proc = None
        self.out = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        rows = []
        for line in out.splitlines():
            f = [v.strip() for v in line.split(",")]
            if len(f) < 10:
                continue
            if self.uuid and self.uuid not in f[0]:
                continue
            rows.append(f)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None
        loaded = [r for r in rows if (num(r[4]) or 0) > 0] or rows
        sm = [num(r[1]) for r in loaded if num(r[1])]
        reasons = set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in loaded:
            for name, v in zip(names, r[6:10]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": num(loaded[0][2]), "samples": len(loaded),
                "power_w_max": max((num(r[3]) or 0) for r in loaded), "reasons": sorted(reasons)}


def make_workload(name: str, cpu_only: bool = False):
    """The seeded workload and its x.  cpu_only: take the generators from oracle/'s own build of
    the generator source instead of the GPU library (the reference arm loads no product code)."""
    from benchmark_spmv_using_csr_gb300 import gen
    if cpu_only:
        import oracle
        gen.use_library(oracle.gen_library_path())
    a = gen.WORKLOADS[name]()
    x = gen.uniform(a.n, 7)
    return a, x


def l2_text(a) -> str:
    mb = alg_bytes(a.m, a.n, a.nnz, 8, 8, 8) / 1e6
    size = (f"inputs larger than L2 ({mb:.0f} MB of algorithmic bytes against a 129 MB L2)"
            if mb > 129 else f"inputs of {mb:.1f} MB, which fit in the 129 MB L2")
    return size + "; the GPU arm writes 256 MiB before every timed step to flush L2"


def workload_config(name: str, a, x) -> dict:
    """The `config` object both arms print: the workload, its sizes, its algorithmic bytes and a
    CRC-32 of its arrays (row_ptr, col_idx, val, x), which shows that both arms ran the same
    matrix."""
    import zlib

    import numpy as np
    crc = 0
    for arr in (a.row_ptr, a.col, a.val, x):
        crc = zlib.crc32(np.ascontiguousarray(arr).view(np.uint8), crc)
    return {"workload": name, "description": WORKLOAD_TEXT[name], "m": a.m, "n": a.n,
            "nnz": a.nnz, "bytes_per_step": alg_bytes(a.m, a.n, a.nnz, 8, 8, 8),
            "matrix_crc32": f"{crc:08x}", "l2": l2_text(a)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(seconds: float, dist=None) -> float:
    """The slowest rank's time: each rank's seconds all-reduced with MAX (a CUDA tensor under
    NCCL, a host tensor under gloo); the local value when there is no process group."""
    if dist is None:
        return seconds
    import torch
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_gbs(world: int, bytes_per_step: int, steps: int, seconds: float) -> float:
    """Aggregate GB/s of `world` replicas that each moved bytes_per_step * steps bytes, timed by
    the slowest rank (weak scaling: the per-rank work is fixed)."""
    return world * bytes_per_step * steps / seconds / 1e9


# ---------------------------------------------------------------------------------------
# reference arm: the reference's CPU path (port) on all host cores
# ---------------------------------------------------------------------------------------
def run_reference(args) -> None:
    """The reference's CPU path on all host cores: its own OpenMP CSR loop (spmv_cuda/main.cu:
    377-393) compiled from its sources into oracle/_ref/libref.so where that was built, else the
    C port in oracle/.  Rank 0 only; no GPU library is loaded."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import numpy as np
    import oracle
    a, x = make_workload(args.workload, cpu_only=True)
    threads = os.cpu_count() or 1
    B = alg_bytes(a.m, a.n, a.nnz, 8, 8, 8)
    y = np.zeros(a.m)
    if oracle.ref_lib() is not None:
        kind = "reference"
        what = ("the reference's own OpenMP CSR loop (spmv_cuda/main.cu:377-393), compiled from "
                "its source by oracle/Makefile (oracle/_ref/libref.so)")

        def step():
            oracle.ref_omp(a.row_ptr, a.col, a.val, x, threads, runs=1, y=y)
    else:
        kind = "port"
        what = ("the C port of the reference's OpenMP CSR loop (spmv_cuda/main.cu:377-393) in "
                "oracle/; the reference's own loop was not compiled on this host")

        def step():
            oracle.csr_omp(a.row_ptr, a.col, a.val, x, threads, y=y)
    for _ in range(args.warmup):
        step()
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        ts.append(time.perf_counter() - t0)
    sec = sum(ts)
    value = B * args.steps / sec / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 2), "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * sec / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": workload_config(args.workload, a, x),
        "parallelism": f"{threads} host threads (rank 0 only)",
        "cpu_baseline": {"value": round(value, 2), "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": f"one whole-matrix pass per step, {args.steps} steps: {what}"},
        "e2e": {"value": round(value, 2), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------------------
def run_ours(args) -> None:
    import numpy as np
    import torch

    import benchmark_spmv_using_csr_gb300 as sp
    import oracle

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if not os.path.exists(sp.LIB_PATH):
        sp.build()

    a, x = make_workload(args.workload)
    B = alg_bytes(a.m, a.n, a.nnz, 8, 8, 8)

    def barrier():
        if dist is not None:
            dist.barrier()

    # pinned host buffers for x and y (the e2e leg reads / writes them every step)
    x_pin = torch.from_numpy(x).pin_memory()
    y_pin = torch.zeros(a.m, dtype=torch.float64).pin_memory()
    y_np = y_pin.numpy()
    # the autotuner's full table on this matrix, for the report: the schedule itself is the one
    # prepare_mem chooses (the learned network, or the sweep below its confidence threshold),
    # as for any caller of the reference's API, unless --config sets one
    tuning = autotune_workload(a, x) if args.tune_table else None
    h = sp.BhsparseSpmvCuda(sp.VALUE_F64)
    if args.config is not None:
        assert h.set_config(*args.config) == 0, h.last_error
    assert h.set_device(local) == 0
    assert h.init_platform() == 0, h.last_error
    t_prep = time.perf_counter()
    rc = h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val, x_pin.numpy(), y_np)
    assert rc == 0, h.last_error
    t_prep = time.perf_counter() - t_prep
    seg, tpw, warps, stages = h.get_config()
    choice = schedule_choice(h, tuning)
    if tuning is not None:
        tuning["prepare_mem_choice"] = choice

    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")

    def step_async():
        assert h.run_phase(sptr, 3) == 0, h.last_error

    # warm-up, then a short soak so that the clock sampler sees the GPU under this load
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step_async()
    assert h.check() == 0, h.last_error
    try:
        uuid = str(torch.cuda.get_device_properties(local).uuid)
    except Exception:
        uuid = None
    sampler = ClockSampler(uuid)
    sampler.start()
    t_end = time.perf_counter() + args.soak
    with torch.cuda.stream(stream):
        while time.perf_counter() < t_end:
            for _ in range(20):
                flush.fill_(1)
                step_async()
            stream.synchronize()

    # timed region: exactly K steps (tile kernel + calibration, the calibration launched as a
    # programmatic dependent), L2 flushed before each, CUDA events around each step
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            e0, e1 = ev[i]
            e0.record(stream)
            assert h.run_phase(sptr, 3) == 0, h.last_error
            e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    assert h.check() == 0, h.last_error
    step_ms = [e0.elapsed_time(e1) for e0, e1 in ev]
    total_s = max_over_ranks(sum(step_ms) / 1e3, dist)
    value = whole_job_gbs(world, B, args.steps, total_s)

    # the tile kernel alone (roofline) and the calibration alone, each launched on its own
    # between events, on the same flushed-L2 footing (outside the timed region)
    kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
            torch.cuda.Event(enable_timing=True)) for _ in range(min(args.steps, 50))]
    with torch.cuda.stream(stream):
        for i, (e0, e1, e2) in enumerate(kev):
            flush.fill_(i & 0xFF)
            e0.record(stream)
            assert h.run_phase(sptr, 1) == 0, h.last_error
            e1.record(stream)
            assert h.run_phase(sptr, 2) == 0, h.last_error
            e2.record(stream)
    torch.cuda.synchronize()
    assert h.check() == 0, h.last_error
    kern_ms = [e0.elapsed_time(e1) for e0, e1, _ in kev]
    cal_ms = [e1.elapsed_time(e2) for _, e1, e2 in kev]

    # end to end through the C ABI with host buffers (pinned), copies inside the timed region:
    # (1) bhsp_run_stream over the K steps' right-hand sides (two pinned x and y buffers used
    #     alternately), each step's x uploaded and y downloaded, overlapping the neighbouring
    #     SpMVs; (2) the reference's per-call sequence set_x / run_benchmark / get_y
    x_pin2 = torch.from_numpy(x[::-1].copy()).pin_memory()
    y_pin2 = torch.zeros(a.m, dtype=torch.float64).pin_memory()
    xs = [(x_pin if i % 2 == 0 else x_pin2).data_ptr() for i in range(args.steps)]
    ys = [(y_pin if i % 2 == 0 else y_pin2).data_ptr() for i in range(args.steps)]
    assert h.run_stream(xs[:4], ys[:4]) == 0, h.last_error
    barrier()
    t0 = time.perf_counter()
    assert h.run_stream(xs, ys) == 0, h.last_error
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    barrier()
    e2e_value = whole_job_gbs(world, B, args.steps, e2e_s)
    x_ptr = x_pin.data_ptr()
    for _ in range(3):
        assert h.set_x_ptr(x_ptr) == 0 and h.run_benchmark() == 0 and h.get_y() == 0
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        assert h.set_x_ptr(x_ptr) == 0, h.last_error
        assert h.run_benchmark() == 0, h.last_error
        assert h.get_y() == 0, h.last_error
    e2e_call_s = max_over_ranks(time.perf_counter() - t0, dist)
    barrier()
    e2e_call_value = whole_job_gbs(world, B, args.steps, e2e_call_s)
    # the same per-call sequence on pageable host arrays, as the reference's driver allocates them
    # (malloc); a second handle at the same schedule
    x_pg, y_pg = x.copy(), np.zeros(a.m)
    h2 = sp.BhsparseSpmvCuda(sp.VALUE_F64)
    assert h2.set_config(seg, tpw, warps, stages) == 0 and h2.set_device(local) == 0
    assert h2.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val, x_pg, y_pg) == 0, h2.last_error
    for _ in range(3):
        assert h2.set_x(x_pg) == 0 and h2.run_benchmark() == 0 and h2.get_y() == 0
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        assert h2.set_x(x_pg) == 0, h2.last_error
        assert h2.run_benchmark() == 0, h2.last_error
        assert h2.get_y() == 0, h2.last_error
    e2e_pg_s = max_over_ranks(time.perf_counter() - t0, dist)
    barrier()
    e2e_pg_value = whole_job_gbs(world, B, args.steps, e2e_pg_s)
    assert np.array_equal(y_pg, y_np)
    h2.free_mem()
    h2.close()

    # correctness of the benchmarked y against the FP64 compensated oracle
    ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, x)
    scale = oracle.csr_absrow(a.row_ptr, a.col, a.val, x)
    rel_err = oracle.componentwise_error(y_np, ystar, scale)

    line = None
    if rank == 0:
        peak, peak_kind = measured_peak()
        kmean = statistics.mean(kern_ms)
        achieved = B / (kmean * 1e-3) / 1e9
        kw = f"k_tiles_f64_{args.workload}"
        traffic = profile_traffic(kw)
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(statistics.mean(step_ms), 5), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generators; no dataset)",
            "config": workload_config(args.workload, a, x),
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "reference_formula_bytes": reference_formula_bytes(a.m, a.nnz, 8),
            "schedule": {"nnz_per_lane": seg, "tiles_per_worker": tpw, "warps_per_cta": warps,
                         "tma_stages": stages},
            "pct_peak": round(100.0 * value / peak, 2),
            "rel_error": {"componentwise_vs_fp64_dot2": rel_err, "tolerance": 1e-12},
            "phases_ms": {"tile_kernel": round(kmean, 5),
                          "calibration_alone": round(statistics.mean(cal_ms), 5),
                          "note": "each phase launched alone between events; in the timed "
                                  "steps the calibration is a programmatic dependent of the "
                                  "tile kernel"},
            "sector_roofline": None if args.workload != "powerlaw_4m" else {
                "unit": "G sectors/s", "achieved": round(l2_sectors(a) / (kmean * 1e-3) / 1e9, 1),
                "peak": SECTOR_PEAK_G,
                "frac": round(l2_sectors(a) / (kmean * 1e-3) / 1e9 / SECTOR_PEAK_G, 3),
                "sectors_per_launch": l2_sectors(a),
                "note": "32-byte sectors the SMs take from L2 per SpMV (one per random x gather, "
                        "plus val / col_idx / row_ptr at 32 bytes a sector) against the sector "
                        "rate of a probe of fully random gathers, with streamed indices, into an "
                        "L2-resident vector on GB300 (~1 sector per clock per SM, equal for the "
                        "read-only, L2-only and plain load paths); the binding unit on this "
                        "matrix"},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "traffic": traffic, "peak_kind": f"{peak_kind} (hbm_gbs copy, burst)",
                         "kernel": "FP64 tile kernel alone (k_tiles_persistent<PolF64> above one "
                                   "wave of workers, else k_tiles<PolF64>)"},
            "e2e": {"value": round(e2e_value, 2), "unit": UNIT,
                    "h2d_bytes_per_step": a.n * 8, "d2h_bytes_per_step": a.m * 8,
                    "path": "bhsp_run_stream over the K steps' pinned host x / y (upload of "
                            "x_{i+1} and download of y_{i-1} overlap SpMV i)",
                    "per_call": {"value": round(e2e_call_value, 2), "unit": UNIT,
                                 "path": "bhsp_set_x + bhsp_run_benchmark + bhsp_get_y per "
                                         "step, pinned host x / y"},
                    "per_call_pageable": {"value": round(e2e_pg_value, 2), "unit": UNIT,
                                          "path": "the same per-call sequence on pageable "
                                                  "(malloc'd) host x / y: x read by a copy "
                                                  "kernel where the device reads pageable "
                                                  "memory, y written back by cudaMemcpy"}},
            "tuning": tuning if tuning is not None else {"prepare_mem_choice": choice},
            "gpu_launches": 2 * args.steps,
            "clocks": clocks,
            "prepare_mem_s": round(t_prep, 3),
        }
    h.free_mem()
    h.close()

    if rank == 0 and args.forms:
        line["forms"] = measure_forms(args, a, x, ystar)
        line["comparators"] = measure_comparators(args, a, x, ystar)
    if rank == 0 and args.forms:
        line["other_configs"] = measure_other_configs(args)
    if rank == 0 and args.batched:
        line["batched"] = measure_batched(args)
    if rank == 0 and args.cpu_baseline > 0:
        line["cpu_baseline"] = cpu_baseline(a, x, B, args.cpu_baseline)
        line["cpu_baseline"]["openmp"] = cpu_openmp(a, x, B, max(1.0, args.cpu_baseline / 5))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def measure_forms(args, a, x, ystar) -> dict:
    """The other value types on the same workload: device GB/s on their own algorithmic
    bytes, non-zeros/s, and their error against the FP64 oracle.  Each form runs the schedule
    its handle's prepare_mem chooses (that value type's learned network, or the sweep), shown
    beside the autotuner's table for that value type."""
    import torch

    import benchmark_spmv_using_csr_gb300 as sp
    import oracle
    out = {}
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    steps = max(10, min(args.steps, 50))
    for vt, sv, sx in ((sp.VALUE_F32, 4, 4), (sp.VALUE_MIXED_F32, 4, 4), (sp.VALUE_MIXED_BF16, 2, 4)):
        tuning = autotune_workload(a, x, vt)
        r = _time_form(vt, None, a, x, flush, steps, tuning)
        if "error" in r:
            out[sp.VALUE_NAMES[vt]] = {"error": r["error"]}
            continue
        ms, y = r["ms"], r["y"]
        Bf = alg_bytes(a.m, a.n, a.nnz, sv, sx, 4)
        out[sp.VALUE_NAMES[vt]] = {
            "gbs": round(Bf / (ms * 1e-3) / 1e9, 1), "ms_per_step": round(ms, 5),
            "gnnz_per_s": round(a.nnz / (ms * 1e-3) / 1e9, 2), "schedule": r["choice"],
            "autotuner_best": {"schedule": tuning["pick"], "ms": round(tuning["best_ms"], 5)},
            "normwise_err_vs_fp64_oracle": oracle.normwise_error(y, ystar)}
    return out


def _time_form(vt, cfg, a, x, flush, steps, tuning=None) -> dict:
    """Whole steps of one value type through the handle (L2 flushed before each, CUDA events),
    at schedule cfg or, with cfg None, the one prepare_mem chooses: {"ms", "y", "choice"} or
    {"error"}."""
    import numpy as np
    import torch

    import benchmark_spmv_using_csr_gb300 as sp
    h = sp.BhsparseSpmvCuda(vt)
    if cfg is not None:
        assert h.set_config(*cfg) == 0, h.last_error
    dt = sp.host_dtype(vt)
    y = np.zeros(a.m, dt)
    if h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val.astype(dt), x.astype(dt), y):
        err = h.last_error
        h.close()
        return {"error": err}
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        for _ in range(5):
            h.run_phase(stream.cuda_stream, 3)
        evs = []
        for i in range(steps):
            flush.fill_(i & 0xFF)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            h.run_phase(stream.cuda_stream, 3)
            e1.record(stream)
            evs.append((e0, e1))
    torch.cuda.synchronize()
    assert h.check() == 0, h.last_error
    ms = statistics.mean(e0.elapsed_time(e1) for e0, e1 in evs)
    assert h.get_y() == 0
    choice = schedule_choice(h, tuning)
    h.close()
    return {"ms": ms, "y": y, "choice": choice}


def measure_fp64(args, a, x, config=None) -> dict:
    """Plain FP64 through the handle on one matrix: device GB/s per whole step (L2 flushed
    before each, CUDA events), the schedule (prepare_mem's choice unless given, beside the
    autotuner's best), and the componentwise error against the FP64 compensated oracle."""
    import numpy as np
    import torch

    import benchmark_spmv_using_csr_gb300 as sp
    import oracle
    tuning = autotune_workload(a, x)
    h = sp.BhsparseSpmvCuda(sp.VALUE_F64)
    if config is not None:
        assert h.set_config(*config) == 0, h.last_error
    y = np.zeros(max(a.m, 1))
    assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val, x, y) == 0, h.last_error
    choice = schedule_choice(h, tuning)
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    steps = max(10, min(args.steps, 50))
    with torch.cuda.stream(stream):
        for _ in range(5):
            assert h.run_phase(sptr, 3) == 0, h.last_error
        evs = []
        for i in range(steps):
            flush.fill_(i & 0xFF)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            assert h.run_phase(sptr, 3) == 0, h.last_error
            e1.record(stream)
            evs.append((e0, e1))
    torch.cuda.synchronize()
    assert h.check() == 0 and h.get_y() == 0, h.last_error
    ms = statistics.mean(e0.elapsed_time(e1) for e0, e1 in evs)
    B = alg_bytes(a.m, a.n, a.nnz, 8, 8, 8)
    err = oracle.componentwise_error(y[:a.m], oracle.csr_dot2(a.row_ptr, a.col, a.val, x),
                                     oracle.csr_absrow(a.row_ptr, a.col, a.val, x))
    h.close()
    return {"gbs": round(B / (ms * 1e-3) / 1e9, 1), "ms_per_step": round(ms, 5),
            "pct_of_peak": round(100 * B / (ms * 1e-3) / 1e9 / measured_peak()[0], 1),
            "bytes_per_step": B, "schedule": choice,
            "autotuner_best": {"schedule": tuning["pick"], "ms": round(tuning["best_ms"], 5)},
            "componentwise_err_vs_fp64_oracle": err, "tolerance": 1e-12}


def measure_other_configs(args) -> dict:
    """The benchmark's other matrices: the 27-point stencil (plain FP64 and the FP32- and
    BF16-stored forms with their errors) and the 5-point Laplacian (plain FP64; the case the
    reference runs on the CPU, with the serial loop's rate beside it)."""
    import oracle
    out = {}
    a, x = make_workload("stencil27_160")
    ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, x)
    out["stencil27_160"] = {"m": a.m, "nnz": a.nnz, "fp64": measure_fp64(args, a, x),
                            "forms": measure_forms(args, a, x, ystar)}
    del a, x, ystar
    a, x = make_workload("stencil5_256")
    B = alg_bytes(a.m, a.n, a.nnz, 8, 8, 8)
    r = measure_fp64(args, a, x)
    r["note"] = "5.2 MB of bytes: L2-resident after the flush write and launch-bound"
    out["stencil5_256"] = {"m": a.m, "nnz": a.nnz, "fp64": r,
                           "cpu_serial": cpu_baseline(a, x, B, 1.0)}
    return out


def measure_comparators(args, a, x, ystar) -> dict:
    """The reference driver's GPU comparators on the same FP64 matrix (include/spmv_compare.h):
    the CSR-vector kernel with the CUSP schedule and cuSPARSE's generic SpMV, each timed like
    the headline (L2 flushed before every launch, CUDA events, same algorithmic bytes)."""
    import numpy as np
    import torch

    import benchmark_spmv_using_csr_gb300 as sp
    import oracle
    from benchmark_spmv_using_csr_gb300 import compare
    rp, ci = torch.from_numpy(a.row_ptr).cuda(), torch.from_numpy(a.col).cuda()
    val, xd = torch.from_numpy(a.val).cuda(), torch.from_numpy(x).cuda()
    y = torch.zeros(a.m, dtype=torch.float64, device="cuda")
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    B = alg_bytes(a.m, a.n, a.nnz, 8, 8, 8)
    steps = max(10, min(args.steps, 50))
    scale = oracle.csr_absrow(a.row_ptr, a.col, a.val, x)

    def timed(fn):
        for _ in range(3):
            fn()
        evs = []
        for i in range(steps):
            flush.fill_(i & 0xFF)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            evs.append((e0, e1))
        torch.cuda.synchronize()
        ms = statistics.mean(e0.elapsed_time(e1) for e0, e1 in evs)
        err = oracle.componentwise_error(y.cpu().numpy(), ystar, scale)
        return {"gbs": round(B / (ms * 1e-3) / 1e9, 1), "ms_per_step": round(ms, 5),
                "componentwise_err_vs_fp64_oracle": err}

    out = {}
    tpv = compare.vector_width(a.m, a.nnz)
    out["csr_vector"] = timed(lambda: compare.csr_vector(sp.VALUE_F64, rp, ci, val, xd, y, tpv))
    out["csr_vector"]["threads_per_row"] = tpv
    try:
        cs = compare.Cusparse(sp.VALUE_F64, rp, ci, val, xd, y)
        out["cusparse_spmv_csr_alg1"] = timed(cs.run)
        cs.close()
    except RuntimeError as e:
        out["cusparse_spmv_csr_alg1"] = {"unavailable": str(e)}
    del rp, ci, val, xd, y, flush
    torch.cuda.empty_cache()
    return out


def cpu_openmp(a, x, B, seconds: float) -> dict:
    """The reference's OpenMP CSR loop (spmv_cuda/main.cu:377-393) at its 4 threads
    (main.cu:370) and at every host thread, whole-matrix passes for about `seconds` each: the
    reference's own loop from oracle/_ref where it was built, else the oracle's C port."""
    import numpy as np
    import oracle
    ref = oracle.ref_lib() is not None
    y = np.zeros(max(a.m, 1))
    out = {"kind": "reference" if ref else "port"}
    for label, threads in (("threads_4", 4), ("threads_all", os.cpu_count() or 1)):
        passes = 0
        t0 = time.perf_counter()
        while True:
            if ref:
                oracle.ref_omp(a.row_ptr, a.col, a.val, x, threads, runs=1, y=y)
            else:
                oracle.csr_omp(a.row_ptr, a.col, a.val, x, threads, y=y)
            passes += 1
            el = time.perf_counter() - t0
            if el >= seconds:
                break
        out[label] = {"value": round(B * passes / el / 1e9, 3), "unit": UNIT, "cores": threads,
                      "passes": passes}
    return out


SOURCE_NAMES = {0: "caller (--config)", 1: "fixed default (no network)", 2: "learned network",
                3: "autotune sweep (network below its confidence threshold)"}


def schedule_choice(h, tuning) -> dict:
    """The schedule prepare_mem chose, where it came from, and its time in the autotuner's table
    as a fraction of the best."""
    src, conf = h.schedule_source()
    cfg = tuple(h.get_config())
    key = ",".join(map(str, cfg))
    t = tuning["table_ms"].get(key) if tuning else None
    return {"schedule": list(cfg), "source": SOURCE_NAMES.get(src, str(src)),
            "confidence": round(conf, 4),
            "frac_of_autotuner_best": round(tuning["best_ms"] / t, 4) if t else None}


def autotune_workload(a, x, vt=None) -> dict:
    """Run the library's autotuner (every candidate schedule, median of 11 timed runs, L2
    flushed before each) on the workload in value type vt (plain FP64 by default) and return
    its table and pick."""
    import torch

    import benchmark_spmv_using_csr_gb300 as sp
    from benchmark_spmv_using_csr_gb300 import tune
    vt = sp.VALUE_F64 if vt is None else vt
    rp, ci = torch.from_numpy(a.row_ptr).cuda(), torch.from_numpy(a.col).cuda()
    val, xd = torch.from_numpy(a.val).cuda(), torch.from_numpy(x).cuda()
    if vt != sp.VALUE_F64:  # storage types of the other forms; x and y in FP32
        val = val.to(torch.bfloat16 if vt == sp.VALUE_MIXED_BF16 else torch.float32)
        xd = xd.float()
    y = torch.zeros(a.m, dtype=xd.dtype, device="cuda")
    ms, best = tune.autotune(vt, rp, ci, val, xd, y, warmup=2, reps=11)
    cands = tune.candidates()
    del rp, ci, val, xd, y
    torch.cuda.empty_cache()
    return {"pick": list(cands[best]), "best_ms": float(ms[best]),
            "table_ms": {",".join(map(str, c)): round(float(t), 4) for c, t in zip(cands, ms)}}


def measure_batched(args) -> dict:
    """The batched workload: 512 matrices (rows log-uniform in [1e3, 2e5], mixed generators),
    FP32 storage with compensated accumulation, k right-hand sides, one persistent kernel
    replayed from a CUDA graph at the batched autotuner's pick -- against the plain FP64 form
    launched once per matrix and right-hand side (512*k sequential plain launches), and against
    the plain FP64 form on the whole concatenated block-diagonal matrix at its autotuned
    schedule (one SpMV per right-hand side).  nnz*k per second, and the normwise error of a
    subset of matrices against the FP64 oracle."""
    import numpy as np
    import torch

    import benchmark_spmv_using_csr_gb300 as sp
    import oracle
    from benchmark_spmv_using_csr_gb300 import batch, gen, tune
    mats = gen.batch_workload(512)
    nnz = sum(a.nnz for a in mats)
    mats_m, mats_n = sum(a.m for a in mats), sum(a.n for a in mats)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")

    def timed(fn, reps):
        for _ in range(3):
            fn()
        evs = []
        for i in range(reps):
            flush.fill_(i & 0xFF)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            evs.append((e0, e1))
        torch.cuda.synchronize()
        return statistics.median(p.elapsed_time(q) for p, q in evs)

    plans = []
    for a in mats:
        rp, ci = torch.from_numpy(a.row_ptr).cuda(), torch.from_numpy(a.col).cuda()
        v = torch.from_numpy(a.val).cuda()
        xx = torch.from_numpy(gen.uniform(a.n, 1)).cuda()
        yy = torch.zeros(a.m, dtype=torch.float64, device="cuda")
        plans.append((sp.Plan(sp.VALUE_F64, a.m, a.n, rp, ci), rp, ci, v, xx, yy))

    def plain_all():
        for p, _, _, v, xx, yy in plans:
            p.execute(v, xx, yy)
    ms_plain = timed(plain_all, 5)
    out = {"matrices": len(mats), "nnz": nnz, "rows": sum(a.m for a in mats),
           "plain_fp64_sequential": {"ms_per_rhs": round(ms_plain, 4),
                                     "gnnz_per_s": round(nnz / ms_plain / 1e6, 2),
                                     "launches_per_rhs": 2 * len(mats)}}
    for p in plans:
        p[0].close()
    del plans
    torch.cuda.empty_cache()
    # the plain FP64 form on the concatenated matrix: the same non-zeros in one SpMV
    cat = batch.concatenate(mats)
    rp, ci = torch.from_numpy(cat["row_ptr"]).cuda(), torch.from_numpy(cat["col"]).cuda()
    v64 = torch.from_numpy(cat["val"]).cuda()
    x64 = torch.from_numpy(gen.uniform(cat["n"], 1)).cuda()
    y64 = torch.zeros(cat["m"], dtype=torch.float64, device="cuda")
    tab, best = tune.autotune(sp.VALUE_F64, rp, ci, v64, x64, y64, warmup=1, reps=5)
    cfg = tune.candidates()[best]
    pc = sp.Plan(sp.VALUE_F64, cat["m"], cat["n"], rp, ci, seg=cfg[0], tiles_per_worker=cfg[1],
                 warps_per_cta=cfg[2], stages=cfg[3])
    ms_cat = timed(lambda: pc.execute(v64, x64, y64), 10)
    pc.check()
    out["plain_fp64_concatenated"] = {"ms_per_rhs": round(ms_cat, 4),
                                      "gnnz_per_s": round(nnz / ms_cat / 1e6, 2),
                                      "schedule": list(cfg), "launches_per_rhs": pc.launches}
    pc.close()
    del rp, ci, v64, x64, y64, cat
    torch.cuda.empty_cache()
    for k in (1, 2, 4, 8):
        xh = gen.uniform(mats_n * k, 3).reshape(mats_n, k).astype(np.float32)
        xd = torch.from_numpy(xh).cuda()
        yd = torch.zeros((mats_m, k), dtype=torch.float32, device="cuda")
        # the batched autotuner's pick for this k (its table, and the default schedule's time)
        b, tb = batch.tuned(mats, k, xd, yd, reps=5)
        dflt = ",".join(map(str, (32 if k == 4 else 16, 4, 4)))
        ms = timed(lambda: b.execute(xd, yd, use_graph=True), 10)
        b.check()
        ys, no = b.split(yd.cpu().numpy()), b.cat["n_off"]
        worst = 0.0
        for i in range(0, len(mats), 23):
            a = mats[i]
            for j in range(k):
                ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, xh[no[i]:no[i + 1], j].astype(np.float64))
                if np.linalg.norm(ystar) > 0:
                    worst = max(worst, oracle.normwise_error(ys[i][:, j], ystar))
        gk = nnz * k / ms / 1e6
        info = b.info()
        out[f"k{k}"] = {"ms": round(ms, 4), "gnnz_k_per_s": round(gk, 2),
                        "vs_plain_fp64_sequential": round(ms_plain * k / ms, 2),
                        "vs_plain_fp64_concatenated": round(ms_cat * k / ms, 2),
                        "normwise_err_vs_fp64_oracle_max": worst, "launches": info["launches"],
                        "graph": True, "schedule": tb["pick"],
                        "variant": {"one_head": info["one_head"], "x_l2_only": info["x_l2_only"]},
                        "default_schedule_ms": tb["table_ms"][dflt],
                        "tuning_table_ms": tb["table_ms"]}
        b.close()
        del xd, yd
        torch.cuda.empty_cache()
    return out


def cpu_baseline(a, x, B, seconds: float) -> dict:
    """The reference's serial CSR loop (spmv_cuda/main.cu:755-761) on one host core, whole-
    matrix passes until `seconds` have elapsed: the reference's own loop compiled from its source
    (oracle/_ref, kind "reference") where it was built, else the oracle's C port (kind "port")."""
    import numpy as np
    import oracle
    ref = oracle.ref_lib() is not None
    y = np.zeros(max(a.m, 1))
    passes = 0
    t0 = time.perf_counter()
    while True:
        if ref:
            oracle.ref_serial(a.row_ptr, a.col, a.val, x, y=y)
        else:
            oracle.csr_serial_rows(a.row_ptr, a.col, a.val, x, y, 0, a.m)
        passes += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    what = ("the reference's own loop compiled from its source in oracle/_ref" if ref
            else "C port in oracle/")
    return {"value": round(B * passes / el / 1e9, 3), "unit": UNIT, "cores": 1,
            "kind": "reference" if ref else "port",
            "sample": f"{passes} whole-matrix passes of the serial CSR loop (spmv_cuda/main.cu:"
                      f"755-761, {what}) in {el:.1f} s on one host core"}


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--workload", choices=tuple(WORKLOAD_TEXT), default="powerlaw_4m")
    ap.add_argument("--config", type=int, nargs=4, default=None,
                    metavar=("NNZ_PER_LANE", "TILES_PER_WORKER", "WARPS_PER_CTA", "STAGES"),
                    help="tile schedule (default: the autotuner's pick on this matrix)")
    ap.add_argument("--soak", type=float, default=1.5, help="seconds of untimed steps for clocks")
    ap.add_argument("--no-tune-table", dest="tune_table", action="store_false",
                    help="skip the autotuner's table of the headline matrix (it is only reported)")
    ap.add_argument("--cpu-baseline", type=float, default=10.0,
                    help="seconds of serial CPU baseline (0 = skip)")
    ap.add_argument("--no-forms", dest="forms", action="store_false")
    ap.add_argument("--no-batched", dest="batched", action="store_false",
                    help="skip the batched multi-RHS measurement")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
