"""bench.py's multi-rank logic on CPU: world_size-2 gloo ranks agree on the slowest rank's time,
the whole-job value is the sum over replicas, and the reference arm runs and prints on rank 0
only (every other rank exits 0 without work)."""
import os
import socket
import subprocess
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(1.5 + rank, dist)
        out[rank] = (t, bench.whole_job_gbs(world, 10**9, 4, t))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    world = 2
    out = mp.get_context("spawn").Manager().dict()  # no fork of this multi-threaded process
    mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        t, gbs = out[r]
        assert t == 2.5  # the slower rank's time, on every rank
        assert gbs == pytest.approx(world * 4 / 2.5)


def test_single_process_passthrough():
    assert bench.max_over_ranks(0.25) == 0.25
    assert bench.whole_job_gbs(1, 2 * 10**9, 3, 2.0) == pytest.approx(3.0)


def test_reference_arm_nonzero_rank_is_silent():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "3"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_reference_arm_rank0_prints_one_line():
    import json
    env = dict(os.environ, RANK="0", LOCAL_RANK="0", WORLD_SIZE="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "stencil5_256", "--steps", "3", "--warmup", "3"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "GB/s" and d["value"] > 0
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "GB/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["workload"] == "stencil5_256"
