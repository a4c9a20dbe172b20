"""GPU parity of the partition (tile_ptr + dirty bits) and of the bit-flag words against the
oracle, bit for bit, at the reference geometry (32 x SEG_H, SEG_H = 4 for FP64 and 8 for
FP32, spmv_cuda/common.h:39-46) and at the tuned geometries, through the C ABI."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

SEGS = (4, 8, 16, 32)


def _gpu_partition(rp_np, nnz, seg):
    import torch
    import benchmark_spmv_using_csr_gb300 as sp
    rp = torch.from_numpy(rp_np).cuda()
    tp = sp.partition(rp, nnz, 32 * seg)
    bf = sp.bitflags(rp, nnz, seg, tp)
    torch.cuda.synchronize()
    return (tp.cpu().numpy().view(np.uint32), bf.cpu().numpy().view(np.uint32).reshape(-1, 32))


def test_known_6x6(cuda_ok):
    import json, os
    from conftest import GOLDEN
    d = json.load(open(os.path.join(GOLDEN, "known_6x6.json")))
    rp = np.array(d["row_ptr"], np.int32)
    for seg in SEGS:
        tp, bf = _gpu_partition(rp, int(rp[-1]), seg)
        assert tp.tolist() == d[f"tile_ptr_{seg}"]
        assert bf.tolist() == d[f"bitflags_{seg}"]


def test_golden_cases(cuda_ok, golden_cases):
    d, names = golden_cases
    for name in names:
        rp = d[f"{name}.row_ptr"]
        nnz = int(rp[-1])
        for seg in SEGS:
            tp, bf = _gpu_partition(rp, nnz, seg)
            assert np.array_equal(tp, d[f"{name}.tile_ptr_{seg}"]), (name, seg)
            assert np.array_equal(bf, d[f"{name}.bitflags_{seg}"].reshape(-1, 32)), (name, seg)


def _random_rows(rng):
    m = int(rng.integers(1, 20000))
    kind = rng.integers(0, 4)
    if kind == 0:
        lens = rng.integers(0, 8, m)
    elif kind == 1:
        lens = rng.integers(0, 300, m)
    elif kind == 2:
        lens = np.where(rng.random(m) < 0.9, 0, rng.integers(1, 50, m))
    else:
        lens = rng.zipf(2.1, m).clip(1, 5000)
    lens[rng.random(m) < rng.choice([0.0, 0.05, 0.3])] = 0
    rp = np.zeros(m + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    return rp


def test_random_row_patterns(cuda_ok):
    rng = np.random.default_rng(123)
    for _ in range(60):
        rp = _random_rows(rng)
        nnz = int(rp[-1])
        for seg in SEGS:
            tp, bf = _gpu_partition(rp, nnz, seg)
            tpo = oracle.partition(rp, nnz, 32 * seg)
            assert np.array_equal(tp, tpo), seg
            assert np.array_equal(bf, oracle.bitflags(rp, nnz, 32, seg, tpo).reshape(-1, 32)), seg


def test_full_size_partition(cuda_ok):
    """Both benchmark matrices: tile_ptr bit-exact at the FP64 and FP32 reference geometries
    and at the default tuned geometry (32 x 32)."""
    import torch
    import benchmark_spmv_using_csr_gb300 as sp
    from benchmark_spmv_using_csr_gb300 import gen
    for a in (gen.powerlaw_4m(), gen.stencil27_160()):
        rp = torch.from_numpy(a.row_ptr).cuda()
        for seg in (4, 8, 32):
            tp = sp.partition(rp, a.nnz, 32 * seg).cpu().numpy().view(np.uint32)
            assert np.array_equal(tp, oracle.partition(a.row_ptr, a.nnz, 32 * seg)), (a.name, seg)


def test_validate_csr(cuda_ok):
    import torch
    import benchmark_spmv_using_csr_gb300 as sp
    rp = torch.tensor([0, 2, 3, 3], dtype=torch.int32, device="cuda")
    ci = torch.tensor([0, 2, 1], dtype=torch.int32, device="cuda")
    assert sp.validate_csr(rp, ci, 3) == sp.BHSPARSE_SUCCESS
    assert sp.validate_csr(rp, ci, 2) == sp.BHSPARSE_INVALID_CSR  # col 2 >= n
    bad = torch.tensor([0, 2, 1, 3], dtype=torch.int32, device="cuda")
    assert sp.validate_csr(bad, ci, 3) == sp.BHSPARSE_INVALID_CSR  # not monotone
    short = torch.tensor([0, 2, 3, 2], dtype=torch.int32, device="cuda")
    assert sp.validate_csr(short, ci, 3) == sp.BHSPARSE_INVALID_CSR  # row_ptr[m] != nnz
