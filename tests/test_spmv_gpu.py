"""GPU parity of y = A.x through the C ABI (handle API = the reference's class, plan API =
device buffers) against the oracle.

Tolerances (stated here, componentwise relative to (|A|.|x|)_i against the FP64 compensated
oracle y*): FP64 <= 1e-12, FP32 <= 1e-5; integer-valued data bit-exact against the serial
loop (the reference's own check, spmv_cuda/main.cu:789-806); mixed forms <= 1e-6 normwise.
"""
import numpy as np
import pytest

import oracle
from conftest import TOL_F32, TOL_F64, TOL_MIXED_NORMWISE

import benchmark_spmv_using_csr_gb300 as sp
from benchmark_spmv_using_csr_gb300 import gen

pytestmark = pytest.mark.gpu

# (non-zeros per lane, tiles per worker, warps per CTA, stages): direct loads (0 stages) and
# the TMA-staged ring (2, 3 or 4 stages)
CONFIGS = [(8, 1, 4, 0), (8, 3, 8, 0), (16, 1, 8, 0), (16, 5, 4, 0), (32, 1, 4, 0), (32, 9, 4, 0),
           (8, 1, 4, 2), (8, 7, 8, 3), (16, 2, 4, 3), (16, 4, 8, 2), (32, 3, 4, 2), (32, 1, 4, 3),
           (8, 5, 4, 4), (16, 3, 4, 4)]


def run_handle(vt, rp, col, val, x, cfg=None, y0=None, repeat=1):
    m = rp.size - 1
    n = x.size
    dt = sp.host_dtype(vt)
    s = sp.BhsparseSpmvCuda(vt)
    if cfg is not None:
        assert s.set_config(*cfg) == 0
    assert s.init_platform() == 0, s.last_error
    y = np.zeros(max(m, 1), dt) if y0 is None else np.ascontiguousarray(y0, dt)
    rc = s.prepare_mem(m, n, int(rp[-1]), rp, col, val.astype(dt), x.astype(dt), y)
    assert rc == 0, s.last_error
    for _ in range(repeat):
        assert s.run_benchmark() == 0, s.last_error
    assert s.get_y() == 0, s.last_error
    assert s.free_mem() == 0
    s.close()
    return y[:m].copy()


def int_csr(rng, m=None, n=None, maxlen=None, empty=None):
    m = int(rng.integers(1, 6000)) if m is None else m
    maxlen = int(rng.choice([3, 12, 60, 400, 2500])) if maxlen is None else maxlen
    lens = rng.integers(0, maxlen, m)
    e = rng.choice([0.0, 0.05, 0.4]) if empty is None else empty
    lens[rng.random(m) < e] = 0
    rp = np.zeros(m + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    n = int(rng.integers(1, 7000)) if n is None else n
    col = np.concatenate([np.sort(rng.choice(n, min(int(l), n), replace=False)) for l in lens]
                         ).astype(np.int32) if rp[-1] else np.zeros(0, np.int32)
    rp[1:] = np.cumsum(np.minimum(lens, n))
    val = rng.integers(-9, 10, int(rp[-1])).astype(np.float64)
    x = rng.integers(-9, 10, n).astype(np.float64)
    return rp, col, val, x


MIXED_CONFIGS = [(16, 4, 4, 0), (8, 3, 8, 2), (16, 2, 4, 3), (32, 1, 4, 2)]


@pytest.mark.parametrize("cfg", MIXED_CONFIGS)
def test_mixed_forms_configs(cuda_ok, cfg):
    rng = np.random.default_rng(77)
    a, x = _real_case(rng, "powerlaw")
    ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, x)
    y = run_handle(sp.VALUE_MIXED_F32, a.row_ptr, a.col, a.val, x, cfg)
    assert oracle.normwise_error(y, ystar) <= TOL_MIXED_NORMWISE
    yb = run_handle(sp.VALUE_MIXED_BF16, a.row_ptr, a.col, a.val, x, cfg)
    ystar_b = oracle.csr_dot2(a.row_ptr, a.col, bf16_round(a.val),
                              x.astype(np.float32).astype(np.float64))
    assert oracle.normwise_error(yb, ystar_b) <= TOL_MIXED_NORMWISE


def test_known_6x6_all_forms(cuda_ok):
    rp = np.array([0, 3, 9, 11, 11, 12, 15], np.int32)
    col = np.array([0, 2, 5, 0, 1, 2, 3, 4, 5, 2, 4, 4, 2, 3, 4], np.int32)
    val = np.arange(1, 16, dtype=np.float64)
    x = np.ones(6)
    for vt in (sp.VALUE_F64, sp.VALUE_F32, sp.VALUE_MIXED_F32, sp.VALUE_MIXED_BF16):
        for cfg in CONFIGS[:3]:
            y = run_handle(vt, rp, col, val, x, cfg)
            assert y.astype(np.float64).tolist() == [6, 39, 21, 0, 12, 42], (vt, cfg)


@pytest.mark.parametrize("vt", [sp.VALUE_F64, sp.VALUE_F32])
def test_golden_cases_bit_exact(cuda_ok, golden_cases, vt):
    d, names = golden_cases
    for name in names:
        rp, col, val, x = (d[f"{name}.{k}"] for k in ("row_ptr", "col", "val", "x"))
        for cfg in CONFIGS:
            y = run_handle(vt, rp, col, val, x, cfg)
            assert np.array_equal(y.astype(np.float64), d[f"{name}.y"]), (name, cfg)


@pytest.mark.parametrize("vt", [sp.VALUE_F64, sp.VALUE_F32])
def test_random_integer_matrices_bit_exact(cuda_ok, vt):
    rng = np.random.default_rng(99 + vt)
    for i in range(40):
        rp, col, val, x = int_csr(rng)
        yr = oracle.csr_serial(rp, col, val, x)
        cfg = CONFIGS[i % len(CONFIGS)]
        y = run_handle(vt, rp, col, val, x, cfg)
        assert np.array_equal(y.astype(np.float64), yr), (i, cfg)


def test_y_contents_and_repeated_calls(cuda_ok):
    """Unlike the reference (which needs y zeroed, bhsparse_spmv_cuda.h:170-173), the result
    is independent of y's previous contents and stable across calls."""
    rng = np.random.default_rng(5)
    rp, col, val, x = int_csr(rng, m=5000, maxlen=80, empty=0.1)
    yr = oracle.csr_serial(rp, col, val, x)
    y = run_handle(sp.VALUE_F64, rp, col, val, x, (8, 1, 4, 2), y0=np.full(5000, 7.5), repeat=5)
    assert np.array_equal(y, yr)


def _real_case(rng, kind):
    if kind == "powerlaw":
        a = gen.powerlaw(30000, seed=int(rng.integers(1 << 30)))
    elif kind == "stencil27":
        a = gen.stencil3d(24, 20, 17, seed=int(rng.integers(1 << 30)))
    elif kind == "stencil5":
        a = gen.stencil2d(97, 131, seed=int(rng.integers(1 << 30)))
    elif kind == "dense_row":
        a = gen.mixed_rows(20000, 30000, dense_row=777, mean_len=5, empty_frac=0.2,
                           seed=int(rng.integers(1 << 30)))
    elif kind == "empty90":
        a = gen.mixed_rows(50000, 20000, mean_len=12, empty_frac=0.9, seed=int(rng.integers(1 << 30)))
    else:
        a = gen.blockdiag(9000, 9000, 32)
    x = gen.uniform(a.n, int(rng.integers(1 << 30)))
    return a, x


KINDS = ["powerlaw", "stencil27", "stencil5", "dense_row", "empty90", "blockdiag"]


@pytest.mark.parametrize("kind", KINDS)
def test_real_valued_fp64_tolerance(cuda_ok, kind):
    rng = np.random.default_rng(KINDS.index(kind))
    a, x = _real_case(rng, kind)
    ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, x)
    scale = oracle.csr_absrow(a.row_ptr, a.col, a.val, x)
    for cfg in CONFIGS[::2]:
        y = run_handle(sp.VALUE_F64, a.row_ptr, a.col, a.val, x, cfg)
        assert oracle.componentwise_error(y, ystar, scale) <= TOL_F64, cfg


@pytest.mark.parametrize("kind", KINDS)
def test_real_valued_fp32_tolerance(cuda_ok, kind):
    rng = np.random.default_rng(100 + KINDS.index(kind))
    a, x = _real_case(rng, kind)
    v32, x32 = a.val.astype(np.float32), x.astype(np.float32)
    ystar = oracle.csr_dot2(a.row_ptr, a.col, v32.astype(np.float64), x32.astype(np.float64))
    scale = oracle.csr_absrow(a.row_ptr, a.col, v32.astype(np.float64), x32.astype(np.float64))
    for cfg in CONFIGS[1::2]:
        y = run_handle(sp.VALUE_F32, a.row_ptr, a.col, v32, x32, cfg)
        assert oracle.componentwise_error(y, ystar, scale) <= TOL_F32, cfg


def bf16_round(v):
    m, e = np.frexp(np.asarray(v, np.float64))
    return np.ldexp(np.round(m * 256.0), e - 8)


@pytest.mark.parametrize("kind", KINDS)
def test_mixed_forms_normwise(cuda_ok, kind):
    rng = np.random.default_rng(200 + KINDS.index(kind))
    a, x = _real_case(rng, kind)
    ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, x)
    y = run_handle(sp.VALUE_MIXED_F32, a.row_ptr, a.col, a.val, x, (16, 4, 4, 0))
    assert oracle.normwise_error(y, ystar) <= TOL_MIXED_NORMWISE
    # BF16 storage: the arithmetic is judged against y* of the BF16-rounded values and FP32 x
    yb = run_handle(sp.VALUE_MIXED_BF16, a.row_ptr, a.col, a.val, x, (16, 4, 4, 3))
    ystar_b = oracle.csr_dot2(a.row_ptr, a.col, bf16_round(a.val),
                              x.astype(np.float32).astype(np.float64))
    assert oracle.normwise_error(yb, ystar_b) <= TOL_MIXED_NORMWISE


def test_edge_shapes(cuda_ok):
    cases = []
    cases.append((np.zeros(5, np.int32), np.zeros(0, np.int32), np.zeros(0), np.ones(3)))  # m=4, nnz=0
    cases.append((np.array([0, 1], np.int32), np.array([0], np.int32), np.array([3.0]), np.array([2.0])))
    rp = np.array([0, 0, 0, 2000, 2000], np.int32)
    cases.append((rp, np.arange(2000, dtype=np.int32), np.ones(2000), np.ones(2000)))
    for rp, col, val, x in cases:
        yr = oracle.csr_serial(rp, col, val, x)
        for vt in (sp.VALUE_F64, sp.VALUE_F32):
            for cfg in CONFIGS:
                y = run_handle(vt, rp, col, val, x, cfg, y0=np.full(rp.size - 1, 3.0))
                assert np.array_equal(y.astype(np.float64), yr), (rp.size, vt, cfg)


def test_invalid_csr_is_rejected(cuda_ok):
    s = sp.BhsparseSpmvCuda(sp.VALUE_F64)
    y = np.zeros(2)
    rc = s.prepare_mem(2, 2, 2, np.array([0, 1, 2], np.int32), np.array([0, 5], np.int32),
                       np.ones(2), np.ones(2), y)
    assert rc == sp.BHSPARSE_INVALID_CSR
    rc = s.prepare_mem(2, 2, 2, np.array([0, 2, 1], np.int32), np.array([0, 1], np.int32),
                       np.ones(2), np.ones(2), y)
    assert rc == sp.BHSPARSE_INVALID_CSR
    assert s.run_benchmark() == sp.BHSPARSE_NOT_PREPARED
    s.close()


def test_plan_api_on_torch_tensors(cuda_ok):
    import torch
    rng = np.random.default_rng(17)
    a = gen.powerlaw(50000, seed=5)
    x = gen.uniform(a.n, 6)
    rp, ci = torch.from_numpy(a.row_ptr).cuda(), torch.from_numpy(a.col).cuda()
    val, xd = torch.from_numpy(a.val).cuda(), torch.from_numpy(x).cuda()
    y = torch.full((a.m,), float("nan"), dtype=torch.float64, device="cuda")
    p = sp.Plan(sp.VALUE_F64, a.m, a.n, rp, ci)
    assert p.launches == 2
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        p.execute(val, xd, y)
        p.check()
    ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, x)
    scale = oracle.csr_absrow(a.row_ptr, a.col, a.val, x)
    assert oracle.componentwise_error(y.cpu().numpy(), ystar, scale) <= TOL_F64
    del rng


def _long_rows_with_short(rng, m, n, long_len=27, short_every=100, empty_every=211):
    """Integer CSR: rows of long_len non-zeros, every short_every-th row 1..7 long (two row
    heads in one lane's chunk), every empty_every-th row empty (dirty tiles)."""
    lens = np.full(m, long_len)
    lens[::short_every] = rng.integers(1, 8, lens[::short_every].size)
    lens[5::empty_every] = 0
    rp = np.zeros(m + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    col = np.concatenate([np.sort(rng.choice(n, int(l), replace=False)) for l in lens]
                         ).astype(np.int32)
    val = rng.integers(-9, 10, int(rp[-1])).astype(np.float64)
    x = rng.integers(-9, 10, n).astype(np.float64)
    return rp, col, val, x


def _chunk_form(rp, col, vt, seg):
    import torch
    p = sp.Plan(vt, rp.size - 1, int(col.max()) + 1 if col.size else 1,
                torch.from_numpy(rp).cuda(), torch.from_numpy(col).cuda(), seg=seg)
    try:
        return p.chunk_form()
    finally:
        p.close()


@pytest.mark.parametrize("seg", [8, 16, 32])
def test_one_head_chunk_form_decision(cuda_ok, seg):
    """The plan counts the non-empty rows shorter than a chunk (4 slots at seg 8, else 8) and
    takes the one-head form when they can break at most 1/4 of the warp-chunks."""
    rng = np.random.default_rng(5)
    cw = 4 if seg == 8 else 8
    for a, expect in ((gen.stencil3d(24, 20, 17, seed=3), True), (gen.powerlaw(30000, seed=4), False)):
        lens = np.diff(a.row_ptr)
        short = int(np.count_nonzero((lens > 0) & (lens < cw)))
        got_short, on = _chunk_form(a.row_ptr, a.col, sp.VALUE_F64, seg)
        assert got_short == short
        chunks = -(-int(a.row_ptr[-1]) // (32 * cw))
        assert on == (4 * short <= chunks) == expect
    rp, col, _, _ = _long_rows_with_short(rng, 20000, 30000)
    lens = np.diff(rp)
    got_short, on = _chunk_form(rp, col, sp.VALUE_F64, seg)
    assert got_short == int(np.count_nonzero((lens > 0) & (lens < cw))) and on


def _x_locality(rp, col):
    """numpy restatement of the plan's sample: every max(1, nnz // 2^20)-th non-zero, near when
    its column is within 4 of the previous entry of its row or of the same-position entry of
    the previous row."""
    nnz = int(rp[-1])
    step = nnz // (1 << 20) if nnz > (1 << 20) else 1
    j = np.arange(0, nnz, step, dtype=np.int64)
    r = np.searchsorted(rp.astype(np.int64), j, side="right") - 1
    start = rp[r].astype(np.int64)
    c = col[j].astype(np.int64)
    near = np.zeros(j.size, bool)
    inrow = j > start
    near[inrow] = np.abs(c[inrow] - col[j[inrow] - 1]) <= 4
    ok = (~near) & (r > 0)
    ps = np.where(ok, rp[np.maximum(r - 1, 0)], 0).astype(np.int64)
    ok &= ps + (j - start) < start
    near[ok] = np.abs(c[ok] - col[ps[ok] + (j[ok] - start[ok])]) <= 4
    return j.size, int(near.sum())


def test_gather_path_decision(cuda_ok):
    """The plan samples the columns' locality and gathers x from L2 only (ld.global.cg) when
    fewer than half of the sampled non-zeros have a near column: off for stencils and block
    matrices, on for random columns."""
    import torch
    cases = ((gen.stencil3d(24, 20, 17, seed=3), False), (gen.stencil2d(97, 131, seed=2), False),
             (gen.blockdiag(9000, 9000, 32), False), (gen.powerlaw(30000, seed=4), True),
             (gen.density(20000, 20000, 1e-3, seed=6), True))
    for a, l2 in cases:
        p = sp.Plan(sp.VALUE_F64, a.m, a.n, torch.from_numpy(a.row_ptr).cuda(),
                    torch.from_numpy(a.col).cuda())
        sampled, near, got = p.gather_path()
        p.close()
        assert (sampled, near) == _x_locality(a.row_ptr, a.col)
        assert got == (2 * near < sampled) == l2


@pytest.mark.parametrize("cfg", CONFIGS)
def test_one_head_form_with_fallback_chunks_bit_exact(cuda_ok, cfg):
    """Long rows with sparse short and empty rows: most chunks take the one-head form, the
    chunks where a short row puts two heads into one lane take the per-slot loop, in the
    same launch.  Integer data: bit-exact against the serial loop."""
    rng = np.random.default_rng(cfg[0] * 100 + cfg[1] * 10 + cfg[3])
    rp, col, val, x = _long_rows_with_short(rng, 20000, 30000)
    assert _chunk_form(rp, col, sp.VALUE_F64, cfg[0])[1]
    yr = oracle.csr_serial(rp, col, val, x)
    for vt in (sp.VALUE_F64, sp.VALUE_F32):
        y = run_handle(vt, rp, col, val, x, cfg)
        assert np.array_equal(y, yr.astype(sp.host_dtype(vt)))
    ystar = oracle.csr_dot2(rp, col, val, x)
    for vt in (sp.VALUE_MIXED_F32, sp.VALUE_MIXED_BF16):
        y = run_handle(vt, rp, col, val, x, cfg)
        assert oracle.normwise_error(y, ystar) <= TOL_MIXED_NORMWISE


@pytest.mark.parametrize("cfg", [(8, 3, 4, 0), (16, 4, 4, 0), (32, 4, 4, 0), (32, 2, 8, 0),
                                 (16, 2, 4, 2), (32, 1, 4, 3)])
@pytest.mark.parametrize("long_rows", [True, False])
def test_inf_and_nan_propagate_like_the_serial_loop(cuda_ok, cfg, long_rows):
    """Inf and NaN in x and in the values reach exactly the rows of the serial loop
    (spmv_cuda/main.cu:755-761): a row is NaN where the loop's is NaN, +-Inf where it is, and
    every finite row is bit-exact (integer data).  Long rows take the one-head chunk form,
    short ones the per-slot loop."""
    rng = np.random.default_rng(cfg[0] * 10 + cfg[3] + (100 if long_rows else 0))
    if long_rows:
        rp, col, val, x = _long_rows_with_short(rng, 12000, 20000)
    else:
        rp, col, val, x = int_csr(rng, m=12000, n=20000, maxlen=12, empty=0.05)
    x[rng.choice(x.size, 6, replace=False)] = [np.inf, -np.inf, np.nan, np.inf, -np.inf, np.nan]
    val[rng.choice(val.size, 4, replace=False)] = [np.inf, -np.inf, np.nan, np.inf]
    yr = oracle.csr_serial(rp, col, val, x)
    assert np.isnan(yr).any() and np.isinf(yr).any()
    for vt in (sp.VALUE_F64, sp.VALUE_F32):
        y = run_handle(vt, rp, col, val, x, cfg).astype(np.float64)
        assert np.array_equal(np.isnan(y), np.isnan(yr))
        assert np.array_equal(np.isposinf(y), np.isposinf(yr))
        assert np.array_equal(np.isneginf(y), np.isneginf(yr))
        fin = np.isfinite(yr)
        assert np.array_equal(y[fin], yr[fin].astype(sp.host_dtype(vt)))
    # compensated accumulation turns an infinite row into NaN (TwoSum's error term of an
    # infinite sum is inf - inf); the finite rows stay finite and the others do not
    for vt in (sp.VALUE_MIXED_F32, sp.VALUE_MIXED_BF16):
        y = run_handle(vt, rp, col, val, x, cfg).astype(np.float64)
        assert np.array_equal(np.isfinite(y), np.isfinite(yr))


def test_set_x_reuses_the_matrix(cuda_ok):
    a = gen.stencil2d(64, 64)
    x1, x2 = gen.uniform(a.n, 1), gen.uniform(a.n, 2)
    s = sp.BhsparseSpmvCuda(sp.VALUE_F64)
    y = np.zeros(a.m)
    assert s.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val, x1, y) == 0
    for xx in (x2, x1, x2):
        assert s.set_x(xx) == 0
        assert s.run_benchmark() == 0 and s.get_y() == 0
        scale = oracle.csr_absrow(a.row_ptr, a.col, a.val, xx)
        assert oracle.componentwise_error(y, oracle.csr_dot2(a.row_ptr, a.col, a.val, xx), scale) <= TOL_F64
    s.close()
