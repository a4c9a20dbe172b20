"""CPU tests of the oracle: pinned against the reference's known-answer case and against an
independent pure-Python restatement (tests/golden/), then exercised on seeded integer
matrices where the reference's own exact-equality check (spmv_cuda/main.cu:789-806) applies.
"""
import json
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN


@pytest.fixture(scope="module")
def known():
    with open(os.path.join(GOLDEN, "known_6x6.json")) as f:
        return json.load(f)


def test_known_6x6_serial(known):
    rp, ci = np.array(known["row_ptr"], np.int32), np.array(known["col_idx"], np.int32)
    val, x = np.array(known["val"]), np.array(known["x"])
    y = oracle.csr_serial(rp, ci, val, x)
    assert y.tolist() == [6.0, 39.0, 21.0, 0.0, 12.0, 42.0]
    assert y.tolist() == [float(v) for v in known["y"]]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_known_6x6_reference_algorithm(known, dtype):
    """The lane-level simulation of SpMV_kernel + host calibration returns the row sums."""
    rp, ci = np.array(known["row_ptr"], np.int32), np.array(known["col_idx"], np.int32)
    r = oracle.bhsparse(rp, ci, np.array(known["val"], dtype), np.array(known["x"], dtype))
    assert r.y.astype(np.float64).tolist() == [float(v) for v in known["y"]]
    # one dirty tile (row 3 is empty) spanning rows 0..6 -- the last tile, so the host
    # fix-up would read row_ptr[m+1] (bhsparse_spmv_cuda.h:199-216): guarded and flagged
    assert r.ndirty == 1 and r.speculator.tolist() == [[0, 6]]
    assert r.oob_guarded


@pytest.mark.parametrize("seg", [4, 8, 16, 32])
def test_known_6x6_partition_and_flags(known, seg):
    rp = np.array(known["row_ptr"], np.int32)
    tp = oracle.partition(rp, int(rp[-1]), 32 * seg)
    assert tp.tolist() == known[f"tile_ptr_{seg}"]
    bf = oracle.bitflags(rp, int(rp[-1]), 32, seg, tp)
    assert bf.tolist() == known[f"bitflags_{seg}"]


def test_known_6x6_hand_derived(known):
    # derived by hand from kernels_cuda.h:116-143 with SEG_H = 4: row starts 0, 3, 9, 11, 12
    # (row 3 is empty) -> word 0 bits 31 and 28, word 2 bits 30 and 28, word 3 bit 31.
    w = known["bitflags_4"][0]
    assert w[0] == 0x90000000 and w[2] == 0x50000000 and w[3] == 0x80000000
    assert sum(1 for v in w if v) == 3
    assert known["tile_ptr_4"] == [0x80000000, 6]


def test_golden_cases(golden_cases):
    d, names = golden_cases
    for name in names:
        rp, col, val, x = (d[f"{name}.{k}"] for k in ("row_ptr", "col", "val", "x"))
        nnz = int(rp[-1])
        y = oracle.csr_serial(rp, col, val, x)
        assert np.array_equal(y, d[f"{name}.y"]), name
        for seg in (4, 8, 16, 32):
            tp = oracle.partition(rp, nnz, 32 * seg)
            assert np.array_equal(tp, d[f"{name}.tile_ptr_{seg}"]), (name, seg)
            bf = oracle.bitflags(rp, nnz, 32, seg, tp)
            assert np.array_equal(bf.reshape(-1, 32), d[f"{name}.bitflags_{seg}"].reshape(-1, 32)), (name, seg)
        for dt in (np.float64, np.float32):
            r = oracle.bhsparse(rp, col, val.astype(dt), x.astype(dt))
            assert np.array_equal(r.y.astype(np.float64), d[f"{name}.y"]), (name, dt)


def _random_int_csr(rng):
    m = int(rng.integers(1, 2500))
    lens = rng.integers(0, int(rng.choice([3, 10, 50, 400, 3000])), size=m)
    lens[rng.random(m) < rng.choice([0.0, 0.05, 0.5])] = 0
    rp = np.zeros(m + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    n = int(rng.integers(1, 5000))
    col = rng.integers(0, n, size=int(rp[-1])).astype(np.int32)
    val = rng.integers(0, 10, size=int(rp[-1])).astype(np.float64)
    x = rng.integers(0, 10, size=n).astype(np.float64)
    return rp, col, val, x


def test_reference_algorithm_matches_serial_on_integer_data():
    """main.cu:789-806 checks bhSPARSE against the serial loop by exact equality on rand()%10
    data; the restatement passes the same check on 200 seeded matrices per precision."""
    rng = np.random.default_rng(7)
    for _ in range(200):
        rp, col, val, x = _random_int_csr(rng)
        yr = oracle.csr_serial(rp, col, val, x)
        for dt in (np.float64, np.float32):
            r = oracle.bhsparse(rp, col, val.astype(dt), x.astype(dt))
            assert np.array_equal(r.y.astype(np.float64), yr)


def test_reference_algorithm_needs_zeroed_y():
    """The reference writes a warp's first row only through the host `+=` of the
    synchronizer (bhsparse_spmv_cuda.h:170-173), so a non-zero incoming y leaks into the
    result; the GPU path does not inherit this (tested in test_spmv_gpu)."""
    rng = np.random.default_rng(11)
    rp, col, val, x = _random_int_csr(rng)
    while int(rp[-1]) < 2000:
        rp, col, val, x = _random_int_csr(rng)
    yr = oracle.csr_serial(rp, col, val, x)
    r = oracle.bhsparse(rp, col, val, x, y0=np.full(rp.size - 1, 5.0))
    assert not np.array_equal(r.y, yr)


def test_partition_is_consistent_with_search():
    rng = np.random.default_rng(3)
    for _ in range(50):
        rp, col, val, x = _random_int_csr(rng)
        nnz = int(rp[-1])
        for ps in (128, 256, 1024):
            tp = oracle.partition(rp, nnz, ps)
            rows = tp & 0x7FFFFFFF
            for t in range(0, tp.size, max(1, tp.size // 7)):
                assert rows[t] == oracle.search_right(rp, min(t * ps, nnz)) - 1
            assert np.all(np.diff(rows.astype(np.int64)) >= 0)
            assert tp[-1] >> 31 == 0


def test_dot2_is_more_accurate_than_serial():
    rng = np.random.default_rng(5)
    m, n = 200, 300
    lens = rng.integers(1, 60, m)
    rp = np.zeros(m + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    col = rng.integers(0, n, int(rp[-1])).astype(np.int32)
    # ill-conditioned rows: huge cancelling terms
    val = rng.standard_normal(int(rp[-1])) * np.where(rng.random(int(rp[-1])) < 0.5, 1e8, 1.0)
    x = rng.standard_normal(n)
    from fractions import Fraction
    ystar = oracle.csr_dot2(rp, col, val, x)
    ys = oracle.csr_serial(rp, col, val, x)
    err_d, err_s = 0.0, 0.0
    for i in range(0, m, 10):
        ex = sum(Fraction(float(val[j])) * Fraction(float(x[col[j]])) for j in range(rp[i], rp[i + 1]))
        err_d = max(err_d, abs(float(Fraction(float(ystar[i])) - ex)))
        err_s = max(err_s, abs(float(Fraction(float(ys[i])) - ex)))
    assert err_d <= err_s


def test_error_metrics():
    y = np.array([1.0, 2.0, 0.0])
    ys = np.array([1.0, 2.0 + 1e-13, 0.0])
    s = np.array([1.0, 2.0, 0.0])
    assert oracle.componentwise_error(y, ys, s) == pytest.approx(5e-14, rel=1e-3)
    assert oracle.componentwise_error(np.array([0.0, 0, 1.0]), np.zeros(3), s) == float("inf")
    assert oracle.normwise_error(ys, y) == pytest.approx(1e-13 / np.sqrt(5), rel=1e-3)


# -- pinned to the reference's own host code, compiled from its sources ---------------------
# oracle/_ref/libref.so is built by `make -C oracle ref` from the reference tree (build() does
# it where the tree is present); without it these tests skip.
needs_ref = pytest.mark.skipif(oracle.ref_lib() is None,
                               reason="oracle/_ref/libref.so not built (no reference tree)")


def _random_real_csr(rng, dtype):
    rp, col, _, _ = _random_int_csr(rng)
    val = rng.uniform(-1.0, 1.0, int(rp[-1])).astype(dtype)
    x = rng.uniform(-1.0, 1.0, int(col.max(initial=0)) + 1).astype(dtype)
    return rp, col, val, x


@needs_ref
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_calibration_matches_reference_code(dtype):
    """The oracle's host calibration (inter-warp += and the speculative fix-up of dirty tiles)
    gives bit for bit the y of the reference's own run_benchmark host code
    (spmv_cuda/bhsparse_spmv_cuda.h:170-222) on the same kernel output, for 300 seeded real-
    valued matrices with empty rows, dirty tiles and dirty last tiles.  Where the last tile is
    dirty the reference reads row_ptr[m+1] and writes y[m]; with one padded entry that write
    is 0 and rows 0..m-1 agree with the oracle's guarded loop."""
    rng = np.random.default_rng(101)
    dirty_cases = last_dirty = 0
    for _ in range(300):
        rp, col, val, x = _random_real_csr(rng, dtype)
        st = oracle.bhsparse_kernel(rp, col, val, x)
        y_o, oob = oracle.calibrate(rp, st)
        y_r, y_m = oracle.ref_calibrate(rp, st)
        assert np.array_equal(y_o, y_r)
        assert y_m == 0
        dirty_cases += st.ndirty > 0
        last_dirty += oob
    assert dirty_cases > 100 and last_dirty > 20


@needs_ref
def test_known_6x6_through_reference_calibration(known):
    rp, ci = np.array(known["row_ptr"], np.int32), np.array(known["col_idx"], np.int32)
    st = oracle.bhsparse_kernel(rp, ci, np.array(known["val"]), np.array(known["x"]))
    y, _ = oracle.ref_calibrate(rp, st)
    assert y.tolist() == [float(v) for v in known["y"]]


@needs_ref
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_serial_and_openmp_loops_match_reference_code(dtype):
    """The oracle's serial loop is bit-identical to the reference's own (spmv_cuda/main.cu:
    753-762), and so is the reference's OpenMP loop (main.cu:377-393) at 1, 4 and all threads:
    each row is summed in row order by one thread."""
    rng = np.random.default_rng(102)
    for _ in range(60):
        rp, col, val, x = _random_real_csr(rng, dtype)
        y_o = oracle.csr_serial(rp, col, val, x)
        assert np.array_equal(y_o, oracle.ref_serial(rp, col, val, x))
        if dtype == np.float64:
            for t in (1, 4, os.cpu_count() or 1):
                assert np.array_equal(y_o, oracle.ref_omp(rp, col, val, x, t, runs=2))
