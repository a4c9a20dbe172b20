"""bhsp_run_stream: many right-hand sides from host memory with overlapped copies, against the
per-call sequence set_x / run_benchmark / get_y and the oracle; the F64 and F32 forms."""
import numpy as np
import pytest
import torch

import oracle
from conftest import TOL_F64

import benchmark_spmv_using_csr_gb300 as sp
from benchmark_spmv_using_csr_gb300 import gen

pytestmark = pytest.mark.gpu


def _pinned(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a)).pin_memory()


@pytest.mark.parametrize("vt", [sp.VALUE_F64, sp.VALUE_F32])
@pytest.mark.parametrize("count", [1, 2, 5])
def test_stream_matches_per_call(cuda_ok, vt, count):
    a = gen.powerlaw(40000, seed=21)
    dt = sp.host_dtype(vt)
    xs = [_pinned(gen.uniform_int(a.n, 30 + i, 10).astype(dt)) for i in range(count)]
    ys = [_pinned(np.full(a.m, -1, dt)) for _ in range(count)]
    val = gen.uniform_int(a.nnz, 7, 10).astype(dt)
    h = sp.BhsparseSpmvCuda(vt)
    y0 = np.zeros(a.m, dt)
    assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, val, xs[0].numpy(), y0) == 0
    assert h.run_stream([x.data_ptr() for x in xs], [y.data_ptr() for y in ys]) == 0, h.last_error
    for i in range(count):  # integer data: exact against the serial loop
        yr = oracle.csr_serial(a.row_ptr, a.col, val.astype(np.float64),
                               xs[i].numpy().astype(np.float64))
        assert np.array_equal(ys[i].numpy().astype(np.float64), yr), i
    # the per-call path on the same handle still works afterwards
    assert h.set_x(xs[-1].numpy()) == 0 and h.run_benchmark() == 0 and h.get_y() == 0
    assert np.array_equal(y0, ys[-1].numpy())
    h.close()


def test_stream_real_values_and_reuse(cuda_ok):
    a = gen.stencil3d(40, 30, 20, seed=4)
    xs = [_pinned(gen.uniform(a.n, 50 + i)) for i in range(6)]
    ys = [_pinned(np.zeros(a.m)) for _ in range(6)]
    h = sp.BhsparseSpmvCuda(sp.VALUE_F64)
    assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val, xs[0].numpy(),
                         np.zeros(a.m)) == 0
    for _ in range(2):  # a second stream call reuses the buffers and streams
        assert h.run_stream([x.data_ptr() for x in xs], [y.data_ptr() for y in ys]) == 0
        for x, y in zip(xs, ys):
            ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, x.numpy())
            scale = oracle.csr_absrow(a.row_ptr, a.col, a.val, x.numpy())
            assert oracle.componentwise_error(y.numpy(), ystar, scale) <= TOL_F64
    assert h.run_stream([], []) == 0
    h.close()


def test_stream_rejects_mixed_and_nulls(cuda_ok):
    a = gen.stencil2d(20, 20)
    h = sp.BhsparseSpmvCuda(sp.VALUE_MIXED_F32)
    assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val, np.ones(a.n),
                         np.zeros(a.m)) == 0
    x = _pinned(np.ones(a.n))
    y = _pinned(np.zeros(a.m))
    assert h.run_stream([x.data_ptr()], [y.data_ptr()]) == sp.BHSPARSE_INVALID_ARGUMENT
    h.close()
    h = sp.BhsparseSpmvCuda(sp.VALUE_F64)
    assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val, np.ones(a.n),
                         np.zeros(a.m)) == 0
    assert h.run_stream([0], [y.data_ptr()]) == sp.BHSPARSE_INVALID_ARGUMENT
    h.close()


def test_run_benchmark_after_stream_keeps_prepared_x(cuda_ok):
    """run_stream works in buffers of its own: the x given to prepare_mem (or the last set_x)
    is still the one run_benchmark uses afterwards, and y on the device is not overwritten."""
    a = gen.powerlaw(30000, seed=5)
    val = gen.uniform_int(a.nnz, 8, 10)
    x0 = gen.uniform_int(a.n, 9, 10)
    y_ref = oracle.csr_serial(a.row_ptr, a.col, val, x0)
    h = sp.BhsparseSpmvCuda(sp.VALUE_F64)
    y = np.zeros(a.m)
    assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, val, x0, y) == 0
    assert h.run_benchmark() == 0
    xs = [_pinned(gen.uniform_int(a.n, 60 + i, 10)) for i in range(3)]
    ys = [_pinned(np.zeros(a.m)) for _ in range(3)]
    assert h.run_stream([v.data_ptr() for v in xs], [v.data_ptr() for v in ys]) == 0
    assert h.get_y() == 0  # the y of the run_benchmark before the stream
    assert np.array_equal(y, y_ref)
    y[:] = -1.0
    assert h.run_benchmark() == 0 and h.get_y() == 0
    assert np.array_equal(y, y_ref)
    h.close()


def test_handle_copies_pageable_and_unaligned_host_arrays(cuda_ok):
    """prepare_mem / set_x / get_y copy pageable host arrays with a kernel where the device
    reads pageable memory, and fall back to cudaMemcpy for buffers that are not 16-byte aligned;
    either way y is exact on integer data, set_x takes effect, and the caller may overwrite x
    as soon as set_x returns."""
    a = gen.powerlaw(50_000, seed=31)
    val = gen.uniform_int(a.nnz, 32, 10)
    for offset in (0, 1):  # 16-byte aligned arrays, then views 8 bytes off
        def arr(v):
            buf = np.zeros(v.size + 2)
            out = buf[offset:offset + v.size]
            out[:] = v
            return out
        x1, x2 = arr(gen.uniform_int(a.n, 33, 10)), arr(gen.uniform_int(a.n, 34, 10))
        y = arr(np.full(a.m, -1.0))
        h = sp.BhsparseSpmvCuda(sp.VALUE_F64)
        assert h.set_config(16, 4, 4, 0) == 0
        assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, val, x1, y) == 0
        assert h.run_benchmark() == 0 and h.get_y() == 0
        assert np.array_equal(y, oracle.csr_serial(a.row_ptr, a.col, val, x1)), offset
        assert h.set_x(x2) == 0
        x2[:] = -7.0  # already read by set_x
        assert h.run_benchmark() == 0 and h.get_y() == 0
        assert np.array_equal(y, oracle.csr_serial(a.row_ptr, a.col, val,
                                                   gen.uniform_int(a.n, 34, 10))), offset
        h.close()


def test_handles_in_concurrent_host_threads(cuda_ok):
    """Handles are independent: eight host threads, each with its own handle (the four value
    types, two matrices), prepare, run and read back at the same time; every y is exact."""
    import threading
    mats = [gen.powerlaw(30000, seed=41), gen.stencil3d(24, 24, 24, seed=42)]
    jobs = [(vt, i) for vt in (sp.VALUE_F64, sp.VALUE_F32, sp.VALUE_MIXED_F32,
                               sp.VALUE_MIXED_BF16) for i in range(2)]
    results, errors = {}, []

    def work(vt, i):
        try:
            a = mats[i]
            dt = sp.host_dtype(vt)
            val = (gen.uniform_int(a.nnz, 50 + i, 10) - 4.0).astype(dt)
            x = (gen.uniform_int(a.n, 60 + i, 10) - 4.0).astype(dt)
            y = np.full(a.m, np.nan, dt)
            h = sp.BhsparseSpmvCuda(vt)
            assert h.init_platform() == 0, h.last_error
            assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, val, x, y) == 0, h.last_error
            for _ in range(3):
                assert h.run_benchmark() == 0, h.last_error
            assert h.get_y() == 0, h.last_error
            h.free_mem()
            h.close()
            results[(vt, i)] = (y.astype(np.float64), val.astype(np.float64),
                                x.astype(np.float64))
        except Exception as e:  # reported on the main thread
            errors.append((vt, i, repr(e)))

    threads = [threading.Thread(target=work, args=j) for j in jobs]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for (vt, i), (y, val, x) in results.items():
        a = mats[i]
        yr = oracle.csr_serial(a.row_ptr, a.col, val, x)
        assert np.array_equal(y, yr), (vt, i)
