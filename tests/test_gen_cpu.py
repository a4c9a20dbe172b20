"""The seeded workload generators give the same matrices from both of their builds: the
package library (used by the GPU arm of bench.py and the tests) and oracle/_build/libgen.so
(used by bench.py's CPU reference arm, which must not load the GPU library)."""
import zlib

import numpy as np
import pytest

import oracle
from benchmark_spmv_using_csr_gb300 import gen


def _crc(a) -> int:
    c = 0
    for arr in (a.row_ptr, a.col, a.val):
        c = zlib.crc32(np.ascontiguousarray(arr).view(np.uint8), c)
    return c


def _make():
    return [gen.powerlaw(150_000, seed=2), gen.stencil3d(23, 19, 17, seed=3),
            gen.stencil2d(64, 64, seed=1), gen.density(20_000, 20_000, 1e-3, seed=9),
            gen.blockdiag(5_000, seed=5), gen.mixed_rows(8_000, 8_000, 17, 6.0, 0.3, seed=4)]


def test_both_generator_builds_agree():
    ours = _make()
    x_ours = gen.uniform(100_003, 7)
    try:
        gen.use_library(oracle.gen_library_path())
        theirs = _make()
        x_theirs = gen.uniform(100_003, 7)
    finally:
        gen._gen_override = None
    for a, b in zip(ours, theirs):
        assert a.m == b.m and a.n == b.n and a.nnz == b.nnz
        assert _crc(a) == _crc(b), a.name
    assert np.array_equal(x_ours, x_theirs)
