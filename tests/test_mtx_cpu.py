"""Matrix Market loading (include/spmv_mtx.h) against the oracle restatement of the reference
driver's loader (oracle/mtx_oracle.py; spmv_cuda/main.cu:570-733), on the committed fixtures of
tests/golden/mtx/ (written by tests/golden/make_mtx.py) and on larger seeded files.

Bit-exact: row_ptr, col_idx, val and the reported sizes; the status codes of the failure
points.  Known answers pin the restatement itself; where the reference tree was present at
build time, oracle/_ref/libmtx_ref.so runs the reference's own banner and size readers
(spmv_cuda/mmio.h:249, :334) on the same files.
"""
import ctypes
import glob
import os

import numpy as np
import pytest

from oracle import mtx_oracle

from benchmark_spmv_using_csr_gb300 import mtx

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIXTURES = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "mtx", "*.mtx")))
VALID = [f for f in FIXTURES if not os.path.basename(f).startswith("err_")]
ERRORS = {
    "err_complex.mtx": -3, "err_array.mtx": -5, "err_banner_prefix.mtx": -2,
    "err_banner_short.mtx": -2, "err_banner_field.mtx": -2, "err_no_size.mtx": -4,
    "err_index.mtx": -6, "err_zero_index.mtx": -6, "err_truncated.mtx": -6, "err_value.mtx": -6,
}


def _check_same(path):
    st, d = mtx_oracle.load(path)
    assert st == 0
    a = mtx.load(path)
    assert (a.m, a.n, a.nnz, a.nnz_file) == (d["m"], d["n"], len(d["col"]), d["nnz_file"])
    assert a.field == d["field"] and a.symmetry == d["symmetry"]
    assert np.array_equal(a.row_ptr, d["row_ptr"])
    assert np.array_equal(a.col, d["col"])
    assert np.array_equal(a.val.view(np.uint64), d["val"].view(np.uint64))
    return a


def test_fixture_set_complete():
    assert len(VALID) == 10 and len(FIXTURES) == 10 + len(ERRORS)


@pytest.mark.parametrize("path", VALID, ids=os.path.basename)
def test_valid_fixture_matches_oracle(path):
    _check_same(path)


@pytest.mark.parametrize("name,status", sorted(ERRORS.items()))
def test_failure_status(name, status):
    path = os.path.join(ROOT, "tests", "golden", "mtx", name)
    assert mtx_oracle.load(path)[0] == status
    with pytest.raises(mtx.MtxError) as e:
        mtx.load(path)
    assert e.value.status == status


def test_missing_file():
    with pytest.raises(mtx.MtxError) as e:
        mtx.load(os.path.join(ROOT, "tests", "golden", "mtx", "no_such_file.mtx"))
    assert e.value.status == -1


def _fix(name):
    return mtx.load(os.path.join(ROOT, "tests", "golden", "mtx", name))


def test_known_answers():
    a = _fix("known6_general_real.mtx")  # spmv_cuda/main.cu:449-451
    assert a.row_ptr.tolist() == [0, 3, 9, 11, 11, 12, 15]
    assert a.col.tolist() == [0, 2, 5, 0, 1, 2, 3, 4, 5, 2, 4, 4, 2, 3, 4]
    assert a.val.tolist() == list(range(1, 16))
    h = _fix("hermitian_real.mtx")  # mirrored like symmetric, placed in file order
    assert h.row_ptr.tolist() == [0, 2, 4, 6]
    assert h.col.tolist() == [0, 1, 0, 2, 1, 2]
    assert h.val.tolist() == [2.5, -1, -1, 4, 4, 1]
    s = _fix("symmetric_pattern.mtx")
    assert s.row_ptr.tolist() == [0, 2, 3, 4, 6, 9]
    assert s.col.tolist() == [0, 2, 4, 0, 3, 4, 1, 3, 4]
    assert s.val.tolist() == [1.0] * 9
    k = _fix("skew_real.mtx")  # the reference does not mirror skew-symmetric files
    assert k.row_ptr.tolist() == [0, 0, 1, 2, 3]
    assert k.col.tolist() == [0, 0, 2] and k.val.tolist() == [1.5, -2, 0.25]
    r = _fix("rect_dups.mtx")  # columns unsorted within a row, duplicates kept
    assert r.row_ptr.tolist() == [0, 2, 5, 6]
    assert r.col.tolist() == [2, 0, 4, 0, 4, 1]
    assert r.val.tolist() == [3, 6, 1, 2, 4, 5]
    e = _fix("empty.mtx")
    assert (e.m, e.n, e.nnz) == (3, 4, 0) and e.row_ptr.tolist() == [0, 0, 0, 0]


@pytest.mark.parametrize("sym", ["general", "symmetric"])
def test_large_seeded_file(tmp_path, sym):
    rng = np.random.default_rng(11 if sym == "general" else 12)
    m = n = 2000
    k = 20000
    flat = rng.choice(m * n, k, replace=False)
    r, c = flat // n, flat % n
    if sym == "symmetric":
        r, c = np.maximum(r, c), np.minimum(r, c)
        keep = np.unique(r * n + c, return_index=True)[1]
        r, c = r[keep], c[keep]
    v = rng.standard_normal(r.size)
    p = tmp_path / f"big_{sym}.mtx"
    with open(p, "w") as fh:
        fh.write(f"%%MatrixMarket matrix coordinate real {sym}\n{m} {n} {r.size}\n")
        fh.writelines(f"{a + 1} {b + 1} {x:.17g}\n" for a, b, x in zip(r, c, v))
    a = _check_same(str(p))
    if sym == "symmetric":  # the loaded matrix equals its transpose
        import scipy.sparse as sps
        A = sps.csr_matrix((a.val, a.col, a.row_ptr), shape=(m, n))
        assert (A != A.T).nnz == 0


def test_reference_values_convention():
    a = _fix("general_real_shuffled.mtx")
    val, x = mtx.reference_values(a, seed=3)
    assert val.shape == (a.nnz,) and x.shape == (a.n,)
    for v in (val, x):
        assert v.dtype == np.float64 and v.min() >= 0 and v.max() <= 9
        assert np.array_equal(v, np.floor(v))


REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libmtx_ref.so")
# the reference's type code: [2] field R/I/P/C, [3] symmetry G/S/H/K (spmv_cuda/mmio.h:36-51)
FIELD_CODE = {"real": "R", "integer": "I", "pattern": "P"}
SYM_CODE = {"general": "G", "symmetric": "S", "hermitian": "H", "skew-symmetric": "K"}


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference tree absent at build time")
@pytest.mark.parametrize("path", VALID + [os.path.join(ROOT, "tests", "golden", "mtx", n)
                                          for n in ("err_complex.mtx", "err_banner_prefix.mtx",
                                                    "err_banner_short.mtx",
                                                    "err_banner_field.mtx")],
                         ids=os.path.basename)
def test_header_against_reference_readers(path):
    L = ctypes.CDLL(REF_LIB)
    tc = ctypes.create_string_buffer(4)
    m, n, nz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    rc = L.ref_mtx_header(path.encode(), tc, ctypes.byref(m), ctypes.byref(n), ctypes.byref(nz))
    st, d = mtx_oracle.load(path)
    if st in (-2, -3):
        assert rc == st
        return
    assert rc == 0
    assert (m.value, n.value, nz.value) == (d["m"], d["n"], d["nnz_file"])
    code = tc.raw.decode()
    assert code[0] == "M" and code[1] == "C"
    assert code[2] == FIELD_CODE[d["field"]] and code[3] == SYM_CODE[d["symmetry"]]
