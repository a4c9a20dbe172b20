"""Matrix Market coordinate files as CSR, through the library's native loader
(include/spmv_mtx.h; the loader of spmv_cuda/main.cu:570-733).

``load`` returns the same :class:`~benchmark_spmv_using_csr_gb300.gen.CSR` the generators do,
so a real matrix runs behind the same API.  ``reference_values`` gives the reference driver's
value convention (integers 0..9 for val and x, spmv_cuda/main.cu:735-743), seeded.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import gen
from ._lib import lib

STATUS = {
    -1: "cannot open the file",
    -2: "could not process the Matrix Market banner",
    -3: "complex matrices are not supported",
    -4: "could not read the size line",
    -5: "array (dense) storage is not supported",
    -6: "an entry is missing, unparsable or out of range",
    -7: "more than 2^31-1 non-zeros after mirroring",
    -8: "out of host memory",
}
FIELDS = ("real", "integer", "pattern")
SYMMETRIES = ("general", "symmetric", "hermitian", "skew-symmetric")


class MtxError(ValueError):
    def __init__(self, status: int, path: str):
        super().__init__(f"{path}: {STATUS.get(status, 'error')} (status {status})")
        self.status = status


class _Info(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int) for k in ("m", "n", "nnz_file", "nnz", "field", "symmetry")]


def load(path: str) -> gen.CSR:
    """Load a coordinate file (real, integer or pattern; general, symmetric, hermitian or
    skew-symmetric) into a CSR; raises MtxError with the loader's status on failure."""
    L = lib()
    h = ctypes.c_void_p()
    rc = L.bhsp_mtx_load(str(path).encode(), ctypes.byref(h))
    if rc != 0:
        raise MtxError(rc, str(path))
    try:
        info = _Info()
        L.bhsp_mtx_get_info(h, ctypes.byref(info))
        m, nnz = info.m, info.nnz

        def arr(ptr, count, ctype, dtype):
            if count == 0 or not ptr:
                return np.zeros(count, dtype)
            return np.ctypeslib.as_array((ctype * count).from_address(ptr)).astype(dtype, copy=True)

        rp = arr(L.bhsp_mtx_row_ptr(h), m + 1, ctypes.c_int, np.int32)
        col = arr(L.bhsp_mtx_col_idx(h), nnz, ctypes.c_int, np.int32)
        val = arr(L.bhsp_mtx_val(h), nnz, ctypes.c_double, np.float64)
        a = gen.CSR(m, info.n, rp, col, val, str(path))
        a.field = FIELDS[info.field]
        a.symmetry = SYMMETRIES[info.symmetry]
        a.nnz_file = info.nnz_file
        return a
    finally:
        L.bhsp_mtx_free(h)


def reference_values(a: gen.CSR, seed: int = 1) -> tuple[np.ndarray, np.ndarray]:
    """(val, x) in the reference driver's convention: integers in [0, 10) for every value and
    every x entry (spmv_cuda/main.cu:735-743), drawn from a seed instead of the clock."""
    return gen.uniform_int(a.nnz, seed, 10), gen.uniform_int(a.n, seed + 1, 10)
