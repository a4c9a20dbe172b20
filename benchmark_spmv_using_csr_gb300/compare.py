"""Comparators timed beside the tile kernel (include/spmv_compare.h): the CSR-vector kernel of
the reference driver's CUSP comparison and cuSPARSE's generic SpMV.  Both take torch CUDA
tensors; neither is a product path."""
from __future__ import annotations

import ctypes

from ._lib import lib

UNAVAILABLE = -3


def _stream(stream) -> int:
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return int(getattr(s, "cuda_stream", s))


def vector_width(m: int, nnz: int) -> int:
    """Threads per row the reference picks from nnz / m (spmv_cuda/main.cu:236-286)."""
    return int(lib().bhsp_csr_vector_width(int(m), int(nnz)))


def csr_vector(value_type: int, row_ptr, col_idx, val, x, y, threads_per_vector: int = 0,
               stream=None) -> None:
    m = row_ptr.numel() - 1
    rc = lib().bhsp_csr_vector(int(value_type), m, row_ptr.data_ptr(), col_idx.data_ptr(),
                               val.data_ptr(), x.data_ptr(), y.data_ptr(), int(threads_per_vector),
                               ctypes.c_void_p(_stream(stream)))
    if rc != 0:
        raise RuntimeError(f"bhsp_csr_vector failed with status {rc}")


class Cusparse:
    """cusparseSpMV (CSR_ALG1) bound to fixed device tensors; raises RuntimeError with
    status -3 when the cuSPARSE library cannot be loaded."""

    def __init__(self, value_type: int, row_ptr, col_idx, val, x, y, n: int | None = None,
                 stream=None):
        self._h = ctypes.c_void_p()
        m = row_ptr.numel() - 1
        n = x.numel() if n is None else n
        self._keep = (row_ptr, col_idx, val, x, y)
        rc = lib().bhsp_cusparse_create(ctypes.byref(self._h), int(value_type), m, int(n),
                                        int(col_idx.numel()), row_ptr.data_ptr(),
                                        col_idx.data_ptr(), val.data_ptr(), x.data_ptr(),
                                        y.data_ptr(), ctypes.c_void_p(_stream(stream)))
        if rc != 0:
            self.status = rc
            raise RuntimeError(f"bhsp_cusparse_create failed with status {rc}")

    def run(self) -> None:
        rc = lib().bhsp_cusparse_run(self._h)
        if rc != 0:
            raise RuntimeError(f"bhsp_cusparse_run failed with status {rc}")

    def close(self) -> None:
        if self._h:
            lib().bhsp_cusparse_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
