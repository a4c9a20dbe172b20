"""Host-side mirror of the reference's ``bhsparse_spmv_cuda`` class, plus a device-buffer
plan API, over the C ABI of ``libspmv_gb300.so``.

``BhsparseSpmvCuda`` has the reference's methods with the same names, arguments and
integer status codes (spmv_cuda/bhsparse_spmv_cuda.h:7-55):

    sp = BhsparseSpmvCuda()                      # value type: VALUE_F64 (USE_DOUBLE=1)
    sp.init_platform()
    sp.prepare_mem(m, n, nnzA, row_ptr, col_idx, val, x, y)   # numpy arrays
    sp.run_benchmark()
    sp.get_y()                                   # fills the y passed to prepare_mem
    sp.free_platform(); sp.free_mem()

``Plan`` runs the same kernels on torch CUDA tensors the caller already holds.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import lib

# status codes (include/spmv_gb300.h; the first two are spmv_cuda/common.h:24-25)
BHSPARSE_SUCCESS = 0
BHSPARSE_UNSUPPORTED_VALUE_TYPE = -1
BHSPARSE_INVALID_ARGUMENT = -2
BHSPARSE_INVALID_CSR = -3
BHSPARSE_CUDA_ERROR = -4
BHSPARSE_NOT_PREPARED = -5
BHSPARSE_DEVICE_CHECK_FAILED = -6
BHSPARSE_OUT_OF_MEMORY = -7
BHSPARSE_NOALLOC_TOO_LARGE = -8

# where a schedule came from (bhsp_choose_schedule / bhsp_get_schedule_source)
SCHEDULE_CALLER, SCHEDULE_DEFAULT, SCHEDULE_LEARNED, SCHEDULE_SWEEP = 0, 1, 2, 3

VALUE_F64 = 0
VALUE_F32 = 1
VALUE_MIXED_F32 = 2
VALUE_MIXED_BF16 = 3
VALUE_NAMES = {VALUE_F64: "f64", VALUE_F32: "f32", VALUE_MIXED_F32: "mixed_f32",
               VALUE_MIXED_BF16: "mixed_bf16"}

# (non-zeros per lane, tiles per worker, warps per CTA, TMA stages; 0 stages = direct loads);
# BF16 storage defaults to 2 stages (its TMA-staged schedule is the faster one)
DEFAULT_CONFIG = (16, 8, 4, 0)


class SpmvError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"status {code}: {msg}")
        self.code = code


def host_dtype(value_type: int):
    """numpy dtype of val / x / y as passed through the handle API."""
    return np.float32 if value_type == VALUE_F32 else np.float64


def _ptr(a) -> int | None:
    return None if a is None else a.ctypes.data


class BhsparseSpmvCuda:
    """One ``bhsparse_spmv_cuda`` object (spmv_cuda/bhsparse_spmv_cuda.h:7-55)."""

    def __init__(self, value_type: int = VALUE_F64):
        self._L = lib()
        self._h = ctypes.c_void_p()
        rc = self._L.bhsp_create(ctypes.byref(self._h), int(value_type))
        if rc != BHSPARSE_SUCCESS:
            raise SpmvError(rc, "bhsp_create failed (unsupported value type?)")
        self.value_type = int(value_type)
        self._keep = ()
        self._y = None

    # -- the reference's methods -------------------------------------------------------
    def init_platform(self) -> int:
        return self._L.bhsp_init_platform(self._h)

    def prepare_mem(self, m: int, n: int, nnzA: int, csrRowPtrA, csrColIdxA, csrValA, x, y) -> int:
        """Copies A, x and y to the device; ``y`` (a writable numpy array) receives the
        result on get_y().  Arrays must be C-contiguous int32 / value-type arrays."""
        dt = host_dtype(self.value_type)
        rp = np.ascontiguousarray(csrRowPtrA, dtype=np.int32)
        ci = np.ascontiguousarray(csrColIdxA, dtype=np.int32)
        va = np.ascontiguousarray(csrValA, dtype=dt)
        xx = np.ascontiguousarray(x, dtype=dt)
        if not (isinstance(y, np.ndarray) and y.dtype == dt and y.flags.c_contiguous
                and y.flags.writeable):
            raise TypeError(f"y must be a writable C-contiguous numpy array of {np.dtype(dt)}")
        if rp.size < m + 1 or ci.size < nnzA or va.size < nnzA or xx.size < n or y.size < m:
            return BHSPARSE_INVALID_ARGUMENT
        self._y = y
        self._keep = (rp, ci, va, xx)
        return self._L.bhsp_prepare_mem(self._h, int(m), int(n), int(nnzA), _ptr(rp), _ptr(ci),
                                        _ptr(va), _ptr(xx), _ptr(y))

    def run_benchmark(self) -> int:
        return self._L.bhsp_run_benchmark(self._h)

    def get_y(self) -> int:
        return self._L.bhsp_get_y(self._h)

    def free_platform(self) -> int:
        return self._L.bhsp_free_platform(self._h)

    def free_mem(self) -> int:
        rc = self._L.bhsp_free_mem(self._h)
        self._keep = ()
        return rc

    # -- additions ---------------------------------------------------------------------
    @property
    def last_error(self) -> str:
        return self._L.bhsp_last_error(self._h).decode()

    def set_device(self, device: int) -> int:
        return self._L.bhsp_set_device(self._h, int(device))

    def set_tuner(self, path: str | None) -> int:
        """Network file for prepare_mem's schedule choice (None = the library's, "" = none)."""
        return self._L.bhsp_set_tuner(self._h, None if path is None else path.encode())

    def schedule_source(self) -> tuple[int, float]:
        """(BHSP_SCHEDULE_* source of the schedule in use, the network's confidence)."""
        src, conf = ctypes.c_int(), ctypes.c_float()
        self._L.bhsp_get_schedule_source(self._h, ctypes.byref(src), ctypes.byref(conf))
        return src.value, float(conf.value)

    def set_config(self, seg: int = 0, tiles_per_worker: int = 0, warps_per_cta: int = 0,
                   stages: int = -1) -> int:
        return self._L.bhsp_set_config(self._h, int(seg), int(tiles_per_worker), int(warps_per_cta),
                                       int(stages))

    def get_config(self) -> tuple[int, int, int, int]:
        a, b, c, d = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._L.bhsp_get_config(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                ctypes.byref(d))
        return a.value, b.value, c.value, d.value

    def set_x(self, x) -> int:
        xx = np.ascontiguousarray(x, dtype=host_dtype(self.value_type))
        rc = self._L.bhsp_set_x(self._h, _ptr(xx))
        self._keep = self._keep[:3] + (xx,) if self._keep else (xx,)
        return rc

    def set_x_ptr(self, ptr: int) -> int:
        """set_x from a raw host address (e.g. pinned memory); the caller keeps it alive."""
        return self._L.bhsp_set_x(self._h, ctypes.c_void_p(ptr))

    def run_stream(self, x_ptrs, y_ptrs) -> int:
        """bhsp_run_stream: y_ptrs[i] = A x_ptrs[i] for every pair of host addresses (pinned
        memory in the handle's value type; the caller keeps it alive), with the copies of
        neighbouring right-hand sides overlapping each SpMV."""
        if len(x_ptrs) != len(y_ptrs):
            raise ValueError("x_ptrs and y_ptrs differ in length")
        k = len(x_ptrs)
        xs = (ctypes.c_void_p * max(k, 1))(*[ctypes.c_void_p(int(p)) for p in x_ptrs])
        ys = (ctypes.c_void_p * max(k, 1))(*[ctypes.c_void_p(int(p)) for p in y_ptrs])
        return self._L.bhsp_run_stream(self._h, k, xs, ys)

    def run_async(self, stream: int = 0) -> int:
        return self._L.bhsp_run_async(self._h, ctypes.c_void_p(stream))

    def run_phase(self, stream: int, phase: int) -> int:
        """1 = tile kernel, 2 = calibration kernel, 3 = both (see bhsp_run_phase)."""
        return self._L.bhsp_run_phase(self._h, ctypes.c_void_p(stream), int(phase))

    def check(self) -> int:
        return self._L.bhsp_check(self._h)

    def device_buffers(self) -> dict:
        ptrs = [ctypes.c_void_p() for _ in range(5)]
        rc = self._L.bhsp_device_buffers(self._h, *[ctypes.byref(p) for p in ptrs])
        if rc != BHSPARSE_SUCCESS:
            raise SpmvError(rc, self.last_error)
        return dict(zip(("row_ptr", "col_idx", "val", "x", "y"), (p.value for p in ptrs)))

    def device_bytes(self) -> int:
        return int(self._L.bhsp_device_bytes(self._h))

    def close(self) -> None:
        if self._h:
            self._L.bhsp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _stream_ptr(stream) -> int:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return int(getattr(stream, "cuda_stream", stream))


class Plan:
    """The SpMV kernels on device buffers (torch CUDA tensors) owned by the caller.

    ``row_ptr`` / ``col_idx`` must stay alive as long as the plan.  ``execute`` enqueues
    y = A.x on the current torch stream (or ``stream``) without synchronising.
    """

    def __init__(self, value_type: int, m: int, n: int, row_ptr, col_idx, nnz: int | None = None,
                 seg: int = 0, tiles_per_worker: int = 0, warps_per_cta: int = 0, stages: int = -1,
                 stream=None):
        self._L = lib()
        self.value_type = int(value_type)
        self.m, self.n = int(m), int(n)
        self.nnz = int(col_idx.numel()) if nnz is None else int(nnz)
        self._rp, self._ci = row_ptr, col_idx
        self._p = ctypes.c_void_p()
        rc = self._L.bhsp_plan_create(ctypes.byref(self._p), self.value_type, self.m, self.n,
                                      self.nnz, row_ptr.data_ptr(), col_idx.data_ptr(), int(seg),
                                      int(tiles_per_worker), int(warps_per_cta), int(stages),
                                      ctypes.c_void_p(_stream_ptr(stream)))
        if rc != BHSPARSE_SUCCESS:
            raise SpmvError(rc, "bhsp_plan_create failed")

    def execute(self, val, x, y, stream=None) -> None:
        rc = self._L.bhsp_plan_execute(self._p, val.data_ptr(), x.data_ptr(), y.data_ptr(),
                                       ctypes.c_void_p(_stream_ptr(stream)))
        if rc != BHSPARSE_SUCCESS:
            raise SpmvError(rc, self.last_error)

    def check(self, stream=None) -> None:
        rc = self._L.bhsp_plan_check(self._p, ctypes.c_void_p(_stream_ptr(stream)))
        if rc != BHSPARSE_SUCCESS:
            raise SpmvError(rc, self.last_error)

    @property
    def launches(self) -> int:
        return int(self._L.bhsp_plan_launches(self._p))

    def tiles(self) -> tuple[int, int, int]:
        tp, nt, tn = ctypes.c_void_p(), ctypes.c_int(), ctypes.c_int()
        self._L.bhsp_plan_tiles(self._p, ctypes.byref(tp), ctypes.byref(nt), ctypes.byref(tn))
        return tp.value, nt.value, tn.value

    def chunk_form(self) -> tuple[int, bool]:
        """(non-empty rows shorter than a chunk, whether the one-head chunk form is on)."""
        sr, oh = ctypes.c_int(), ctypes.c_int()
        rc = self._L.bhsp_plan_chunk_form(self._p, ctypes.byref(sr), ctypes.byref(oh))
        if rc != BHSPARSE_SUCCESS:
            raise SpmvError(rc, self.last_error)
        return sr.value, bool(oh.value)

    def gather_path(self) -> tuple[int, int, bool]:
        """(sampled non-zeros, those with a near column, whether x is gathered from L2 only)."""
        sm, nr, l2 = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        rc = self._L.bhsp_plan_gather_path(self._p, ctypes.byref(sm), ctypes.byref(nr),
                                           ctypes.byref(l2))
        if rc != BHSPARSE_SUCCESS:
            raise SpmvError(rc, self.last_error)
        return sm.value, nr.value, bool(l2.value)

    def set_variant(self, one_head: bool | None = None, l2_only: bool | None = None) -> None:
        """Force the chunk form and / or the gather path (None keeps the plan's rule).  Every
        variant gives the same y; only the speed differs."""
        oh = -1 if one_head is None else int(bool(one_head))
        l2 = -1 if l2_only is None else int(bool(l2_only))
        rc = self._L.bhsp_plan_set_variant(self._p, oh, l2)
        if rc != BHSPARSE_SUCCESS:
            raise SpmvError(rc, "bhsp_plan_set_variant failed")

    def set_grid(self, persistent: bool | None = None) -> None:
        """Force the persistent (True) or the static (False) tile-kernel grid; None keeps the
        rule.  Same y either way."""
        rc = self._L.bhsp_plan_set_grid(self._p, -1 if persistent is None else int(bool(persistent)))
        if rc != BHSPARSE_SUCCESS:
            raise SpmvError(rc, "bhsp_plan_set_grid failed")

    @property
    def last_error(self) -> str:
        return self._L.bhsp_plan_last_error(self._p).decode()

    def close(self) -> None:
        if self._p:
            self._L.bhsp_plan_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def partition(row_ptr, nnz: int, tile_nnz: int, stream=None):
    """tile_ptr (uint32 bit patterns in an int32 tensor) for tiles of tile_nnz non-zeros."""
    import torch
    m = row_ptr.numel() - 1
    nt = (nnz + tile_nnz - 1) // tile_nnz
    out = torch.empty(nt + 1, dtype=torch.int32, device=row_ptr.device)
    rc = lib().bhsp_partition(row_ptr.data_ptr(), m, int(nnz), int(tile_nnz), out.data_ptr(),
                              ctypes.c_void_p(_stream_ptr(stream)))
    if rc != BHSPARSE_SUCCESS:
        raise SpmvError(rc, "bhsp_partition failed")
    return out


def bitflags(row_ptr, nnz: int, seg: int, tile_ptr, stream=None):
    """Raw bit-flag words, shape (ntiles, 32), as an int32 tensor of uint32 bit patterns."""
    import torch
    m = row_ptr.numel() - 1
    nt = tile_ptr.numel() - 1
    out = torch.zeros((max(nt, 0), 32), dtype=torch.int32, device=row_ptr.device)
    rc = lib().bhsp_bitflags(row_ptr.data_ptr(), m, int(nnz), int(seg), tile_ptr.data_ptr(),
                             out.data_ptr(), ctypes.c_void_p(_stream_ptr(stream)))
    if rc != BHSPARSE_SUCCESS:
        raise SpmvError(rc, "bhsp_bitflags failed")
    return out


def validate_csr(row_ptr, col_idx, n: int, stream=None) -> int:
    m = row_ptr.numel() - 1
    return int(lib().bhsp_validate_csr(row_ptr.data_ptr(), col_idx.data_ptr(), m, int(n),
                                       int(col_idx.numel()), ctypes.c_void_p(_stream_ptr(stream))))


def version() -> str:
    return lib().bhsp_version().decode()
