"""ctypes bindings of ``oracle.c`` (the C restatement of the reference path).

Test infrastructure only.  Each wrapper names the reference code it restates
(paths relative to the reference project):

* :func:`partition`         spmv_cuda/utils_cuda.h:6-31, spmv_cuda/kernels_cuda.h:39-53, 114-145
* :func:`bitflags`          spmv_cuda/kernels_cuda.h:114-148
* :func:`bhsparse`          spmv_cuda/kernels_cuda.h:7-269 + spmv_cuda/bhsparse_spmv_cuda.h:166-222
* :func:`bhsparse_kernel`   spmv_cuda/kernels_cuda.h:7-269 alone; :func:`calibrate` the host
                            steps spmv_cuda/bhsparse_spmv_cuda.h:166-222
* :func:`csr_serial`        spmv_cuda/main.cu:755-761
* :func:`csr_omp`           spmv_cuda/main.cu:370-393
* :func:`csr_dot2`          FP64 compensated oracle (Ogita-Rump-Oishi Dot2)

and, where ``make -C oracle ref`` built oracle/_ref/libref.so, the reference's own host code
compiled from its sources (:func:`ref_calibrate`, :func:`ref_serial`, :func:`ref_omp`), which
pins the restatements above.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liboracle.so")
_lock = threading.Lock()
_lib = None

LANES = 32  # THREADBUNCH, spmv_cuda/common.h:39
STEP = 7    # spmv_cuda/common.h:48
SEG_H_F64 = 4  # spmv_cuda/common.h:43
SEG_H_F32 = 8  # spmv_cuda/common.h:45

_i32p = ctypes.POINTER(ctypes.c_int32)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_f64p = ctypes.POINTER(ctypes.c_double)
_f32p = ctypes.POINTER(ctypes.c_float)


def build() -> str:
    """Compile ``oracle.c`` with its Makefile (idempotent)."""
    src = os.path.join(_HERE, "oracle.c")
    if not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


def lib() -> ctypes.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            _lib = ctypes.CDLL(build())
            L = _lib
            L.oracle_search_right.argtypes = [_i32p, ctypes.c_int, ctypes.c_int]
            L.oracle_search_right.restype = ctypes.c_int
            L.oracle_num_tiles.argtypes = [ctypes.c_int, ctypes.c_int]
            L.oracle_num_tiles.restype = ctypes.c_int
            L.oracle_num_warps.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
            L.oracle_num_warps.restype = ctypes.c_int
            L.oracle_partition.argtypes = [_i32p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _u32p]
            L.oracle_partition.restype = None
            L.oracle_bitflags.argtypes = [_i32p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, _u32p, _u32p]
            L.oracle_bitflags.restype = None
            for name, vp in (("oracle_bhsparse_f64", _f64p), ("oracle_bhsparse_f32", _f32p)):
                f = getattr(L, name)
                f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, vp, vp,
                              ctypes.c_int, ctypes.c_int, vp, _i32p, vp, _i32p, _i32p, _i32p]
                f.restype = ctypes.c_int
            for name, vp in (("oracle_bhsparse_kernel_f64", _f64p),
                             ("oracle_bhsparse_kernel_f32", _f32p)):
                f = getattr(L, name)
                f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, vp, vp,
                              ctypes.c_int, ctypes.c_int, vp, _i32p, vp, _i32p, _i32p]
                f.restype = ctypes.c_int
            for name, vp in (("oracle_calibrate_f64", _f64p), ("oracle_calibrate_f32", _f32p)):
                f = getattr(L, name)
                f.argtypes = [ctypes.c_int, _i32p, ctypes.c_int, _i32p, vp, ctypes.c_int, _i32p,
                              vp, _i32p]
                f.restype = None
            L.oracle_csr_serial_f64.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
            L.oracle_csr_serial_f32.argtypes = [ctypes.c_int, _i32p, _i32p, _f32p, _f32p, _f32p]
            L.oracle_csr_serial_rows_f64.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p,
                                                     _f64p, _f64p, _f64p]
            L.oracle_csr_omp_f64.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p, _f64p, _f64p,
                                             ctypes.c_int]
            L.oracle_csr_omp_f32.argtypes = [ctypes.c_int, _i32p, _i32p, _f32p, _f32p, _f32p,
                                             ctypes.c_int]
            L.oracle_csr_dot2.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p, _f64p, _f64p,
                                          ctypes.c_int]
            L.oracle_csr_absrow.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p, _f64p, _f64p,
                                            ctypes.c_int]
            L.oracle_max_threads.restype = ctypes.c_int
        return _lib


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def _c(a, dtype) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=dtype)


def num_tiles(nnz: int, ps: int) -> int:
    return int(lib().oracle_num_tiles(int(nnz), int(ps)))


def num_warps(nnz: int, seg_h: int, step: int = STEP) -> int:
    return int(lib().oracle_num_warps(int(nnz), int(seg_h), int(step)))


def search_right(row_ptr, key: int) -> int:
    rp = _c(row_ptr, np.int32)
    return int(lib().oracle_search_right(_p(rp, _i32p), int(key), rp.size))


def partition(row_ptr, nnz: int, ps: int) -> np.ndarray:
    """tile_ptr[0..ntiles] as uint32: row of boundary t*ps, bit 31 = tile t dirty."""
    rp = _c(row_ptr, np.int32)
    m = rp.size - 1
    out = np.zeros(num_tiles(nnz, ps) + 1, dtype=np.uint32)
    lib().oracle_partition(_p(rp, _i32p), m, int(nnz), int(ps), _p(out, _u32p))
    return out


def bitflags(row_ptr, nnz: int, lanes: int, seg: int, tile_ptr=None) -> np.ndarray:
    """Raw bit-flag words, shape (ntiles, lanes), before lane 0's head bit is forced."""
    rp = _c(row_ptr, np.int32)
    m = rp.size - 1
    ps = lanes * seg
    if tile_ptr is None:
        tile_ptr = partition(rp, nnz, ps)
    tp = _c(tile_ptr, np.uint32)
    nt = num_tiles(nnz, ps)
    out = np.zeros((nt, lanes), dtype=np.uint32)
    lib().oracle_bitflags(_p(rp, _i32p), m, int(nnz), int(lanes), int(seg), _p(tp, _u32p),
                          _p(out, _u32p))
    return out


class BhsparseResult:
    """Everything the simulated reference kernel + host calibration produce."""

    def __init__(self, y, sync_idx, sync_val, spec, ndirty, oob_guarded):
        self.y = y
        self.sync_idx = sync_idx
        self.sync_val = sync_val
        self.speculator = spec
        self.ndirty = ndirty
        self.oob_guarded = oob_guarded


def bhsparse(row_ptr, col, val, x, n: int | None = None, seg_h: int | None = None,
             step: int = STEP, y0=None) -> BhsparseResult:
    """Lane-level simulation of SpMV_kernel + run_benchmark's host calibration.

    The value type follows ``val.dtype`` (float64 -> USE_DOUBLE=1, float32 ->
    USE_DOUBLE=0).  ``y0`` is the y the object holds before the call (zeros,
    as spmv_cuda/main.cu:769 sets it, when omitted).
    """
    rp = _c(row_ptr, np.int32)
    ci = _c(col, np.int32)
    m = rp.size - 1
    nnz = int(rp[-1]) if m >= 0 else 0
    if np.asarray(val).dtype == np.float32:
        vt, vp, fn = np.float32, _f32p, lib().oracle_bhsparse_f32
        seg_h = SEG_H_F32 if seg_h is None else seg_h
    else:
        vt, vp, fn = np.float64, _f64p, lib().oracle_bhsparse_f64
        seg_h = SEG_H_F64 if seg_h is None else seg_h
    v = _c(val, vt)
    xx = _c(x, vt)
    n = xx.size if n is None else n
    y = np.zeros(max(m, 1), dtype=vt) if y0 is None else _c(y0, vt).copy()
    nw = num_warps(nnz, seg_h, step)
    sidx = np.zeros(max(nw, 1), dtype=np.int32)
    sval = np.zeros(max(nw, 1), dtype=vt)
    spec = np.zeros(2 * max(num_tiles(nnz, LANES * seg_h), 1), dtype=np.int32)
    nd = ctypes.c_int(0)
    fl = ctypes.c_int(0)
    rc = fn(m, int(n), nnz, _p(rp, _i32p), _p(ci, _i32p), _p(v, vp), _p(xx, vp), int(seg_h),
            int(step), _p(y, vp), _p(sidx, _i32p), _p(sval, vp), _p(spec, _i32p),
            ctypes.byref(nd), ctypes.byref(fl))
    if rc < 0:
        raise ValueError("unsupported geometry")
    return BhsparseResult(y[:m], sidx[:nw], sval[:nw], spec[:2 * nd.value].reshape(-1, 2),
                          nd.value, bool(fl.value & 1))


class KernelStage:
    """What the simulated SpMV_kernel leaves before run_benchmark's host steps: the compacted
    y, the synchronizer (one entry per warp) and the speculator (dirty tiles)."""

    def __init__(self, y, sync_idx, sync_val, spec, ndirty):
        self.y = y
        self.sync_idx = sync_idx
        self.sync_val = sync_val
        self.speculator = spec
        self.ndirty = ndirty


def bhsparse_kernel(row_ptr, col, val, x, seg_h: int | None = None, step: int = STEP,
                    y0=None) -> KernelStage:
    """Lane-level simulation of SpMV_kernel alone (spmv_cuda/kernels_cuda.h:7-269)."""
    rp = _c(row_ptr, np.int32)
    ci = _c(col, np.int32)
    m = rp.size - 1
    nnz = int(rp[-1]) if m >= 0 else 0
    if np.asarray(val).dtype == np.float32:
        vt, vp, fn = np.float32, _f32p, lib().oracle_bhsparse_kernel_f32
        seg_h = SEG_H_F32 if seg_h is None else seg_h
    else:
        vt, vp, fn = np.float64, _f64p, lib().oracle_bhsparse_kernel_f64
        seg_h = SEG_H_F64 if seg_h is None else seg_h
    v, xx = _c(val, vt), _c(x, vt)
    y = np.zeros(max(m, 1), dtype=vt) if y0 is None else _c(y0, vt).copy()
    nw = num_warps(nnz, seg_h, step)
    sidx = np.zeros(max(nw, 1), dtype=np.int32)
    sval = np.zeros(max(nw, 1), dtype=vt)
    spec = np.zeros(2 * max(num_tiles(nnz, LANES * seg_h), 1), dtype=np.int32)
    nd = ctypes.c_int(0)
    rc = fn(m, xx.size, nnz, _p(rp, _i32p), _p(ci, _i32p), _p(v, vp), _p(xx, vp), int(seg_h),
            int(step), _p(y, vp), _p(sidx, _i32p), _p(sval, vp), _p(spec, _i32p),
            ctypes.byref(nd))
    if rc < 0:
        raise ValueError("unsupported geometry")
    return KernelStage(y[:m].copy(), sidx[:nw].copy(), sval[:nw].copy(),
                       spec[:2 * nd.value].copy(), nd.value)


def calibrate(row_ptr, stage: KernelStage):
    """The oracle's restatement of run_benchmark's host steps (bhsparse_spmv_cuda.h:166-222)
    applied to a copy of stage.y: (y, True if the fix-up would have read row_ptr[m+1])."""
    rp = _c(row_ptr, np.int32)
    m = rp.size - 1
    vt = stage.y.dtype
    vp = _f32p if vt == np.float32 else _f64p
    fn = lib().oracle_calibrate_f32 if vt == np.float32 else lib().oracle_calibrate_f64
    y = np.zeros(max(m, 1), vt)
    y[:m] = stage.y
    sidx, sval = _c(stage.sync_idx, np.int32), _c(stage.sync_val, vt)
    spec = _c(stage.speculator, np.int32) if stage.ndirty else np.zeros(2, np.int32)
    fl = ctypes.c_int(0)
    fn(m, _p(rp, _i32p), int(sidx.size), _p(sidx, _i32p), _p(sval, vp), int(stage.ndirty),
       _p(spec, _i32p), _p(y, vp), ctypes.byref(fl))
    return y[:m], bool(fl.value & 1)


# -- the reference's own host loops, compiled from its sources (oracle/_ref/libref.so) --------
_REF_SO = os.path.join(_HERE, "_ref", "libref.so")
_ref = None


def ref_lib():
    """oracle/_ref/libref.so (oracle/ref_harness.cpp around the reference's host calibration,
    serial and OpenMP loops, built by ``make -C oracle ref``), or None where it was not built."""
    global _ref
    with _lock:
        if _ref is None and os.path.exists(_REF_SO):
            L = ctypes.CDLL(_REF_SO)
            for sfx, vp in (("f64", _f64p), ("f32", _f32p)):
                f = getattr(L, "ref_calibrate_" + sfx)
                f.argtypes = [ctypes.c_int, _i32p, vp, vp, ctypes.c_int, vp, _i32p, _i32p,
                              ctypes.c_int]
                f.restype = None
                f = getattr(L, "ref_serial_" + sfx)
                f.argtypes = [ctypes.c_int, _i32p, _i32p, vp, vp, vp]
                f.restype = None
                f = getattr(L, "ref_omp_" + sfx)
                f.argtypes = [ctypes.c_int, _i32p, _i32p, vp, vp, vp, ctypes.c_int, ctypes.c_int]
                f.restype = None
            _ref = L
        return _ref


def ref_calibrate(row_ptr, stage: KernelStage):
    """The reference's own host calibration (spmv_cuda/bhsparse_spmv_cuda.h:170-222, compiled
    from its source) applied to a copy of stage.y: (y[:m], value it wrote at y[m]).  row_ptr, y
    and y_temp get one extra entry (row_ptr[m+1] = row_ptr[m]) so that the fix-up's read of
    row_ptr[m+1] and write of y[m] for a dirty last tile stay inside the buffers."""
    L = ref_lib()
    rp = _c(row_ptr, np.int32)
    m = rp.size - 1
    rpp = np.concatenate([rp, rp[-1:]])
    vt = stage.y.dtype
    vp = _f32p if vt == np.float32 else _f64p
    fn = L.ref_calibrate_f32 if vt == np.float32 else L.ref_calibrate_f64
    y = np.zeros(m + 1, vt)
    y[:m] = stage.y
    yt = np.zeros(m + 1, vt)
    sidx, sval = _c(stage.sync_idx, np.int32), _c(stage.sync_val, vt)
    spec = _c(stage.speculator, np.int32) if stage.ndirty else np.zeros(2, np.int32)
    fn(int(sidx.size), _p(sidx, _i32p), _p(sval, vp), _p(y, vp), int(stage.ndirty), _p(yt, vp),
       _p(spec, _i32p), _p(rpp, _i32p), m)
    return y[:m], y[m]


def ref_serial(row_ptr, col, val, x, y=None) -> np.ndarray:
    """The reference's own serial CSR loop (spmv_cuda/main.cu:753-762, compiled from its source),
    into ``y`` when given (contiguous, of val's type, at least max(m, 1) entries)."""
    L = ref_lib()
    rp, ci = _c(row_ptr, np.int32), _c(col, np.int32)
    m = rp.size - 1
    vt = np.float32 if np.asarray(val).dtype == np.float32 else np.float64
    vp = _f32p if vt == np.float32 else _f64p
    fn = L.ref_serial_f32 if vt == np.float32 else L.ref_serial_f64
    v, xx = _c(val, vt), _c(x, vt)
    if y is None:
        y = np.zeros(max(m, 1), vt)
    assert y.dtype == vt and y.flags.c_contiguous and y.size >= max(m, 1)
    fn(m, _p(rp, _i32p), _p(ci, _i32p), _p(v, vp), _p(xx, vp), _p(y, vp))
    return y[:m]


def ref_omp(row_ptr, col, val, x, threads: int, runs: int = 1, y=None) -> np.ndarray:
    """The reference's own OpenMP CSR loop (spmv_cuda/main.cu:377-393, compiled from its
    source): `runs` passes on `threads` host threads, into ``y`` when given (float64, no copies
    of the inputs when they are already contiguous int32 / float64)."""
    L = ref_lib()
    rp, ci = _c(row_ptr, np.int32), _c(col, np.int32)
    m = rp.size - 1
    v, xx = _c(val, np.float64), _c(x, np.float64)
    if y is None:
        y = np.zeros(max(m, 1), np.float64)
    L.ref_omp_f64(m, _p(rp, _i32p), _p(ci, _i32p), _p(v, _f64p), _p(xx, _f64p), _p(y, _f64p),
                  int(runs), int(threads))
    return y[:m]


def gen_library_path() -> str:
    """oracle/_build/libgen.so: the package's seeded workload generators (csrc/gen.cpp) built on
    their own by oracle/Makefile, for CPU code that must not load the GPU library."""
    so = os.path.join(_HERE, "_build", "libgen.so")
    if not os.path.exists(so):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return so


def csr_serial(row_ptr, col, val, x) -> np.ndarray:
    rp, ci = _c(row_ptr, np.int32), _c(col, np.int32)
    m = rp.size - 1
    if np.asarray(val).dtype == np.float32:
        v, xx = _c(val, np.float32), _c(x, np.float32)
        y = np.zeros(max(m, 1), np.float32)
        lib().oracle_csr_serial_f32(m, _p(rp, _i32p), _p(ci, _i32p), _p(v, _f32p),
                                    _p(xx, _f32p), _p(y, _f32p))
    else:
        v, xx = _c(val, np.float64), _c(x, np.float64)
        y = np.zeros(max(m, 1), np.float64)
        lib().oracle_csr_serial_f64(m, _p(rp, _i32p), _p(ci, _i32p), _p(v, _f64p),
                                    _p(xx, _f64p), _p(y, _f64p))
    return y[:m]


def csr_serial_rows(row_ptr, col, val, x, y, r0: int, r1: int) -> None:
    """Serial loop over rows [r0, r1) into ``y`` (float64 arrays, no copies)."""
    lib().oracle_csr_serial_rows_f64(int(r0), int(r1), _p(row_ptr, _i32p), _p(col, _i32p),
                                     _p(val, _f64p), _p(x, _f64p), _p(y, _f64p))


def csr_omp(row_ptr, col, val, x, nthreads: int = 0, y=None) -> np.ndarray:
    rp, ci = _c(row_ptr, np.int32), _c(col, np.int32)
    m = rp.size - 1
    if np.asarray(val).dtype == np.float32:
        v, xx = _c(val, np.float32), _c(x, np.float32)
        y = np.zeros(max(m, 1), np.float32) if y is None else y
        lib().oracle_csr_omp_f32(m, _p(rp, _i32p), _p(ci, _i32p), _p(v, _f32p), _p(xx, _f32p),
                                 _p(y, _f32p), int(nthreads))
    else:
        v, xx = _c(val, np.float64), _c(x, np.float64)
        y = np.zeros(max(m, 1), np.float64) if y is None else y
        lib().oracle_csr_omp_f64(m, _p(rp, _i32p), _p(ci, _i32p), _p(v, _f64p), _p(xx, _f64p),
                                 _p(y, _f64p), int(nthreads))
    return y[:m]


def csr_dot2(row_ptr, col, val, x, nthreads: int = 0) -> np.ndarray:
    """FP64 compensated y* (Dot2 per row); val/x are taken as float64."""
    rp, ci = _c(row_ptr, np.int32), _c(col, np.int32)
    v, xx = _c(val, np.float64), _c(x, np.float64)
    m = rp.size - 1
    y = np.zeros(max(m, 1), np.float64)
    lib().oracle_csr_dot2(m, _p(rp, _i32p), _p(ci, _i32p), _p(v, _f64p), _p(xx, _f64p),
                          _p(y, _f64p), int(nthreads))
    return y[:m]


def csr_absrow(row_ptr, col, val, x, nthreads: int = 0) -> np.ndarray:
    """(|A|.|x|)_i in float64: the scale of the componentwise tolerance."""
    rp, ci = _c(row_ptr, np.int32), _c(col, np.int32)
    v, xx = _c(val, np.float64), _c(x, np.float64)
    m = rp.size - 1
    y = np.zeros(max(m, 1), np.float64)
    lib().oracle_csr_absrow(m, _p(rp, _i32p), _p(ci, _i32p), _p(v, _f64p), _p(xx, _f64p),
                            _p(y, _f64p), int(nthreads))
    return y[:m]


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def componentwise_error(y, y_star, absrow) -> float:
    """max_i |y_i - y*_i| / (|A|.|x|)_i over rows with a non-zero scale."""
    y = np.asarray(y, np.float64)
    d = np.abs(y - y_star)
    s = np.asarray(absrow, np.float64)
    nz = s > 0
    if (~nz).any() and np.any(d[~nz] != 0):
        return float("inf")
    return float((d[nz] / s[nz]).max()) if nz.any() else 0.0


def normwise_error(y, y_star) -> float:
    """||y - y*||_2 / ||y*||_2."""
    y = np.asarray(y, np.float64)
    den = np.linalg.norm(y_star)
    return float(np.linalg.norm(y - y_star) / den) if den > 0 else float(np.linalg.norm(y))
