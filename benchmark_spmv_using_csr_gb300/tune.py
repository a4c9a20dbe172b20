"""Schedule tuning: the autotuner (a timed sweep of every candidate schedule), the row-length
features of a matrix, and a persistent timing-table cache keyed by those features.

The learned tuner (:mod:`benchmark_spmv_using_csr_gb300.mlp`) is trained on tables this module
produces and falls back to :func:`autotune` when it is not confident.  Tuning only picks a
schedule (non-zeros per lane, tiles per worker, warps per CTA); it never changes the arithmetic.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os

import numpy as np

from ._lib import lib

NUM_FEATURES = 16
FEATURE_NAMES = (
    "log2_m", "log2_n", "log2_nnz", "log2_mean_len", "log2_std_len", "log2_max_len",
    "empty_frac", "len_1", "len_2_3", "len_4_7", "len_8_15", "len_16_31", "len_32_63",
    "len_64_255", "len_256_4095", "len_ge_4096")


def candidates() -> list[tuple[int, int, int, int]]:
    """(non-zeros per lane, tiles per worker, warps per CTA, stages) of every candidate."""
    L = lib()
    out = []
    for i in range(L.bhsp_tune_num_candidates()):
        v = [ctypes.c_int() for _ in range(4)]
        assert L.bhsp_tune_candidate(i, *[ctypes.byref(c) for c in v]) == 0
        out.append(tuple(c.value for c in v))
    return out


def _stream_ptr(stream) -> int:
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return int(getattr(s, "cuda_stream", s))


def autotune(value_type: int, row_ptr, col_idx, val, x, y, n: int | None = None,
             warmup: int = 2, reps: int = 5, stream=None) -> tuple[np.ndarray, int]:
    """Time every candidate schedule on torch CUDA tensors; returns (ms per candidate, best)."""
    L = lib()
    k = L.bhsp_tune_num_candidates()
    ms = np.zeros(k, np.float32)
    best = ctypes.c_int(-1)
    m = row_ptr.numel() - 1
    n = x.numel() if n is None else n
    rc = L.bhsp_autotune(int(value_type), m, int(n), int(col_idx.numel()), row_ptr.data_ptr(),
                         col_idx.data_ptr(), val.data_ptr(), x.data_ptr(), y.data_ptr(),
                         int(warmup), int(reps), ms.ctypes.data_as(ctypes.c_void_p),
                         ctypes.byref(best), ctypes.c_void_p(_stream_ptr(stream)))
    if rc != 0:
        raise RuntimeError(f"bhsp_autotune failed with status {rc}")
    return ms, best.value


def choose_schedule(value_type: int, row_ptr, col_idx, val, x, y, n: int | None = None,
                    tuner: str | None = None, stream=None) -> dict:
    """The schedule bhsp_choose_schedule picks for a device matrix (torch CUDA tensors): the
    learned network's, or the sweep's below its confidence threshold.  tuner: None = the
    library's network for value_type, "" = none, else a network file.  Returns {"config",
    "source" (SCHEDULE_*), "confidence"}."""
    L = lib()
    c = [ctypes.c_int() for _ in range(4)]
    src, conf = ctypes.c_int(), ctypes.c_float()
    m = row_ptr.numel() - 1
    n = x.numel() if n is None else n
    rc = L.bhsp_choose_schedule(int(value_type), m, int(n), int(col_idx.numel()),
                                row_ptr.data_ptr(), col_idx.data_ptr(), val.data_ptr(),
                                x.data_ptr(), y.data_ptr(),
                                None if tuner is None else tuner.encode(),
                                *[ctypes.byref(v) for v in c], ctypes.byref(src),
                                ctypes.byref(conf), ctypes.c_void_p(_stream_ptr(stream)))
    if rc != 0:
        raise RuntimeError(f"bhsp_choose_schedule failed with status {rc}")
    return {"config": tuple(v.value for v in c), "source": src.value,
            "confidence": float(conf.value)}


def row_features(row_ptr, n: int, stream=None) -> np.ndarray:
    """The 16 row-length features, computed on the device from a torch CUDA row_ptr."""
    f = np.zeros(NUM_FEATURES, np.float32)
    rc = lib().bhsp_row_features(row_ptr.data_ptr(), row_ptr.numel() - 1, int(n),
                                 f.ctypes.data_as(ctypes.c_void_p),
                                 ctypes.c_void_p(_stream_ptr(stream)))
    if rc != 0:
        raise RuntimeError(f"bhsp_row_features failed with status {rc}")
    return f


def feature_counts(row_ptr: np.ndarray) -> np.ndarray:
    """Host computation of the 13 counts the device kernel accumulates (sum, sum of squares,
    max, empty rows, 9 length-bin counts)."""
    L = np.diff(np.asarray(row_ptr, np.int64))
    c = np.zeros(13, np.uint64)
    c[0] = L.sum()
    c[1] = (L.astype(np.uint64) ** 2).sum()
    c[2] = L.max() if L.size else 0
    c[3] = (L == 0).sum()
    nz = L[L > 0]
    lg = np.floor(np.log2(nz)).astype(np.int64) if nz.size else np.zeros(0, np.int64)
    b = np.where(lg <= 5, lg, np.where(lg < 8, 6, np.where(lg < 12, 7, 8)))
    for i in range(9):
        c[4 + i] = (b == i).sum()
    return c


def features_from_counts(m: int, n: int, counts: np.ndarray) -> np.ndarray:
    c = np.ascontiguousarray(counts, np.uint64)
    f = np.zeros(NUM_FEATURES, np.float32)
    lib().bhsp_features_from_counts(int(m), int(n), c.ctypes.data_as(ctypes.c_void_p),
                                    f.ctypes.data_as(ctypes.c_void_p))
    return f


class TuneCache:
    """Timing tables persisted as JSON, keyed by value type and the matrix's feature vector."""

    def __init__(self, path: str):
        self.path = path
        self.table = {}
        if os.path.exists(path):
            with open(path) as fh:
                self.table = json.load(fh)

    @staticmethod
    def key(value_type: int, features: np.ndarray) -> str:
        h = hashlib.sha1(np.round(np.asarray(features, np.float64), 5).tobytes()).hexdigest()[:16]
        return f"{int(value_type)}:{h}"

    def get(self, value_type: int, features: np.ndarray):
        e = self.table.get(self.key(value_type, features))
        return None if e is None else (np.array(e["ms"], np.float32), int(e["best"]))

    def put(self, value_type: int, features: np.ndarray, ms: np.ndarray, best: int) -> None:
        self.table[self.key(value_type, features)] = {
            "ms": [float(v) for v in ms], "best": int(best),
            "features": [float(v) for v in features]}

    def save(self) -> None:
        tmp = self.path + ".tmp"
        with open(tmp, "w") as fh:
            json.dump(self.table, fh)
        os.replace(tmp, self.path)

    def tune(self, value_type: int, row_ptr, col_idx, val, x, y, n: int | None = None,
             **kw) -> tuple[np.ndarray, int]:
        n = x.numel() if n is None else n
        f = row_features(row_ptr, n)
        hit = self.get(value_type, f)
        if hit is not None:
            return hit
        ms, best = autotune(value_type, row_ptr, col_idx, val, x, y, n=n, **kw)
        self.put(value_type, f, ms, best)
        return ms, best
