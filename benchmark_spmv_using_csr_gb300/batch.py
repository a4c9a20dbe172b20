"""Host side of the batched multi-RHS form: concatenation of many CSR matrices into one
block-diagonal CSR, the device buffers, and the C ABI calls (bhsp_batch_*)."""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import lib


def concatenate(mats) -> dict:
    """Block-diagonal concatenation: row pointers with global non-zero offsets, column indices
    shifted by each matrix's x offset.  Returns the arrays and per-matrix offsets."""
    m_off = np.zeros(len(mats) + 1, np.int64)
    n_off = np.zeros(len(mats) + 1, np.int64)
    z_off = np.zeros(len(mats) + 1, np.int64)
    for i, a in enumerate(mats):
        m_off[i + 1] = m_off[i] + a.m
        n_off[i + 1] = n_off[i] + a.n
        z_off[i + 1] = z_off[i] + a.nnz
    if z_off[-1] > np.iinfo(np.int32).max or m_off[-1] > np.iinfo(np.int32).max:
        raise ValueError("batch too large for int32 indices")
    row_ptr = np.empty(m_off[-1] + 1, np.int32)
    col = np.empty(z_off[-1], np.int32)
    val = np.empty(z_off[-1], np.float64)
    for i, a in enumerate(mats):
        row_ptr[m_off[i]:m_off[i + 1]] = a.row_ptr[:-1] + z_off[i]
        col[z_off[i]:z_off[i + 1]] = a.col + n_off[i]
        val[z_off[i]:z_off[i + 1]] = a.val
    row_ptr[-1] = z_off[-1]
    return {"row_ptr": row_ptr, "col": col, "val": val, "m_off": m_off, "n_off": n_off,
            "nnz_off": z_off, "m": int(m_off[-1]), "n": int(n_off[-1]), "nnz": int(z_off[-1])}


def _stream_ptr(stream) -> int:
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return int(getattr(s, "cuda_stream", s))


class Batch:
    """A batch of CSR matrices on the device with k right-hand sides (FP32 storage)."""

    def __init__(self, mats, k: int = 1, seg: int = 0, tiles_per_worker: int = 0,
                 warps_per_cta: int = 0, stream=None):
        import torch
        self.k = int(k)
        self.cat = concatenate(mats)
        self.count = len(mats)
        dev = "cuda"
        self.row_ptr = torch.from_numpy(self.cat["row_ptr"]).to(dev)
        self.col = torch.from_numpy(self.cat["col"]).to(dev)
        self.val = torch.from_numpy(self.cat["val"].astype(np.float32)).to(dev)
        self._b = ctypes.c_void_p()
        rc = lib().bhsp_batch_create(ctypes.byref(self._b), self.count, self.cat["m"],
                                     self.cat["n"], self.cat["nnz"], self.row_ptr.data_ptr(),
                                     self.col.data_ptr(), self.k, int(seg), int(tiles_per_worker),
                                     int(warps_per_cta), ctypes.c_void_p(_stream_ptr(stream)))
        if rc != 0:
            raise RuntimeError(f"bhsp_batch_create failed with status {rc}")

    def reschedule(self, seg: int, tiles_per_worker: int, warps_per_cta: int, stream=None) -> None:
        """Rebuild the batch's plan at another schedule on the same device buffers."""
        old = self._b
        self._b = ctypes.c_void_p()
        rc = lib().bhsp_batch_create(ctypes.byref(self._b), self.count, self.cat["m"],
                                     self.cat["n"], self.cat["nnz"], self.row_ptr.data_ptr(),
                                     self.col.data_ptr(), self.k, int(seg), int(tiles_per_worker),
                                     int(warps_per_cta), ctypes.c_void_p(_stream_ptr(stream)))
        if rc != 0:
            self._b = old
            raise RuntimeError(f"bhsp_batch_create failed with status {rc}")
        if old:
            lib().bhsp_batch_destroy(old)

    @property
    def m(self) -> int:
        return self.cat["m"]

    @property
    def n(self) -> int:
        return self.cat["n"]

    @property
    def nnz(self) -> int:
        return self.cat["nnz"]

    def execute(self, x, y, use_graph: bool = True, stream=None) -> None:
        """x: float32 CUDA tensor [n_total, k]; y: float32 CUDA tensor [m_total, k]."""
        rc = lib().bhsp_batch_execute(self._b, self.val.data_ptr(), x.data_ptr(), y.data_ptr(),
                                      1 if use_graph else 0, ctypes.c_void_p(_stream_ptr(stream)))
        if rc != 0:
            raise RuntimeError(f"bhsp_batch_execute failed ({rc}): {self.last_error}")

    def check(self, stream=None) -> None:
        rc = lib().bhsp_batch_check(self._b, ctypes.c_void_p(_stream_ptr(stream)))
        if rc != 0:
            raise RuntimeError(f"batched kernel check failed ({rc}): {self.last_error}")

    def info(self) -> dict:
        v = [ctypes.c_int() for _ in range(4)]
        lib().bhsp_batch_info(self._b, *[ctypes.byref(c) for c in v])
        out = dict(zip(("ntiles", "nworkers", "grid", "launches"), (c.value for c in v)))
        oh, l2 = ctypes.c_int(), ctypes.c_int()
        lib().bhsp_batch_variant(self._b, ctypes.byref(oh), ctypes.byref(l2))
        out.update(one_head=bool(oh.value), x_l2_only=bool(l2.value))
        return out

    def set_variant(self, one_head: bool | None = None, l2_only: bool | None = None) -> None:
        """Force the chunk form (one right-hand side only) and / or the gather path; None keeps
        the batch's rule.  Every variant gives the same y."""
        oh = -1 if one_head is None else int(bool(one_head))
        l2 = -1 if l2_only is None else int(bool(l2_only))
        rc = lib().bhsp_batch_set_variant(self._b, oh, l2)
        if rc != 0:
            raise RuntimeError(f"bhsp_batch_set_variant failed with status {rc}")

    @property
    def last_error(self) -> str:
        return lib().bhsp_batch_last_error(self._b).decode()

    def split(self, y_host: np.ndarray) -> list:
        """Per-matrix views of a host copy of y ([m_total, k])."""
        o = self.cat["m_off"]
        return [y_host[o[i]:o[i + 1]] for i in range(self.count)]

    def close(self) -> None:
        if self._b:
            lib().bhsp_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune_candidates() -> list[tuple[int, int, int]]:
    """(non-zeros per lane, tiles per worker, warps per CTA) of every batched candidate."""
    L = lib()
    out = []
    for i in range(L.bhsp_batch_tune_num_candidates()):
        v = [ctypes.c_int() for _ in range(3)]
        assert L.bhsp_batch_tune_candidate(i, *[ctypes.byref(c) for c in v]) == 0
        out.append(tuple(c.value for c in v))
    return out


def autotune(b: "Batch", x, y, warmup: int = 1, reps: int = 5, stream=None):
    """Time every batched candidate schedule on the batch's matrices (graph replay, L2 flushed
    before each timed run) with CUDA tensors x [n, k] and y [m, k]; returns (ms per candidate,
    index of the fastest)."""
    L = lib()
    ms = np.zeros(L.bhsp_batch_tune_num_candidates(), np.float32)
    best = ctypes.c_int(-1)
    rc = L.bhsp_batch_autotune(b.count, b.m, b.n, b.nnz, b.row_ptr.data_ptr(), b.col.data_ptr(),
                               b.k, b.val.data_ptr(), x.data_ptr(), y.data_ptr(), int(warmup),
                               int(reps), ms.ctypes.data_as(ctypes.c_void_p), ctypes.byref(best),
                               ctypes.c_void_p(_stream_ptr(stream)))
    if rc != 0:
        raise RuntimeError(f"bhsp_batch_autotune failed with status {rc}")
    return ms, best.value


def tuned(mats, k: int, x, y, cache=None, reps: int = 5):
    """A Batch at the schedule the batched autotuner picks for these matrices and k (looked up
    in, or added to, a tune.TuneCache keyed by k and the concatenated matrix's row features).
    Returns (batch, {"pick", "ms", "table", "cached"})."""
    from . import tune
    b = Batch(mats, k=k)
    key_vt = 100 + int(k)  # cache namespace of the batched form at k right-hand sides
    feats = tune.row_features(b.row_ptr, b.n)
    hit = cache.get(key_vt, feats) if cache is not None else None
    if hit is not None:
        ms, best = hit
    else:
        ms, best = autotune(b, x, y, reps=reps)
        if cache is not None:
            cache.put(key_vt, feats, ms, best)
            cache.save()
    cands = tune_candidates()
    b.reschedule(*cands[best])
    return b, {"pick": list(cands[best]), "ms": float(ms[best]),
                "table_ms": {",".join(map(str, c)): round(float(t), 4) for c, t in zip(cands, ms)},
                "cached": hit is not None}
