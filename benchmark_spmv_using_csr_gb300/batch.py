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
        return dict(zip(("ntiles", "nworkers", "grid", "launches"), (c.value for c in v)))

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
