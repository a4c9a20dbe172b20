"""Seeded synthetic CSR workloads (numpy), generated by the library's C generators.

The three single-matrix workloads of the benchmark:

* ``stencil5_256``  -- 2D 5-point Laplacian on a 256x256 grid (m = n = 65,536,
  nnz = 326,656), values 4 / -1 plus uniform[-1e-3, 1e-3];
* ``powerlaw_4m``   -- m = n = 4,194,304, row lengths floor(xmin * U^(-1/1.1)) clipped
  to [1, 200,000] (a Zipf(2.1) tail) with xmin = 1.98 so that the mean non-empty row has
  about 15 entries (about 60 M non-zeros), 5 % of rows forced empty, distinct sorted
  uniform columns, values and x uniform[-1, 1];
* ``stencil27_160`` -- 3D 27-point stencil on a 160^3 grid (m = n = 4,096,000,
  nnz = 109,215,352), weights 26 / -1 times (1 + uniform[-0.01, 0.01]).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from ._lib import SIGNATURES, lib

_gen_override = None


def use_library(path: str) -> None:
    """Take the generators from another build of csrc/gen.cpp (a shared library exporting the
    bhsp_gen_* functions of include/spmv_gen.h), so that a CPU-only process can build the same
    seeded matrices without loading the GPU library."""
    global _gen_override
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        if name.startswith("bhsp_gen_"):
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
    _gen_override = L


def _lib():
    return _gen_override if _gen_override is not None else lib()


POWERLAW_ALPHA = 2.1
POWERLAW_XMIN = 1.98
POWERLAW_MAX_LEN = 200_000
POWERLAW_EMPTY = 0.05


@dataclass
class CSR:
    m: int
    n: int
    row_ptr: np.ndarray  # int32 [m+1]
    col: np.ndarray      # int32 [nnz]
    val: np.ndarray      # float64 [nnz]
    name: str = ""

    @property
    def nnz(self) -> int:
        return int(self.row_ptr[-1]) if self.m >= 0 else 0


def _p(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def _check(rc, what):
    if rc < 0:
        raise ValueError(f"{what} failed ({rc})")
    return rc


def uniform(count: int, seed: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    out = np.empty(max(count, 0), np.float64)
    _check(_lib().bhsp_gen_uniform(int(count), int(seed), float(lo), float(hi), _p(out)), "uniform")
    return out


def uniform_int(count: int, seed: int, modulus: int = 10) -> np.ndarray:
    """Integer-valued doubles in [0, modulus): the reference's rand()%10 data, seeded."""
    out = np.empty(max(count, 0), np.float64)
    _check(_lib().bhsp_gen_uniform_int(int(count), int(seed), int(modulus), _p(out)), "uniform_int")
    return out


def stencil2d(nx: int, ny: int | None = None, noise: float = 1e-3, seed: int = 1) -> CSR:
    ny = nx if ny is None else ny
    nnz = _check(_lib().bhsp_gen_stencil2d_nnz(nx, ny), "stencil2d_nnz")
    m = nx * ny
    rp = np.empty(m + 1, np.int32)
    col = np.empty(nnz, np.int32)
    val = np.empty(nnz, np.float64)
    _check(_lib().bhsp_gen_stencil2d(nx, ny, float(noise), int(seed), _p(rp), _p(col), _p(val)),
           "stencil2d")
    return CSR(m, m, rp, col, val, f"stencil5_{nx}x{ny}")


def stencil3d(nx: int, ny: int | None = None, nz: int | None = None, noise: float = 0.01,
              seed: int = 1) -> CSR:
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    nnz = _check(_lib().bhsp_gen_stencil3d_nnz(nx, ny, nz), "stencil3d_nnz")
    m = nx * ny * nz
    rp = np.empty(m + 1, np.int32)
    col = np.empty(nnz, np.int32)
    val = np.empty(nnz, np.float64)
    _check(_lib().bhsp_gen_stencil3d(nx, ny, nz, float(noise), int(seed), _p(rp), _p(col), _p(val)),
           "stencil3d")
    return CSR(m, m, rp, col, val, f"stencil27_{nx}x{ny}x{nz}")


def _fill(m, n, rp, seed, lo=-1.0, hi=1.0):
    nnz = int(rp[-1])
    col = np.empty(nnz, np.int32)
    val = np.empty(nnz, np.float64)
    _check(_lib().bhsp_gen_random_fill(m, n, _p(rp), float(lo), float(hi), int(seed), _p(col),
                                      _p(val)), "random_fill")
    return col, val


def powerlaw(m: int, n: int | None = None, alpha: float = POWERLAW_ALPHA,
             xmin: float = POWERLAW_XMIN, max_len: int = POWERLAW_MAX_LEN,
             empty_frac: float = POWERLAW_EMPTY, seed: int = 2) -> CSR:
    n = m if n is None else n
    rp = np.empty(m + 1, np.int32)
    _check(_lib().bhsp_gen_powerlaw_rows(m, float(alpha), float(xmin), min(int(max_len), n),
                                        float(empty_frac), int(seed), _p(rp)), "powerlaw_rows")
    col, val = _fill(m, n, rp, seed + 1000)
    return CSR(m, n, rp, col, val, f"powerlaw_{m}")


def density(m: int, n: int, dens: float, seed: int = 3) -> CSR:
    rp = np.empty(m + 1, np.int32)
    _check(_lib().bhsp_gen_density_rows(m, n, float(dens), int(seed), _p(rp)), "density_rows")
    col, val = _fill(m, n, rp, seed + 1000)
    return CSR(m, n, rp, col, val, f"density_{m}")


def mixed_rows(m: int, n: int, dense_row: int = -1, mean_len: float = 8.0,
               empty_frac: float = 0.0, seed: int = 4) -> CSR:
    """Poisson(mean_len) rows with an optional fully dense row and forced-empty rows."""
    rp = np.empty(m + 1, np.int32)
    _check(_lib().bhsp_gen_mixed_rows(m, n, int(dense_row), float(mean_len), float(empty_frac),
                                     int(seed), _p(rp)), "mixed_rows")
    col, val = _fill(m, n, rp, seed + 1000)
    return CSR(m, n, rp, col, val, f"mixed_{m}")


def blockdiag(m: int, n: int | None = None, bs: int = 32, seed: int = 5) -> CSR:
    n = m if n is None else n
    rp = np.empty(m + 1, np.int32)
    _check(_lib().bhsp_gen_blockdiag_rows(m, n, int(bs), _p(rp)), "blockdiag_rows")
    nnz = int(rp[-1])
    col = np.empty(nnz, np.int32)
    val = np.empty(nnz, np.float64)
    _check(_lib().bhsp_gen_blockdiag_fill(m, n, int(bs), -1.0, 1.0, int(seed), _p(rp), _p(col),
                                         _p(val)), "blockdiag_fill")
    return CSR(m, n, rp, col, val, f"blockdiag{bs}_{m}")


def from_row_lengths(lengths, n: int, seed: int = 6) -> CSR:
    lengths = np.asarray(lengths, np.int64)
    m = lengths.size
    rp = np.zeros(m + 1, np.int64)
    rp[1:] = np.cumsum(lengths)
    if rp[-1] > np.iinfo(np.int32).max:
        raise ValueError("too many non-zeros")
    rp = rp.astype(np.int32)
    col, val = _fill(m, n, rp, seed)
    return CSR(m, n, rp, col, val, f"rows_{m}")


# --- the benchmark's single-matrix workloads ------------------------------------------
def stencil5_256(seed: int = 1) -> CSR:
    return stencil2d(256, 256, noise=1e-3, seed=seed)


def powerlaw_4m(seed: int = 2) -> CSR:
    return powerlaw(4_194_304, seed=seed)


def stencil27_160(seed: int = 3) -> CSR:
    return stencil3d(160, 160, 160, noise=0.01, seed=seed)


WORKLOADS = {"stencil5_256": stencil5_256, "powerlaw_4m": powerlaw_4m,
             "stencil27_160": stencil27_160}


# --- the batched workload: many matrices of uneven size from a mix of generators -----------
BATCH_KINDS = ("stencil2d", "stencil3d", "powerlaw", "density", "blockdiag")


def batch_member(m_target: int, kind: str, seed: int) -> CSR:
    """One square matrix of about m_target rows from the named generator."""
    if kind == "stencil2d":
        nx = max(1, int(round(m_target ** 0.5)))
        return stencil2d(nx, max(1, int(round(m_target / nx))), seed=seed)
    if kind == "stencil3d":
        nx = max(1, int(round(m_target ** (1.0 / 3.0))))
        ny = nx
        return stencil3d(nx, ny, max(1, int(round(m_target / (nx * ny)))), seed=seed)
    if kind == "powerlaw":
        return powerlaw(m_target, seed=seed)
    if kind == "density":
        return density(m_target, m_target, 1e-4, seed=seed)
    if kind == "blockdiag":
        return blockdiag(m_target, m_target, 32, seed=seed)
    raise ValueError(kind)


def batch_workload(count: int = 512, m_lo: int = 1_000, m_hi: int = 200_000, seed: int = 4,
                   kinds=BATCH_KINDS) -> list:
    """`count` matrices with row counts log-uniform in [m_lo, m_hi], each drawn from a seeded
    mix of generators (2D/3D stencil, power-law rows, uniform density 1e-4, block-diagonal
    32x32 dense blocks)."""
    u = uniform(2 * count, seed, 0.0, 1.0)
    mats = []
    for i in range(count):
        m = int(round(np.exp(np.log(m_lo) + u[2 * i] * (np.log(m_hi) - np.log(m_lo)))))
        kind = kinds[min(int(u[2 * i + 1] * len(kinds)), len(kinds) - 1)]
        a = batch_member(m, kind, seed * 100_003 + i)
        a.name = f"{kind}_{a.m}"
        mats.append(a)
    return mats
