"""Regenerate the golden fixtures under tests/golden/.

known_6x6.json
    The reference's only known-answer case, the 6x6 matrix of
    spmv_cuda/main.cu:449-451 (row_ptr, col_idx, val = 1..15) with x = 1
    (main.cu:472-474).  When the reference tree is given (first argument, or the
    REFERENCE_ROOT environment variable) the arrays are parsed from its main.cu; otherwise
    the committed copy is reused.  Expected y, tile_ptr and bit-flag words are computed here by a
    pure-Python restatement of the reference formulas (independent of oracle/oracle.c):
      * y: the serial loop, main.cu:480-486;
      * tile_ptr: binary_search_right_boundary_kernel (utils_cuda.h:6-31) at every tile
        boundary (kernels_cuda.h:43-49), bit 31 = dirty (kernels_cuda.h:119-145);
      * bit flags: kernels_cuda.h:116-143.

cases.npz
    Small seeded integer-valued CSR matrices that exercise the edge cases of the path
    (empty rows at the start / middle / end, all-empty, rows longer than a tile, nnz a
    multiple of the tile, single row, single non-zero), with the same pure-Python
    expected outputs at geometries 32x4, 32x8, 32x16 and 32x32.  Integer data keep every
    partial sum exact, so y is compared bit for bit (the reference's own check,
    main.cu:789-806).

Run:  python tests/golden/make_golden.py [REFERENCE_TREE]
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFERENCE_ROOT", "")
GEOMS = (4, 8, 16, 32)


def search_right(row_ptr, key):
    start, stop = 0, len(row_ptr) - 1
    while stop >= start:
        med = (stop + start) // 2
        if key >= row_ptr[med]:
            start = med + 1
        else:
            stop = med - 1
    return start


def partition(row_ptr, nnz, ps):
    m = len(row_ptr) - 1
    nt = (nnz + ps - 1) // ps
    tp = [search_right(row_ptr, min(t * ps, nnz)) - 1 for t in range(nt + 1)]
    out = []
    for t in range(nt + 1):
        v = tp[t]
        if t < nt and tp[t] != tp[t + 1]:
            stop = m - 1 if tp[t + 1] == m else tp[t + 1]
            if any(row_ptr[r] == row_ptr[r + 1] for r in range(tp[t], stop + 1)):
                v |= 0x80000000
        out.append(v)
    return out


def bitflags(row_ptr, nnz, seg, tile_ptr):
    m = len(row_ptr) - 1
    ps = 32 * seg
    words = []
    for t in range(len(tile_ptr) - 1):
        lo, hi = tile_ptr[t] & 0x7FFFFFFF, tile_ptr[t + 1] & 0x7FFFFFFF
        w = [0] * 32
        stop = m - 1 if hi == m else hi
        for r in range(lo, stop + 1):
            if row_ptr[r] == row_ptr[r + 1]:
                continue
            off = row_ptr[r] - t * ps
            if 0 <= off < ps:
                w[off // seg] |= 1 << (31 - off % seg)
        words.append(w)
    return words


def serial_y(row_ptr, col, val, x):
    return [sum(x[col[j]] * val[j] for j in range(row_ptr[i], row_ptr[i + 1]))
            for i in range(len(row_ptr) - 1)]


def parse_known_6x6():
    path = os.path.join(REF, "spmv_cuda", "main.cu")
    if not os.path.exists(path):
        with open(os.path.join(HERE, "known_6x6.json")) as f:
            d = json.load(f)
        return d["row_ptr"], d["col_idx"], d["val"], d["source"]
    src = open(path).read()

    def arr(name):
        mt = re.search(name + r"\[\d+\]\s*=\s*\{([^}]*)\}", src)
        return [float(v) if "." in v else int(v) for v in mt.group(1).replace(" ", "").split(",")]

    return (arr("row_ptr"), arr("col_idx"), [float(v) for v in arr("val")],
            "spmv_cuda/main.cu:449-451 (arrays), :472-474 (x = 1)")


def known_case():
    rp, ci, va, src = parse_known_6x6()
    m = len(rp) - 1
    x = [1.0] * m
    d = {"source": src, "row_ptr": rp, "col_idx": ci, "val": va, "x": x,
         "y": serial_y(rp, ci, va, x)}
    for seg in GEOMS:
        tp = partition(rp, rp[-1], 32 * seg)
        d[f"tile_ptr_{seg}"] = tp
        d[f"bitflags_{seg}"] = bitflags(rp, rp[-1], seg, tp)
    return d


def random_cases():
    rng = np.random.default_rng(20240601)
    cases = []

    def add(name, lens, n):
        lens = np.asarray(lens, np.int64)
        rp = np.zeros(lens.size + 1, np.int64)
        rp[1:] = np.cumsum(lens)
        nnz = int(rp[-1])
        col = np.concatenate([np.sort(rng.choice(n, int(l), replace=False)) if l else
                              np.zeros(0, np.int64) for l in lens]) if nnz else np.zeros(0, np.int64)
        val = rng.integers(-9, 10, nnz).astype(np.float64)
        x = rng.integers(-9, 10, n).astype(np.float64)
        cases.append((name, rp.astype(np.int32), col.astype(np.int32), val, x))

    add("leading_empty", [0, 0, 0] + list(rng.integers(1, 20, 60)), 200)
    add("trailing_empty", list(rng.integers(1, 20, 60)) + [0] * 5, 200)
    lens = rng.integers(0, 12, 400)
    lens[rng.random(400) < 0.3] = 0
    add("scattered_empty", lens, 300)
    add("all_empty", [0] * 17, 5)
    add("single_row_long", [3000], 4000)
    add("one_nnz", [0, 1, 0], 3)
    add("exact_tiles", [128] * 8, 512)
    add("long_rows_mixed", [1, 700, 2, 0, 0, 1500, 3, 0, 40] * 3, 2000)
    add("short_rows", [1] * 1100 + [2] * 300, 50)
    add("ninety_pct_empty", np.where(rng.random(3000) < 0.9, 0, rng.integers(1, 30, 3000)), 500)
    return cases


def main():
    d = known_case()
    with open(os.path.join(HERE, "known_6x6.json"), "w") as f:
        json.dump(d, f, indent=1)
    arrays = {}
    names = []
    for name, rp, col, val, x in random_cases():
        names.append(name)
        nnz = int(rp[-1])
        arrays[f"{name}.row_ptr"] = rp
        arrays[f"{name}.col"] = col
        arrays[f"{name}.val"] = val
        arrays[f"{name}.x"] = x
        arrays[f"{name}.y"] = np.array(serial_y(rp.tolist(), col.tolist(), val.tolist(), x.tolist()),
                                       np.float64)
        for seg in GEOMS:
            tp = partition(rp.tolist(), nnz, 32 * seg)
            arrays[f"{name}.tile_ptr_{seg}"] = np.array(tp, np.uint32)
            arrays[f"{name}.bitflags_{seg}"] = np.array(bitflags(rp.tolist(), nnz, seg, tp),
                                                        np.uint32).reshape(-1, 32)
    arrays["names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "cases.npz"), **arrays)
    print("wrote", len(names), "cases and known_6x6.json")


if __name__ == "__main__":
    main()
