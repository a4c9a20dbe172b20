"""CPU restatement of the reference driver's Matrix Market loading (test infrastructure).

Only the tests use this module: it is the checker for the library's native loader
(include/spmv_mtx.h), never a product path.  Pure Python, for small files.

It follows:
  * mm_read_banner, spmv_cuda/mmio.h:249-330 -- five tokens, a "%%MatrixMarket" prefix, the
    other four tokens compared case-insensitively;
  * mm_read_mtx_crd_size, spmv_cuda/mmio.h:334-361 -- '%' lines skipped, then three integers
    (a blank line defers them to the following tokens);
  * the loader of spmv_cuda/main.cu:570-733 -- complex refused (:591-595); real / integer /
    pattern entries (:629-648, pattern value 1.0); 1-based to 0-based (:650-653); symmetric and
    hermitian files mirrored (:606-612, :661-668, :690-716); row counts, an exclusive scan
    (:670-681) and a stable placement in file order (:690-725).
The status codes are those of include/spmv_mtx.h.  Where the reference has no defined
behaviour (indices out of range, a truncated entry list, array storage, a size line with fewer
than three integers) the restatement returns the library's error status for it.
"""
from __future__ import annotations

import numpy as np

OK, OPEN_FAILED, BAD_BANNER, COMPLEX, BAD_SIZE, UNSUPPORTED, BAD_ENTRY, TOO_LARGE = (
    0, -1, -2, -3, -4, -5, -6, -7)


def read_banner(line: str):
    """(status, storage, field, symmetry) from the first line (mmio.h:249-330)."""
    t = line.split()
    if len(t) < 5:
        return BAD_BANNER, None, None, None
    banner, mtx, crd, data, sym = t[0], t[1].lower(), t[2].lower(), t[3].lower(), t[4].lower()
    if not banner.startswith("%%MatrixMarket"):
        return BAD_BANNER, None, None, None
    if mtx != "matrix" or crd not in ("coordinate", "array"):
        return BAD_BANNER, None, None, None
    if data not in ("real", "complex", "pattern", "integer"):
        return BAD_BANNER, None, None, None
    if sym not in ("general", "symmetric", "hermitian", "skew-symmetric"):
        return BAD_BANNER, None, None, None
    return OK, crd, data, sym


def load(path: str):
    """Return (status, dict) with m, n, nnz_file, row_ptr, col, val, field, symmetry."""
    try:
        with open(path, "rb") as fh:
            text = fh.read().decode("latin-1")
    except OSError:
        return OPEN_FAILED, None
    lines = text.split("\n")
    st, crd, data, sym = read_banner(lines[0]) if lines else (BAD_BANNER, None, None, None)
    if st != OK:
        return st, None
    if data == "complex":
        return COMPLEX, None
    if crd == "array":
        return UNSUPPORTED, None
    i = 1
    while True:
        if i >= len(lines) or (i == len(lines) - 1 and lines[i] == ""):
            return BAD_SIZE, None
        ln = lines[i]
        i += 1
        if ln.startswith("%"):
            continue
        t = ln.split()
        if not t:
            continue
        if len(t) < 3:
            return BAD_SIZE, None
        try:
            m, n, nzf = int(t[0]), int(t[1]), int(t[2])
        except ValueError:
            return BAD_SIZE, None
        break
    toks = "\n".join(lines[i:]).split()
    per = 2 if data == "pattern" else 3
    if len(toks) < per * nzf:
        return BAD_ENTRY, None
    mirror = sym in ("symmetric", "hermitian")
    rows, cols, vals = [], [], []
    for e in range(nzf):
        tk = toks[per * e:per * e + per]
        try:
            r, c = int(tk[0]), int(tk[1])
            if data == "real":
                v = float(tk[2])
            elif data == "integer":
                v = float(int(tk[2]))
            else:
                v = 1.0
        except ValueError:
            return BAD_ENTRY, None
        if not (1 <= r <= m and 1 <= c <= n):
            return BAD_ENTRY, None
        if mirror and r != c and (c > m or r > n):
            return BAD_ENTRY, None
        rows.append(r - 1)
        cols.append(c - 1)
        vals.append(v)
    # row counts, exclusive scan, stable placement (main.cu:618-716)
    counter = [0] * (m + 1)
    for e in range(nzf):
        counter[rows[e]] += 1
    if mirror:
        for e in range(nzf):
            if rows[e] != cols[e]:
                counter[cols[e]] += 1
    row_ptr = [0] * (m + 1)
    acc = 0
    for r in range(m + 1):
        row_ptr[r] = acc
        acc += counter[r]
    nnz = row_ptr[m] + counter[m]
    if nnz > 2**31 - 1:
        return TOO_LARGE, None
    col = [0] * nnz
    val = [0.0] * nnz
    fill = [0] * (m + 1)
    for e in range(nzf):
        r, c, v = rows[e], cols[e], vals[e]
        o = row_ptr[r] + fill[r]
        col[o], val[o] = c, v
        fill[r] += 1
        if mirror and r != c:
            o = row_ptr[c] + fill[c]
            col[o], val[o] = r, v
            fill[c] += 1
    return OK, {"m": m, "n": n, "nnz_file": nzf, "field": data, "symmetry": sym,
                "row_ptr": np.array(row_ptr, np.int32), "col": np.array(col, np.int32),
                "val": np.array(val, np.float64)}
