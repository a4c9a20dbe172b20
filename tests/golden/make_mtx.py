"""Writes the Matrix Market fixtures of tests/golden/mtx/ (deterministic; rerun to regenerate).

Each file exercises one part of the reference driver's loader (spmv_cuda/main.cu:570-733 with
the NIST reader of spmv_cuda/mmio.h): fields, symmetry kinds, comments, blank lines, case,
CRLF line ends, entry order, and the failure points.  The expected CSR of the valid files is
the oracle restatement's (oracle/mtx_oracle.py), itself pinned by the known answers in
tests/test_mtx_cpu.py and, where the reference tree is present, by the reference's own
banner and size readers (oracle/mtx_ref.c).
"""
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mtx")


def write(name, text):
    with open(os.path.join(HERE, name), "w", newline="") as fh:
        fh.write(text)


def entries(rows, cols, vals=None, fmt="{:.17g}"):
    out = []
    for k, (r, c) in enumerate(zip(rows, cols)):
        out.append(f"{r + 1} {c + 1}" + ("" if vals is None else " " + fmt.format(vals[k])))
    return "\n".join(out) + "\n"


def main():
    os.makedirs(HERE, exist_ok=True)
    # 1. the reference's 6x6 known answer (main.cu:449-451), row-major entries
    rp = [0, 3, 9, 11, 11, 12, 15]
    col = [0, 2, 5, 0, 1, 2, 3, 4, 5, 2, 4, 4, 2, 3, 4]
    rows = [r for r in range(6) for _ in range(rp[r + 1] - rp[r])]
    write("known6_general_real.mtx", "%%MatrixMarket matrix coordinate real general\n"
          "% the 6x6 known-answer matrix\n6 6 15\n" + entries(rows, col, list(range(1, 16))))
    rng = np.random.default_rng(7)
    # 2. shuffled general real, upper-case tokens, comments and a blank line before the size
    m, n, k = 40, 30, 180
    flat = rng.choice(m * n, k, replace=False)
    r, c = flat // n, flat % n
    v = rng.uniform(-1e3, 1e3, k)
    write("general_real_shuffled.mtx", "%%MatrixMarket MATRIX Coordinate REAL General\n"
          "%comment one\n% comment two\n\n" + f"{m} {n} {k}\n" + entries(r, c, v))
    # 3. integer field with negative values, tab separated
    m, n, k = 17, 23, 60
    flat = rng.choice(m * n, k, replace=False)
    r, c = flat // n, flat % n
    iv = rng.integers(-50, 50, k)
    write("general_integer.mtx", "%%MatrixMarket matrix coordinate integer general\n"
          f"{m}\t{n}\t{k}\n" + "".join(f"{a + 1}\t{b + 1}\t{x}\n" for a, b, x in zip(r, c, iv)))
    # 4. pattern field (values 1.0), with empty rows and columns
    m, n, k = 25, 25, 40
    flat = rng.choice(12 * 25, k, replace=False)
    r, c = 2 * (flat // 25), flat % 25
    write("general_pattern.mtx", "%%MatrixMarket matrix coordinate pattern general\n"
          f"{m} {n} {k}\n" + entries(r, c))
    # 5. symmetric real: lower triangle with diagonal, scientific notation, CRLF line ends
    m = 20
    pairs = sorted({(int(a), int(b)) for a, b in rng.integers(0, m, (70, 2)) if a >= b})
    r = [p[0] for p in pairs]
    c = [p[1] for p in pairs]
    v = rng.uniform(-5, 5, len(pairs))
    body = entries(r, c, v, fmt="{:.6e}").replace("\n", "\r\n")
    write("symmetric_real_crlf.mtx", "%%MatrixMarket matrix coordinate real symmetric\r\n"
          f"{m} {m} {len(pairs)}\r\n" + body)
    # 6. hermitian banner with a real field (mirrored like symmetric)
    write("hermitian_real.mtx", "%%MatrixMarket matrix coordinate real hermitian\n"
          "3 3 4\n1 1 2.5\n2 1 -1\n3 2 4\n3 3 1\n")
    # 7. skew-symmetric: loaded as stored, unmirrored
    write("skew_real.mtx", "%%MatrixMarket matrix coordinate real skew-symmetric\n"
          "4 4 3\n2 1 1.5\n3 1 -2\n4 3 0.25\n")
    # 8. symmetric pattern
    write("symmetric_pattern.mtx", "%%MatrixMarket matrix coordinate pattern symmetric\n"
          "5 5 6\n1 1\n3 1\n5 2\n4 4\n5 4\n5 5\n")
    # 9. no entries
    write("empty.mtx", "%%MatrixMarket matrix coordinate real general\n3 4 0\n")
    # 10. rectangular, entries unsorted within rows, duplicate coordinates kept
    write("rect_dups.mtx", "%%MatrixMarket matrix coordinate real general\n"
          "3 5 6\n2 5 1\n2 1 2\n1 3 3\n2 5 4\n3 2 5\n1 1 6\n")
    # failure points
    write("err_complex.mtx", "%%MatrixMarket matrix coordinate complex general\n2 2 1\n1 1 1 0\n")
    write("err_array.mtx", "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n")
    write("err_banner_prefix.mtx", "%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1\n")
    write("err_banner_short.mtx", "%%MatrixMarket matrix coordinate real\n2 2 1\n1 1 1\n")
    write("err_banner_field.mtx", "%%MatrixMarket matrix coordinate quaternion general\n"
          "2 2 1\n1 1 1\n")
    write("err_no_size.mtx", "%%MatrixMarket matrix coordinate real general\n% only comments\n")
    write("err_index.mtx", "%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1\n4 1 2\n")
    write("err_zero_index.mtx", "%%MatrixMarket matrix coordinate real general\n3 3 1\n0 1 1\n")
    write("err_truncated.mtx", "%%MatrixMarket matrix coordinate real general\n3 3 3\n1 1 1\n"
          "2 2 2\n")
    write("err_value.mtx", "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 abc\n")


if __name__ == "__main__":
    main()
