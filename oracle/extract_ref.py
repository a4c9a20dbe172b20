"""Build step: cut the reference's own host loops out of its sources into oracle/_ref/.

Three regions of plain C++ in the reference are the CPU side of the path.  This script finds
each by its anchor lines (not by line numbers), brace-matches the block and writes it verbatim
into oracle/_ref/ (git-ignored build output), with a first comment line naming the file and
lines it came from.  oracle/ref_harness.cpp then compiles the blocks inside functions whose
parameters carry the names the blocks use, so the compiled code is the reference's own:

* calib.inc  -- spmv_cuda/bhsparse_spmv_cuda.h, run_benchmark's host steps after the kernel:
                the inter-warp calibration loop and the speculative fix-up of dirty tiles
                (from "for (int i = 0; i < _threadbunch_num; i++)" up to "return err;");
* serial.inc -- spmv_cuda/main.cu, the serial CSR loop that gives y_ref
                (the "for (int iter = 0; iter < ref_iter; iter++)" block);
* omp.inc    -- spmv_cuda/main.cu, the OpenMP CSR loop
                (the "for (int iter = 0; iter < NUM_RUN; iter++)" block).

Usage:  python oracle/extract_ref.py REFERENCE_TREE OUT_DIR
(oracle/Makefile's ``ref`` target runs it when the reference tree is present).
"""
from __future__ import annotations

import os
import sys


def _find(lines, needle, start=0):
    for i in range(start, len(lines)):
        if needle in lines[i]:
            return i
    raise SystemExit(f"anchor not found: {needle!r}")


def _block(lines, first):
    """Lines [first, end] of the statement starting at `first` whose braces balance at `end`."""
    depth, opened = 0, False
    for i in range(first, len(lines)):
        depth += lines[i].count("{") - lines[i].count("}")
        opened = opened or "{" in lines[i]
        if opened and depth == 0:
            return first, i
    raise SystemExit(f"unbalanced block at line {first + 1}")


def _write(out_dir, name, rel, lines, a, b):
    with open(os.path.join(out_dir, name), "w") as f:
        f.write(f"// extracted from {rel} lines {a + 1}-{b + 1} (build output, not committed)\n")
        f.write(f"#line {a + 1} \"{rel}\"\n")
        f.writelines(lines[a:b + 1])


def main(ref: str, out_dir: str) -> None:
    os.makedirs(out_dir, exist_ok=True)
    rel = "spmv_cuda/bhsparse_spmv_cuda.h"
    with open(os.path.join(ref, rel)) as f:
        h = f.readlines()
    run = _find(h, "int bhsparse_spmv_cuda::run_benchmark()")
    a = _find(h, "for (int i = 0; i < _threadbunch_num; i++)", run)
    b = _find(h, "return err;", a) - 1
    _write(out_dir, "calib.inc", rel, h, a, b)

    rel = "spmv_cuda/main.cu"
    with open(os.path.join(ref, rel)) as f:
        m = f.readlines()
    a = _find(m, "for (int iter = 0; iter < ref_iter; iter++)")
    a, b = _block(m, a)
    _write(out_dir, "serial.inc", rel, m, a, b)
    a = _find(m, "for (int iter = 0; iter < NUM_RUN; iter++)")
    a, b = _block(m, a)
    _write(out_dir, "omp.inc", rel, m, a, b)


if __name__ == "__main__":
    if len(sys.argv) != 3:
        raise SystemExit(__doc__)
    main(sys.argv[1], sys.argv[2])
