"""Build and run the library's hardware probes (sm_103a): ``gather_rate.cu``, the random-gather
and host-copy rates behind bench.py's sector roofline.

    python -m benchmark_spmv_using_csr_gb300.probes
"""
from __future__ import annotations

import os
import subprocess
import sys

from ..build import ARCH, BUILD, _nvcc, _stale

HERE = os.path.dirname(os.path.abspath(__file__))


def main() -> int:
    src = os.path.join(HERE, "gather_rate.cu")
    exe = os.path.join(BUILD, "gather_rate")
    os.makedirs(BUILD, exist_ok=True)
    if _stale(exe, [src]):
        cmd = [_nvcc()] + ARCH + ["-O3", "-std=c++17", src, "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            print(r.stdout + r.stderr, file=sys.stderr)
            return r.returncode
    return subprocess.run([exe]).returncode


if __name__ == "__main__":
    sys.exit(main())
