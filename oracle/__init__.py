"""CPU oracle for the speculative segmented-sum CSR SpMV (test infrastructure).

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may use this package, and only as the checker or the timed CPU
baseline.  The product library never imports it.
"""
from .oracle import *  # noqa: F401,F403
