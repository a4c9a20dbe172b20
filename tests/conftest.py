"""Shared test set-up: the `gpu` marker, the repository root on sys.path, and helpers."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


GOLDEN = os.path.join(ROOT, "tests", "golden")

# Tolerances (componentwise, relative to (|A|.|x|)_i; normwise for the mixed forms)
TOL_F64 = 1e-12
TOL_F32 = 1e-5
TOL_MIXED_NORMWISE = 1e-6


def load_cases():
    d = np.load(os.path.join(GOLDEN, "cases.npz"))
    names = [str(n) for n in d["names"]]
    return d, names


@pytest.fixture(scope="session")
def golden_cases():
    return load_cases()


@pytest.fixture(scope="session")
def cuda_ok():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return True
