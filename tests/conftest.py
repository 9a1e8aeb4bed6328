"""Shared pytest configuration: the `gpu` marker and fixture loaders."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_cases(name):
    """Load tests/golden/<name>.npz as a list of per-case dicts."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    count = int(z["count"])
    cases = [dict() for _ in range(count)]
    for key in z.files:
        if key == "count":
            continue
        idx, field = key[1:].split("_", 1)
        cases[int(idx)][field] = z[key]
    return cases


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:  # pragma: no cover
        return False
