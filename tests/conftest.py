import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN) as g:
        return {k: g[k] for k in g.files}


def rel_err(a, b):
    """max |a-b| / max(|b|, tiny): error relative to the reference array's scale."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    s = np.max(np.abs(b)) if b.size else 0.0
    return float(np.max(np.abs(a - b)) / max(s, 1e-300)) if a.size else 0.0
