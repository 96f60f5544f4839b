import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the native library")


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN) as g:
        return {k: g[k] for k in g.files}


def rel_err(got, ref):
    """max |got - ref| / (max(ref) - min(ref)) -- the parity measure of this path."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    rng = float(ref.max() - ref.min()) if ref.size else 0.0
    d = float(np.abs(got - ref).max()) if ref.size else 0.0
    return d / rng if rng > 0 else d
