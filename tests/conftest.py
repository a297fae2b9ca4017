import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running check")


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def rel_err(a, b):
    """Per-moment max |a - b| / max |b| (the parity metric).

    Moments that vanish in exact arithmetic (|b| at round-off level, e.g. a
    z-flux of a flow without z-velocity; below 1e-6 of the largest moment)
    are measured against the largest moment instead of their own round-off.
    """
    import numpy as np
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    num = np.abs(a - b).reshape(a.shape[0], -1).max(axis=1)
    den = np.abs(b).reshape(b.shape[0], -1).max(axis=1)
    gmax = den.max()
    den = np.where(den < 1e-6 * gmax, gmax, den)
    return num / np.maximum(den, 1e-300)
