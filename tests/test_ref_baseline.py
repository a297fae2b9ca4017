"""The CPU baseline's slab runner computes the global problem.

oracle/ref_baseline.py runs the reference's generated Cython kernel on one
x-slab per process and exchanges the x faces between slabs every step, as
pylbm's MPI ranks do (pylbm/storage.py:307-367).  Four slabs of the 16^3
Taylor-Green vortex after 20 steps reproduce the reference pylbm's own
single-process run (tests/golden/tgv3d_n16.npz).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def test_four_slabs_reproduce_the_reference_run():
    import ref_baseline

    if not ref_baseline.reference_available():
        pytest.skip("oracle/_ref (the reference's generated kernel) is not built here")
    gold = np.load(os.path.join(ROOT, "tests", "golden", "tgv3d_n16.npz"))
    _, _, f = ref_baseline.run_slabs(n=16, steps=19, procs=4, keep_state=True)
    m = np.einsum("ij,xyzj->ixyz", gold["M"], f)
    ref = gold["m20"]
    err = np.abs(m - ref).reshape(19, -1).max(1) / np.abs(ref).reshape(19, -1).max(1).max()
    assert err.max() < 1e-13, err
