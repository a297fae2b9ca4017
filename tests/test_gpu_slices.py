"""Device-side slices: ``sim.m[key, i0, ...]`` and ``sim.F[k, ...]`` copy
only the selected nodes (lbm_gather) and equal numpy indexing of the full
field bit for bit."""
import numpy as np
import pytest

from pylbm_gb300 import Simulation
from pylbm_gb300 import workloads as W

pytestmark = pytest.mark.gpu

INDEX_2D = [(slice(None), 5), (slice(3, 40, 3), slice(None)), (-1, slice(None, None, -2)), (7, 9),
            (slice(10, 2, -3), slice(1, 60, 7))]
INDEX_3D = [(slice(None), slice(None), 8), (4, slice(2, 14, 5), -3), (slice(None, None, -1), 0, slice(None))]


@pytest.mark.parametrize("dtype", ["float64", "float32", "bfloat16"])
def test_moment_and_population_slices_2d(dtype):
    sim = Simulation(W.cylinder(nx=96, ny=64, radius=5, center=(24, 33), re=40.0), dtype=dtype)
    sim.run(7)
    for key in (W.RHO, W.QX, 4):
        full = sim.m[key]
        for ix in INDEX_2D:
            assert np.array_equal(sim.m[(key,) + ix], full[ix])
    for k in (0, 5, 8):
        full = sim.F[k]
        for ix in INDEX_2D:
            assert np.array_equal(sim.F[(k,) + ix], full[ix])
    sim.free()


def test_slices_3d():
    sim = Simulation(W.tgv3d(n=16), dtype="float32")
    sim.run(3)
    for key in (W.RHO, W.QZ):
        full = sim.m[key]
        for ix in INDEX_3D:
            assert np.array_equal(sim.m[(key,) + ix], full[ix])
    with pytest.raises(IndexError):
        sim.m[W.RHO, 16, 0, 0]
    sim.free()
