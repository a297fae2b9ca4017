"""Bounce-back box walls folded into the step (lbm_one_time_step_walls).

On the lid-driven cavity and cube every boundary link is a bounce-back link
of a box wall; the step applies them in its pull, in one launch, and must
give the populations of the boundary launch followed by the step bit for bit
in every storage type (the folded value is rounded through the storage type
as the ghost store rounds it).
"""
import numpy as np
import pytest

from pylbm_gb300 import Simulation
from pylbm_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", ["float64", "float32", "float16", "bfloat16"])
@pytest.mark.parametrize("case", ["cavity", "cube", "cube_odd"])
def test_folded_walls_equal_boundary_launch(case, dtype):
    make = {"cavity": lambda: W.cavity(n=64), "cube": lambda: W.cavity3d(n=24),
            "cube_odd": lambda: W.cavity3d(n=17)}[case]
    out = []
    for fold in (True, False):
        sim = Simulation(make(), dtype=dtype)
        assert sim._walls is not None
        assert sim.fold_walls  # the default
        sim.fold_walls = fold
        assert sim.launches_per_step() == (1 if fold else 2)
        sim.run(25)
        sim.one_time_step()
        out.append(np.array([sim.F[k] for k in range(sim.scheme.nv)]))
        sim.free()
    assert np.all(np.isfinite(out[0]))
    assert np.array_equal(out[0], out[1])


def test_bounded_flows_with_other_methods_keep_the_boundary_launch():
    for d in (W.cylinder(nx=192, ny=64, radius=8, center=(48, 33), re=80.0), W.karman(dx=1.0 / 32)):
        sim = Simulation(d, dtype="float32")
        assert sim._walls is None and sim.launches_per_step() == 2
        sim.free()
