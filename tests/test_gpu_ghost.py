"""Observed ghost copies on the GPU: the same interior as pylbm's full
refresh, bit for bit, with fewer launches per step."""
import numpy as np
import pytest

import demo_cases
from pylbm_gb300 import Simulation
from pylbm_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CASES = ["poiseuille", "lid_driven_cavity", "karman_vortex_street", "air_conditioning", "rayleigh_benard",
         "poiseuille_3d", "bend", "d1q5_advection", "karman_3d"]


def interior(sim):
    return np.array([sim.F[k] for k in range(sim.scheme.nv)])


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("name", CASES)
def test_observed_ghosts_equal_full_refresh(name, dtype):
    build = demo_cases.CASES[name][0]
    out = {}
    for halo in ("full", "observed"):
        sim = Simulation(build(), dtype=dtype, halo=halo)
        sim.run(12)
        out[halo] = interior(sim)
        sim.free()
    assert np.isfinite(out["full"]).all()
    assert np.array_equal(out["full"], out["observed"])


def test_disc_flow_one_boundary_launch():
    d = W.cylinder(nx=192, ny=64, radius=8, center=(48, 33), re=80.0)
    out = {}
    for halo in ("full", "observed"):
        sim = Simulation(d, dtype="float32", halo=halo)
        sim.run(30)
        out[halo] = interior(sim)
        if halo == "observed":
            # periodic y: the copies of the two y ghost rows join the disc,
            # inflow and outflow links in one launch before the step
            assert sim._ghost is not None and sim._ghost["joined"]
            assert sim.launches_per_step() == 2
        else:
            assert sim.launches_per_step() == 3
        sim.free()
    assert np.array_equal(out["full"], out["observed"])


def test_walled_channel_drops_the_refresh():
    sim = Simulation(W.karman(dx=1.0 / 32), dtype="float32")
    assert sim._ghost is None and not sim._full_halo
    assert sim.launches_per_step() == 2  # Bouzidi and outflow in one launch, then the step
    sim.free()
