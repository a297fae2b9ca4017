"""pylbm's own golden demo results through generator='cuda' (float64 on the GPU).

Same fixtures and tolerance as test_demo_goldens.py (the CPU oracle); the GPU
run must also stay within round-off of the oracle on every moment.
"""
import numpy as np
import pytest

import demo_cases
from conftest import golden, rel_err
from oracle import OracleSimulation
from pylbm_gb300 import Simulation
from test_demo_goldens import assert_golden, conserved_fields

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", list(demo_cases.CASES))
def test_cuda_reproduces_reference_golden(name):
    build, final_time, _, fields = demo_cases.CASES[name]
    g = golden(f"demo_{name}.npz")
    sim = Simulation(build())
    demo_cases.run_to(sim, final_time)
    assert sim.nt == int(g["steps"])
    m = np.array([sim.m[k] for k in range(sim.scheme.nv)])
    assert_golden(conserved_fields(sim, m, fields, g["mask"]), g, fields)
    # the float64 parity form rounds constants to pylbm's printed 15-16
    # digits where the oracle keeps exact float64 matrices: ~1e-11 after the
    # 51 steps at la = 10 of the Orszag-Tang case
    o = OracleSimulation(build())
    demo_cases.run_to(o, final_time)
    assert rel_err(m, o.moments()).max() < 1e-10
    sim.free()


def test_h5_output_matches_reference_golden_file(tmp_path):
    """sim.write_h5 (one device-to-host copy of the conserved moments) gives
    the fields of pylbm's own golden HDF5 file for the Poiseuille demo."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import h5lite

    build, final_time, _, fields = demo_cases.CASES["poiseuille"]
    g = golden("demo_poiseuille.npz")
    sim = Simulation(build())
    demo_cases.run_to(sim, final_time)
    sim.write_h5("poiseuille", str(tmp_path))
    back = h5lite.read(str(tmp_path / "poiseuille.h5"))
    assert np.array_equal(back["x_0"], sim.domain.coords[0]) and np.array_equal(back["x_1"], sim.domain.coords[1])
    for key, cons in fields.items():
        ref = g[key]
        diff = np.abs(back[cons].T - ref)
        assert np.all(diff <= np.maximum(1e-14 * np.abs(ref), 1e-7)), key
    assert (tmp_path / "poiseuille.xdmf").exists()
    sim.free()


@pytest.mark.parametrize("name", ["karman_vortex_street", "poiseuille", "air_conditioning", "poiseuille_3d",
                                  "karman_3d", "poiseuille_vec"])
def test_batched_boundary_launch_equals_per_method(name):
    """All boundary methods in one launch give the per-method result bit for bit."""
    build, final_time, _, fields = demo_cases.CASES[name]
    out = []
    for batch in (True, False):
        sim = Simulation(build())
        sim.batch_boundary = batch
        sim.run(20)
        out.append(np.array([sim.m[k] for k in range(sim.scheme.nv)]))
        batched = sim._bc_batch is not None
        sim.free()
    assert np.array_equal(out[0], out[1])
    if name == "karman_vortex_street":
        # the outflow's corner links read wall ghosts the Bouzidi method writes:
        # they take the Bouzidi formula of those slots inside the one launch
        assert batched


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_batched_boundary_launch_disc_flow(dtype):
    """Disc, inflow and outflow of the channel periodic in y: one launch, the
    per-method result (FP64: bit for bit; FP32: the batch computes on the
    stored deviations in FP32, the per-method kernels in FP64)."""
    from pylbm_gb300 import workloads as W
    d = W.cylinder(nx=192, ny=64, radius=8, center=(48, 33), re=80.0)
    out = []
    for batch in (True, False):
        sim = Simulation(d, dtype=dtype)
        sim.batch_boundary = batch
        sim.run(30)
        out.append(np.array([sim.m[k] for k in range(sim.scheme.nv)]))
        assert sim._bc_batch is not None
        sim.free()
    if dtype == "float64":
        assert np.array_equal(out[0], out[1])
    else:
        for k in range(3):
            assert np.abs(out[0][k] - out[1][k]).max() <= 2e-6 * np.abs(out[1][k]).max()
