"""pylbm's own Simulation with generator='cuda' on the GPU (pylbm_gb300.plugin).

The same two runs as tests/test_pylbm_plugin.py -- pylbm's classes driving
the backend through ``call_genfunction`` -- with the CUDA device itself:
the 32^2 cavity after 300 steps against the reference's own Cython run
(bit for bit: the module computes the reference generator's printed forms,
and pylbm's boundary right-hand sides come from the module's equilibrium
and m2f on the GPU), and pylbm's Poiseuille demo (Bouzidi, NeumannX)
against pylbm's own golden result.  Skipped where the reference sources are
not present (they are not shipped with this package).
"""
import numpy as np
import pytest
import sympy as sp

import demo_cases
from conftest import golden, rel_err
from pylbm_gb300 import workloads as W
from test_pylbm_plugin import reference_pylbm

pytestmark = pytest.mark.gpu


@pytest.fixture()
def cuda_pylbm():
    from pylbm_gb300 import plugin

    pylbm = reference_pylbm()
    plugin.install(pylbm, device=plugin.CudaDevice)
    return pylbm


def test_pylbm_simulation_cavity_on_the_gpu_matches_reference(cuda_pylbm):
    pylbm = cuda_pylbm
    d = W.cavity(n=32, bc=pylbm.bc)
    d["generator"] = "cuda"
    sim = pylbm.Simulation(d)
    assert type(sim.container.F.array).__name__ == "DeviceArray"
    for _ in range(300):
        sim.one_time_step()
    m = np.array([np.array(sim.m[k]) for k in range(9)])
    assert rel_err(m, golden("cavity_n32.npz")["m300"]).max() <= 1e-14


def test_pylbm_simulation_poiseuille_on_the_gpu_matches_golden(cuda_pylbm):
    pylbm = cuda_pylbm
    build, final_time, _, fields = demo_cases.CASES["poiseuille"]
    d = build(bc=pylbm.bc)
    d["generator"] = "cuda"
    sim = pylbm.Simulation(d)
    demo_cases.run_to(sim, final_time)
    g = golden("demo_poiseuille.npz")
    assert sim.nt == int(g["steps"])
    mask = sim.domain.in_or_out[1:-1, 1:-1] == sim.domain.valin
    vals = {}
    for key, cons in fields.items():
        v = np.array(sim.m[sp.Symbol(cons)], dtype=np.float64)
        v[~mask] = 0.0
        vals[key] = v
    from test_demo_goldens import assert_golden
    assert_golden(vals, g, fields)
