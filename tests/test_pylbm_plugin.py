"""pylbm's own Simulation with generator='cuda' (pylbm_gb300.plugin).

The reference package is imported from its sources (with the import shims of
oracle/shims) and ``plugin.install`` adds the backend without editing it.
pylbm's own classes then run: ``Simulation.__init__`` builds a CudaContainer,
the boundary methods compute their right-hand sides through the module's
``equilibrium`` and ``m2f``, ``move2gpu`` uploads the lists,
``one_time_step`` calls ``Array.update`` (update_x/_y) and each method's
``update`` through ``call_genfunction``, and ``sim.m[...]`` reads through
``f2m``.

Here (no GPU) the device is tests/host_device.py: the same routine names and
parameter names as the CUDA module, computed by the C oracle, every call
recorded.  The GPU test (tests/test_gpu_pylbm_plugin.py) runs the CUDA
device itself.  Cases: the 32^2 cavity (bounce-back walls and lid) after
300 steps against the reference's own Cython run (tests/golden/cavity_n32.npz),
and pylbm's Poiseuille demo (Bouzidi walls and inflow, NeumannX outflow)
against pylbm's own golden result.
"""
import os
import sys

import numpy as np
import pytest
import sympy as sp

import demo_cases
from conftest import ROOT, golden, rel_err
from pylbm_gb300 import workloads as W
from pylbm_gb300.generator import routine_signatures


def reference_pylbm():
    """The reference package, imported from $PYLBM_REFERENCE (default: a
    'reference' folder beside this repository); skip when absent."""
    ref = os.environ.get("PYLBM_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
    if not os.path.isfile(os.path.join(ref, "pylbm", "__init__.py")):
        pytest.skip("the reference pylbm sources are not present on this machine")
    sys.dont_write_bytecode = True  # nothing is written into the reference tree
    for p in (ref, os.path.join(ROOT, "oracle", "shims")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import pylbm
    return pylbm


@pytest.fixture()
def host_pylbm():
    from host_device import HostDevice
    from pylbm_gb300 import plugin

    pylbm = reference_pylbm()
    device = HostDevice()
    plugin.install(pylbm, device=device)
    return pylbm, device


def _moments(sim, nv):
    return np.array([np.array(sim.m[k]) for k in range(nv)])


def test_pylbm_simulation_runs_the_cavity_through_the_plugin(host_pylbm):
    pylbm, device = host_pylbm
    d = W.cavity(n=32, bc=pylbm.bc)
    d["generator"] = "cuda"
    sim = pylbm.Simulation(d)
    assert type(sim.container).__name__ == "CudaContainer"
    assert type(sim.container.F).__name__ == "CudaArray"
    assert type(sim.container.F.array).__name__ == "HostArray"
    assert all(type(m.istore).__name__ == "HostList" for m in sim.bc.methods)
    init_calls = len(device.calls)
    for _ in range(300):
        sim.one_time_step()
    m = _moments(sim, 9)
    g = golden("cavity_n32.npz")
    # the oracle computes with exact constants, the reference with printed
    # ones: the oracle's own bound against this fixture (tests/test_oracle.py)
    assert rel_err(m, g["m300"]).max() < 2e-12
    step_calls = device.calls[init_calls:]
    names = [c[0] for c in step_calls]
    # per step: pylbm's ghost refresh axis by axis, the bounce-back method
    # (walls and lid share it: pylbm groups links by method), the step
    assert len(sim.bc.methods) == 1
    assert names[:4] == ["update_x", "update_y", "bounce_back", "one_time_step"]
    assert names.count("one_time_step") == 300 and names.count("bounce_back") == 300
    assert names.count("update_x") == 300 and names.count("update_y") == 300
    # every call bound exactly the routine's parameters, by name
    sig = routine_signatures(device.modules[0].scheme)
    assert all(set(args) == set(sig[name]) for name, args in device.calls)
    # boundary right-hand sides came from the module's equilibrium and m2f
    first = [c[0] for c in device.calls[:init_calls]]
    assert "equilibrium" in first and "m2f" in first


def test_pylbm_simulation_runs_poiseuille_through_the_plugin(host_pylbm):
    pylbm, device = host_pylbm
    build, final_time, _, fields = demo_cases.CASES["poiseuille"]
    d = build(bc=pylbm.bc)
    d["generator"] = "cuda"
    sim = pylbm.Simulation(d)
    demo_cases.run_to(sim, final_time)
    g = golden("demo_poiseuille.npz")
    assert sim.nt == int(g["steps"])
    names = {c[0] for c in device.calls}
    assert {"Bouzidi_bounce_back", "neumannx", "one_time_step"} <= names
    inner = tuple(slice(1, -1) for _ in range(2))
    mask = sim.domain.in_or_out[inner] == sim.domain.valin
    vals = {}
    for key, cons in fields.items():
        v = np.array(sim.m[sp.Symbol(cons)], dtype=np.float64)
        v[~mask] = 0.0
        vals[key] = v
    from test_demo_goldens import assert_golden
    assert_golden(vals, g, fields)
