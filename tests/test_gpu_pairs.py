"""Two nodes per thread (16-bit storage, packed FP32x2 arithmetic).

The paired kernels evaluate the same generated algebra on two lanes; scheme
modules are compiled without implicit contraction, so every lane rounds as
the one-node kernel does and the results must be identical bit for bit.
"""
import numpy as np
import pytest
import sympy as sp

import demo_cases
from pylbm_gb300 import Simulation
from pylbm_gb300 import workloads as W
from pylbm_gb300.ensemble import Ensemble

pytestmark = pytest.mark.gpu

OMEGA = sp.Symbol("omega")


def _moments(sim):
    return np.array([sim.m[k] for k in range(sim.scheme.nv)])


def _both(dico, dtype, steps):
    out = []
    for pairs in (True, False):
        sim = Simulation(dico, dtype=dtype, node_pairs=pairs)
        sim.run(steps)
        out.append(_moments(sim))
        sim.free()
    return out


@pytest.mark.parametrize("dtype", ["float16", "bfloat16"])
def test_pairs_equal_single_nodes_d3q19(dtype):
    a, b = _both(W.tgv3d(n=32), dtype, 30)
    assert np.array_equal(a, b)
    assert np.all(np.isfinite(a))


@pytest.mark.parametrize("n", [64, 66, 33])
def test_pairs_equal_single_nodes_d2q9(n):
    """Even rows use the paired kernel (66: row length not a multiple of 4); odd rows fall back."""
    a, b = _both(W.shear_layer(n=n, nu=1e-3), "float16", 40)
    assert np.array_equal(a, b)


def test_ensemble_pairs_equal_single_nodes():
    sides = [32, 33, 64, 50, 96]
    nus = [1e-3, 5e-2, 2e-3, 5e-4, 1e-2]
    dicos = [W.shear_layer(n=s, omega=OMEGA, seed=i) for i, s in enumerate(sides)]
    params = [{"omega": W.omega_from_nu(v)} for v in nus]
    res = []
    for pairs in (True, False):
        ens = Ensemble(dicos, params, dtype="float16", tile=(64, 2, 0), pairs=pairs)
        ens.run(31)
        ens.synchronize()
        res.append([ens.moments(i) for i in range(len(dicos))])
        ens.free()
    for i in range(len(dicos)):
        assert np.array_equal(res[0][i], res[1][i]), i
    # same reference state as the ensemble (the odd grid's mean momentum is not 0)
    sim = Simulation(dicos[1], dtype="float16", c0=[1.0, 0.0, 0.0])
    sim.extra_parameters = {OMEGA: params[1]["omega"]}
    sim.run(31)
    assert np.array_equal(res[0][1], _moments(sim))
    sim.free()


def _fits(sim):
    """The host mirror of the kernels' two-node condition (pairs_fit)."""
    lat = sim._lat
    L = sim.dim - 1
    return (lat.n[L] % 2 == 0 and (lat.origin + lat.halo[L]) % 2 == 0 and lat.vstride % 2 == 0
            and all(lat.stride[d] % 2 == 0 for d in range(L)))


@pytest.mark.parametrize("case,dtype", [("disc_flow", "float16"), ("cube", "float16"), ("cube", "bfloat16"),
                                        ("geier_channel", "float16"), ("cavity", "bfloat16"),
                                        ("vectorial_channel", "float16"), ("euler_1d", "bfloat16")])
def test_bounded_pairs_equal_single_nodes(case, dtype):
    """Bounded domains: the two-node step reads the ghost layer the boundary
    methods wrote; results equal the one-node step bit for bit."""
    make = {
        "disc_flow": lambda: W.cylinder(nx=192, ny=64, radius=8, center=(48, 33), re=80.0),
        "cube": lambda: W.cavity3d(n=32),
        "geier_channel": lambda: W.karman(dx=1.0 / 32),
        "cavity": lambda: W.cavity(n=64),
        # D2Q4 x 3 with Bouzidi walls and NeumannX; D1Q3 x 3 Euler with Neumann ends
        "vectorial_channel": lambda: demo_cases.poiseuille_vec(),
        "euler_1d": lambda: demo_cases.euler_1d(),
    }[case]
    out = []
    for pairs in (True, False):
        sim = Simulation(make(), dtype=dtype, node_pairs=pairs)
        assert not sim.periodic
        if pairs:
            assert _fits(sim)
        sim.run(25)
        out.append(_moments(sim))
        sim.free()
    assert np.all(np.isfinite(out[0]))
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("dtype", ["float16", "bfloat16"])
@pytest.mark.parametrize("case", ["tgv", "shear", "shear_long_rows"])
def test_staged_step_equals_direct_loads(case, dtype):
    """Periodic 16-bit steps: the staged kernel (rows copied into shared memory
    by bulk copies on the TMA unit, two nodes per thread) equals the
    direct-load paired kernel bit for bit, and none of its bounded waits gives up."""
    import ctypes

    make = {"tgv": lambda: W.tgv3d(n=32), "shear": lambda: W.shear_layer(n=128, nu=1e-3),
            "shear_long_rows": lambda: W.shear_layer(n=512, nu=1e-3)}[case]
    out = []
    for variant in (1, 0):
        sim = Simulation(make(), dtype=dtype)
        sim.module.call(sim.module.lib.lbm_scheme_set_step_variant(variant))
        sim.run(30)
        out.append(_moments(sim))
        count = ctypes.c_uint32()
        sim.module.call(sim.module.lib.lbm_scheme_wait_timeouts(ctypes.byref(count)))
        assert count.value == 0
        sim.module.call(sim.module.lib.lbm_scheme_set_step_variant(0))
        sim.free()
    assert np.all(np.isfinite(out[0]))
    assert np.array_equal(out[0], out[1])
