"""Batched ensembles: one launch per step for many independent simulations.

Every instance must compute exactly what a single Simulation of the same
dictionary, storage type and run-time parameters computes.
"""
import numpy as np
import pytest
import sympy as sp

from conftest import rel_err
from pylbm_gb300 import Simulation
from pylbm_gb300 import workloads as W
from pylbm_gb300.ensemble import Ensemble, autotune, shear_ensemble

pytestmark = pytest.mark.gpu

OMEGA = sp.Symbol("omega")


def _instances(dtype):
    sides = [32, 48, 64, 40, 96]
    nus = [1e-3, 5e-2, 2e-3, 5e-4, 1e-2]
    dicos = [W.shear_layer(n=s, omega=OMEGA, seed=i) for i, s in enumerate(sides)]
    params = [{"omega": W.omega_from_nu(v)} for v in nus]
    return dicos, params


@pytest.mark.parametrize("dtype", ["float16", "float32", "float64"])
@pytest.mark.parametrize("tile", [(64, 1, 0), (128, 4, 152), (256, 2, 0)])
def test_ensemble_equals_single_runs(dtype, tile):
    dicos, params = _instances(dtype)
    ens = Ensemble(dicos, params, dtype=dtype, tile=tile)
    ens.run(41)
    ens.synchronize()
    for i, (d, p) in enumerate(zip(dicos, params)):
        sim = Simulation(d, dtype=dtype, parity=False)
        sim.extra_parameters = {OMEGA: p["omega"]}
        sim.run(41)
        single = np.array([sim.m[k] for k in range(sim.scheme.nv)])
        assert np.array_equal(ens.moments(i), single), (i, dtype, tile)
        sim.free()
    ens.free()


def test_autotuner_picks_a_valid_tile_and_caches_it():
    dicos, params = _instances("float16")
    ens = Ensemble(dicos, params, dtype="float16")
    block, rows, grid = ens.tile
    assert block in (32, 64, 128, 256) and rows in (1, 2, 4, 8, 16) and grid >= 0
    assert autotune(ens) == ens.tile  # second call reads the cache
    ens.run(10)
    sums, bad = ens.population_sums(0)
    assert bad == 0
    ens.free()


def test_shear_ensemble_fp16_against_fp64_single_runs():
    """Small version of the 512-instance workload: FP16 shifted storage vs FP64 runs."""
    ens, sides, nus = shear_ensemble(count=12, sides=(32, 48, 64), seed=3, dtype="float16")
    ens.run(200)
    for i in range(len(sides)):
        sim = Simulation(ens.dicos[i], dtype="float64", parity=False)
        sim.extra_parameters = {OMEGA: ens.params[i]["omega"]}
        sim.run(200)
        ref = np.array([sim.m[k] for k in range(3)])
        got = ens.moments(i, keys=range(3))
        # density against its own scale, momentum against the flow's momentum
        # scale (the y-momentum is a 5 % perturbation of it)
        err_rho = rel_err(got[:1], ref[:1]).max()
        err_q = np.abs(got[1:] - ref[1:]).max() / np.abs(ref[1:]).max()
        # FP16 stores the deviations with 11 significant bits: 200 steps leave
        # about 1e-4 on the density (measured up to 1.0e-4) and 2e-3 on q
        assert err_rho < 2e-4 and err_q < 5e-3, (i, sides[i], nus[i], err_rho, err_q)
        sim.free()
    ens.free()
