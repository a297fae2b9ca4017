"""pylbm's own golden demo results (tests/reference/*.h5) against the CPU oracle.

The fixtures hold the reference's HDF5 fields at the final time of pylbm's
regression tests (tests/golden/make_demo_golden.py, which also checks that
the reference itself reproduces them from the restated dictionaries of
tests/demo_cases.py).  Tolerance: pylbm's own (tests/conftest.py:306-307).
"""
import numpy as np
import pytest
import sympy as sp

import demo_cases
from conftest import golden
from oracle import OracleSimulation


def fluid_mask(sim, stored):
    """The fixture's fluid mask, or (large fixtures) the simulation's own,
    checked against the fixture's reduced copy of it."""
    if stored.ndim:
        return stored
    dom = sim.domain
    if dom.in_or_out is None:  # periodic along every axis: no solid nodes
        return np.ones(dom.shape_in, dtype=bool)
    inner = tuple(slice(int(h), -int(h)) for h in dom.halo)
    mask = dom.in_or_out[inner] == dom.valin
    assert bool(stored) == bool(mask.all())
    return mask


def conserved_fields(sim, moments, fields, mask):
    mask = fluid_mask(sim, mask)
    out = {}
    for key, cons in fields.items():
        v = np.array(moments[sim.scheme.consm[sp.Symbol(cons)]], dtype=np.float64)
        v[~mask] = 0.0
        out[key] = v
    return out


def assert_golden(values, g, fields):
    for key in fields:
        for suffix, part in demo_cases.reduce_field(values[key]).items():
            ref = g[key + suffix]
            tol = 1e-7 if suffix != "__sum" else 1e-7 * values[key].size
            diff = np.abs(part - ref)
            assert np.all(diff <= np.maximum(1e-14 * np.abs(ref), tol)), (key + suffix, float(diff.max()))


@pytest.mark.parametrize("name", list(demo_cases.CASES))
def test_oracle_reproduces_reference_golden(name):
    build, final_time, _, fields = demo_cases.CASES[name]
    g = golden(f"demo_{name}.npz")
    o = OracleSimulation(build())
    demo_cases.run_to(o, final_time)
    assert o.nt == int(g["steps"])
    vals = conserved_fields(o, o.moments(), fields, g["mask"])
    assert_golden(vals, g, fields)
