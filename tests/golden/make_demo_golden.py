"""Fixtures of pylbm's own golden demo results (tests/reference/*.h5 of the reference).

Run in a container where the reference sources are available (read-only) and
Cython is installed:

    PYTHONDONTWRITEBYTECODE=1 \
    PYTHONPATH=oracle/shims:$PYLBM_REFERENCE python tests/golden/make_demo_golden.py [case ...]

For every case of tests/demo_cases.py this script
1. reads the reference's HDF5 golden file with h5lite (fields stored
   transposed, pylbm/hdf5.py:204-206) and turns it back to [x, y(, z)];
2. runs the reference pylbm (generator='cython') on the restated dictionary,
   built with pylbm's own boundary classes, to the same final time, zeroes the
   non-fluid nodes as pylbm's test harness does (tests/conftest.py:234-242)
   and checks the result against the golden file at pylbm's tolerance
   (rel 1e-14, abs 1e-7) -- this proves the restatement is the demo;
   (cases without a pylbm golden file -- stencils reaching two nodes -- keep
   the reference run itself as the fixture);
3. writes demo_<case>.npz: the golden fields (3D fields reduced by
   demo_cases.reduce_field), the fluid mask (3D: whether every node is
   fluid), the number of steps and the largest reference-vs-golden
   difference.
"""
import os
import sys

import numpy as np
import sympy as sp

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
ROOT = os.path.dirname(TESTS)
REFERENCE = os.environ.get("PYLBM_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
sys.path.insert(0, ROOT)
sys.path.insert(0, TESTS)
sys.path.insert(0, HERE)

import pylbm  # noqa: E402  (reference, through the shims)

import demo_cases  # noqa: E402
import h5lite  # noqa: E402


def fluid_mask(sim):
    """Interior part of in_or_out (pylbm's harness strips one ghost layer,
    tests/conftest.py:234-238; the vmax = 2 cases have two)."""
    shape_in = sim.domain.shape_in
    inner = tuple(slice((n - m) // 2, (n - m) // 2 + m) for n, m in zip(sim.domain.in_or_out.shape, shape_in))
    return sim.domain.in_or_out[inner] == sim.domain.valin


def make(name):
    build, final_time, h5name, fields = demo_cases.CASES[name]
    full = None
    if h5name is not None:
        gold = h5lite.read(os.path.join(REFERENCE, "tests", "reference", h5name + ".h5"))
        full = {k: np.ascontiguousarray(gold[k].T) for k in fields}
    extra = {k: v for k, v in (("circle", pylbm.Circle), ("parallelogram", pylbm.Parallelogram),
                               ("sphere", pylbm.Sphere)) if k in build.__code__.co_varnames}
    sim = pylbm.Simulation(build(bc=pylbm.bc, generator="cython", **extra))
    demo_cases.run_to(sim, final_time)
    mask = fluid_mask(sim)
    worst = 0.0
    if full is None:  # no pylbm golden file: the reference's own run is the fixture
        full = {}
        for key, cons in fields.items():
            full[key] = np.array(sim.m[sp.Symbol(cons)])
            full[key][~mask] = 0.0
    for key, cons in fields.items():
        val = np.array(sim.m[sp.Symbol(cons)])
        val[~mask] = 0.0
        diff = np.abs(val - full[key])
        ok = np.all(diff <= np.maximum(1e-14 * np.abs(full[key]), 1e-7))
        worst = max(worst, float(diff.max()))
        print(f"  {name}.{key}: max |reference - golden| = {diff.max():.3e} {'ok' if ok else 'MISMATCH'}")
        if not ok:
            raise SystemExit(f"{name}: the restated dictionary does not reproduce {h5name}.h5")
    arrays = {}
    for key in fields:
        for suffix, part in demo_cases.reduce_field(full[key]).items():
            arrays[key + suffix] = part
    out = os.path.join(HERE, f"demo_{name}.npz")
    np.savez_compressed(out, mask=mask if mask.size <= 8192 else np.array(bool(mask.all())), steps=np.int64(sim.nt),
                        final_time=np.float64(final_time), reference_maxdiff=np.float64(worst), **arrays)
    print("wrote", out, sim.nt, "steps")


if __name__ == "__main__":
    for case in sys.argv[1:] or list(demo_cases.CASES):
        make(case)
