"""Record the routine names and parameter names of pylbm's generated modules.

pylbm calls every generated routine through ``call_genfunction``
(pylbm/symbolic.py:288-299), which binds arguments by the names
``inspect.getfullargspec(routine).args`` lists.  This script builds the
reference's Cython modules for a set of dictionaries that together use every
boundary method of the hot path, reads those names, and writes
``ref_signatures.json``, which ``tests/test_generator_module.py`` compares
with ``pylbm_gb300.generator.CudaModule``.  Run where the reference sources
and Cython are available:

    PYTHONDONTWRITEBYTECODE=1 \\
    PYTHONPATH=oracle/shims:$PYLBM_REFERENCE python tests/golden/make_signatures.py
"""
import inspect
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import pylbm  # noqa: E402  (reference, through the shims)

import demo_cases  # noqa: E402
from pylbm_gb300 import workloads as W  # noqa: E402

ALGO = ["one_time_step", "f2m", "m2f", "equilibrium", "relaxation", "transport", "source_term"]


def cases():
    yield "cavity_d2q9", W.cavity(n=32, bc=pylbm.bc)
    yield "disc_flow_d2q9", W.cylinder(nx=96, ny=32, radius=5, center=(24, 17), re=40.0, bc=pylbm.bc,
                                       circle=pylbm.Circle)
    yield "poiseuille_vec", demo_cases.poiseuille_vec(bc=pylbm.bc)
    yield "euler_1d", demo_cases.euler_1d(bc=pylbm.bc)
    yield "poiseuille_3d", demo_cases.poiseuille_3d(bc=pylbm.bc)
    yield "karman_geier", demo_cases.karman_vortex_street(dx=1.0 / 32, bc=pylbm.bc, circle=pylbm.Circle)
    yield "tgv3d_d3q19", W.tgv3d(n=8)
    yield "advection_reaction_1d", demo_cases.advection_reaction_1d(bc=pylbm.bc)


def main():
    out = {}
    for name, dico in cases():
        d = dict(dico)
        d["generator"] = "cython"
        d["codegen_option"] = {"directory": tempfile.mkdtemp(prefix=f"sig_{name}_"), "generate": True}
        sim = pylbm.Simulation(d)
        mod = sim.algo.generator.module
        routines = {}
        for r in ALGO:
            fn = getattr(mod, r, None)
            if fn is not None:
                routines[r] = inspect.getfullargspec(fn).args
        for meth in sim.bc.methods:
            fn = meth.function
            routines[fn.__name__] = inspect.getfullargspec(fn).args
        out[name] = {"dim": int(sim.domain.dim),
                     "extra_parameters": sorted(str(k) for k in sim.extra_parameters),
                     "routines": routines}
        print(name, sorted(routines))
    with open(os.path.join(HERE, "ref_signatures.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
