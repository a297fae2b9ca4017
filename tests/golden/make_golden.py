"""Generate the golden fixtures of tests/golden/ by running the reference pylbm.

Run in a container where the reference sources are available (read-only) and
Cython is installed:

    PYTHONDONTWRITEBYTECODE=1 \
    PYTHONPATH=oracle/shims:$PYLBM_REFERENCE python tests/golden/make_golden.py

The shims in oracle/shims stand in for mpi4py (one rank), cerberus,
colorlog, colorama, h5py, matplotlib and numpy-stl, which pylbm imports but
the hot path does not need.  Every fixture records the reference's own
outputs (``generator='cython'`` unless stated) for a workload dictionary of
pylbm_gb300.workloads built with pylbm's boundary classes:

* velocities.npz          velocity numbering of pylbm.stencil.Velocity
* cavity_n32.npz          D2Q9 cavity 32^2: scheme matrices, boundary lists,
                          moments at steps 0, 50 and 300; NumPy-generator drift
* cavity_n256_sampled.npz D2Q9 cavity 256^2 after 1000 steps (the full
                          workload), every 4th node plus two edge strips
* cylinder_small.npz      D2Q9 disc flow 96x32: domain flags/distances,
                          boundary lists, moments after 100 steps
* tgv3d_n16.npz           D3Q19 periodic Taylor-Green 16^3 after 20 steps
* shear_n64.npz           D2Q9 periodic shear layer 64^2 after 200 steps
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import pylbm  # noqa: E402  (reference, through the shims)
from pylbm.stencil import Velocity  # noqa: E402

from pylbm_gb300 import workloads as W  # noqa: E402


def run(dico, steps, gen="cython"):
    d = dict(dico)
    d["generator"] = gen
    t0 = time.time()
    sim = pylbm.Simulation(d)
    snaps = {0: np.array([sim.m[i] for i in range(sim.scheme.stencil.nv_ptr[-1])])}
    done = 0
    for s in sorted(steps):
        while done < s:
            sim.one_time_step()
            done += 1
        snaps[s] = np.array([np.array(sim.m[i]) for i in range(sim.scheme.stencil.nv_ptr[-1])])
    print(f"  {gen}: {time.time() - t0:.1f}s", flush=True)
    return sim, snaps


def bc_lists(sim):
    out = {}
    for i, meth in enumerate(sim.bc.methods):
        out[f"bc{i}_name"] = np.array(type(meth).__name__)
        out[f"bc{i}_istore"] = np.asarray(meth.istore)
        out[f"bc{i}_iload0"] = np.asarray(meth.iload[0])
        out[f"bc{i}_rhs"] = np.asarray(meth.rhs)
    out["bc_count"] = np.array(len(sim.bc.methods))
    return out


def scheme_arrays(sim):
    import sympy as sp
    M = np.array(sim.algo.M.subs(list(sim.scheme.param.items())), dtype=np.float64)
    invM = np.array(sim.algo.invM.subs(list(sim.scheme.param.items())), dtype=np.float64)
    consm = np.array([str(k) for k in sim.scheme.consm.keys()])
    s = np.array([float(sp.sympify(x)) for x in sim.algo.s], dtype=np.float64)
    return {"M": M, "invM": invM, "consm": consm, "s": s}


def main():
    out = {}
    for dim, count in ((1, 9), (2, 49), (3, 125)):
        out[f"v{dim}"] = np.array([Velocity(dim=dim, num=i).v for i in range(count)], dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "velocities.npz"), **out)
    print("velocities")

    print("cavity 32")
    dico = W.cavity(n=32, bc=pylbm.bc)
    sim, snaps = run(dico, [50, 300])
    _, snaps_np = run(dico, [300], gen="numpy")
    fix = {"m0": snaps[0], "m50": snaps[50], "m300": snaps[300], "m300_numpy": snaps_np[300]}
    fix.update(bc_lists(sim))
    fix.update(scheme_arrays(sim))
    np.savez_compressed(os.path.join(HERE, "cavity_n32.npz"), **fix)

    print("cavity 256 x 1000")
    dico = W.cavity(n=256, bc=pylbm.bc)
    sim, snaps = run(dico, [1000])
    m = snaps[1000]
    np.savez_compressed(os.path.join(HERE, "cavity_n256_sampled.npz"),
                        sub=m[:, ::4, ::4], lo_x=m[:, :2, :], hi_x=m[:, -2:, :], lo_y=m[:, :, :2], hi_y=m[:, :, -2:],
                        steps=np.array(1000))

    print("cylinder 96x32")
    dico = W.cylinder(nx=96, ny=32, radius=5, center=(24, 17), re=40.0, bc=pylbm.bc, circle=pylbm.Circle)
    sim, snaps = run(dico, [100])
    fix = {"m100": snaps[100], "flag": sim.domain.flag, "distance": sim.domain.distance,
           "in_or_out": sim.domain.in_or_out}
    fix.update(bc_lists(sim))
    np.savez_compressed(os.path.join(HERE, "cylinder_small.npz"), **fix)

    print("tgv3d 16")
    dico = W.tgv3d(n=16)
    sim, snaps = run(dico, [20])
    fix = {"m0": snaps[0], "m20": snaps[20]}
    fix.update(scheme_arrays(sim))
    np.savez_compressed(os.path.join(HERE, "tgv3d_n16.npz"), **fix)

    print("shear 64")
    dico = W.shear_layer(n=64, nu=1e-3)
    sim, snaps = run(dico, [200])
    np.savez_compressed(os.path.join(HERE, "shear_n64.npz"), m0=snaps[0], m200=snaps[200])
    print("done")


if __name__ == "__main__":
    main()
