"""Generate the full-size fixtures of tests/golden/ by running the reference pylbm.

The workloads are the benchmark configurations at their full sizes, run by
the reference's own Cython generator (single process, float64):

* tgv3d_n256_sampled.npz   D3Q19 MRT periodic Taylor-Green vortex, 256^3,
                           500 steps: all 19 moments at every 16th node,
                           the conserved moments on three full grid lines,
                           per-moment sums and sums of squares over every
                           node, kinetic energy every 100 steps.
* cylinder_2048x512_sampled.npz
                           D2Q9 MRT flow past a disc of radius 32 at
                           (400, 257), 2048x512, Re 200, 20 000 steps: the
                           conserved moments at every 8th node, all 9 moments
                           on the 64x64 patch behind the disc, per-moment sums
                           and sums of squares, and the cross-stream momentum
                           qy at two wake probes every 20 steps (shedding).

Run where the reference sources and Cython are importable, with the import
shims of oracle/shims first on the path; the reference's location comes from
the environment (``PYLBM_REFERENCE``, default: the ``pylbm`` already on
``PYTHONPATH``):

    PYTHONDONTWRITEBYTECODE=1 PYTHONPATH=oracle/shims:$PYLBM_REFERENCE \
        python tests/golden/make_fullsize_golden.py [tgv] [cylinder]

Each case takes minutes of one CPU core (about 12 min for the TGV).
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
if os.environ.get("PYLBM_REFERENCE"):
    sys.path.insert(0, os.environ["PYLBM_REFERENCE"])

import pylbm  # noqa: E402  (reference, through the shims)

from pylbm_gb300 import workloads as W  # noqa: E402

# sampling shared with the tests (tests/test_gpu_fullsize.py)
TGV_STRIDE, TGV_OFFSET = 16, 5
TGV_LINE = (37, 101, 190)          # the x-, y- and z-lines pass through this node
CYL_STRIDE = 8
CYL_PATCH = (slice(432, 496), slice(225, 289))
CYL_PROBES = ((560, 257), (720, 300))
CYL_PROBE_EVERY = 20


def moments(sim, nv):
    return np.array([np.array(sim.m[i]) for i in range(nv)])


def sums(m):
    """Per-moment sum and sum of squares over every interior node (float64, pairwise)."""
    flat = m.reshape(m.shape[0], -1)
    return flat.sum(axis=1), (flat * flat).sum(axis=1)


def tgv():
    n, steps = 256, 500
    d = W.tgv3d(n=n)
    d["generator"] = "cython"
    t0 = time.time()
    sim = pylbm.Simulation(d)
    nv = 19
    print(f"tgv setup {time.time() - t0:.1f}s", flush=True)
    energy = []
    t1 = time.time()
    for s in range(steps + 1):
        if s % 100 == 0:
            m = moments(sim, nv)
            rho = m[0]
            ke = 0.5 * float(((m[1] ** 2 + m[2] ** 2 + m[3] ** 2) / rho).sum())
            energy.append((s, ke))
            print(f"  step {s} ke {ke:.17g} ({time.time() - t1:.0f}s)", flush=True)
        if s < steps:
            sim.one_time_step()
    m = moments(sim, nv)
    i, j, k = TGV_LINE
    sl = slice(TGV_OFFSET, None, TGV_STRIDE)
    s1, s2 = sums(m)
    cons = [0, 1, 2, 3]
    np.savez_compressed(
        os.path.join(HERE, "tgv3d_n256_sampled.npz"),
        sub=m[:, sl, sl, sl], line_x=m[cons][:, :, j, k], line_y=m[cons][:, i, :, k], line_z=m[cons][:, i, j, :],
        sum=s1, sumsq=s2, energy=np.array(energy), steps=np.array(steps), n=np.array(n),
        stride=np.array(TGV_STRIDE), offset=np.array(TGV_OFFSET), line=np.array(TGV_LINE))
    print(f"tgv done {time.time() - t0:.0f}s", flush=True)


def cylinder():
    steps = 20000
    d = W.cylinder(nx=2048, ny=512, radius=32, center=(400, 257), re=200.0, bc=pylbm.bc, circle=pylbm.Circle)
    d["generator"] = "cython"
    t0 = time.time()
    sim = pylbm.Simulation(d)
    nv = 9
    print(f"cylinder setup {time.time() - t0:.1f}s", flush=True)
    probes = []
    t1 = time.time()
    for s in range(steps + 1):
        if s % CYL_PROBE_EVERY == 0:
            qy = sim.m[2]
            probes.append([qy[p] for p in CYL_PROBES])
            if s % 2000 == 0:
                print(f"  step {s} probes {probes[-1]} ({time.time() - t1:.0f}s)", flush=True)
        if s < steps:
            sim.one_time_step()
    m = moments(sim, nv)
    s1, s2 = sums(m)
    sl = slice(None, None, CYL_STRIDE)
    np.savez_compressed(
        os.path.join(HERE, "cylinder_2048x512_sampled.npz"),
        sub=m[:3][:, sl, sl], patch=m[:, CYL_PATCH[0], CYL_PATCH[1]], sum=s1, sumsq=s2,
        probes=np.array(probes), probe_nodes=np.array(CYL_PROBES), probe_every=np.array(CYL_PROBE_EVERY),
        steps=np.array(steps), stride=np.array(CYL_STRIDE),
        patch_origin=np.array([CYL_PATCH[0].start, CYL_PATCH[1].start]))
    print(f"cylinder done {time.time() - t0:.0f}s", flush=True)


if __name__ == "__main__":
    which = sys.argv[1:] or ["tgv", "cylinder"]
    for name in which:
        {"tgv": tgv, "cylinder": cylinder}[name]()
