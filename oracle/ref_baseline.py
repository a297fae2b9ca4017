"""CPU baseline: the reference's generated one_time_step on every host core.

TEST INFRASTRUCTURE ONLY (the CPU legs of bench.py).

pylbm runs on several cores through MPI domain decomposition
(pylbm/mpi_topology.py, one slab per rank, ghost exchange in
pylbm/storage.py:307-367).  Here P spawned processes each own one x-slab of
the D3Q19 Taylor-Green grid in pylbm's Cython layout f[x, y, z, k]
(pylbm/container.py:75-90), refresh their ghost layers by periodic copies and
call the reference's generated ``one_time_step(f, fnew, nx, ny, nz)``
(oracle/_ref, built by oracle/build_ref.py).  All processes start together;
the rate is total node updates / slowest process.  When oracle/_ref is
missing, the C oracle (float64, OpenMP) is timed instead.
"""
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _slab_state(n, x0, x1):
    """TGV equilibrium on the slab [x0, x1) x n x n, AoS with one ghost layer."""
    sys.path.insert(0, ROOT)
    from pylbm_gb300 import workloads as W
    from pylbm_gb300.scheme import Scheme

    dico = W.tgv3d(n=n)
    sc = Scheme(dico)
    dx = dico["space_step"]
    xs = (np.arange(x0 - 1, x1 + 1) + 0.5) * dx
    ys = (np.arange(-1, n + 1) + 0.5) * dx
    X, Y, Z = np.meshgrid(xs, ys, ys, indexing="ij")
    init = dico["init"]
    cons = np.stack([init[W.RHO](X, Y, Z), init[W.QX](X, Y, Z), init[W.QY](X, Y, Z), init[W.QZ](X, Y, Z)])
    feq = sc.feq_numpy(cons.reshape(4, -1)).reshape((sc.nv,) + X.shape)
    return np.ascontiguousarray(np.moveaxis(feq, 0, -1))


def _halo(f):
    f[0] = f[-2]
    f[-1] = f[1]
    f[:, 0] = f[:, -2]
    f[:, -1] = f[:, 1]
    f[:, :, 0] = f[:, :, -2]
    f[:, :, -1] = f[:, :, 1]


def _worker(args):
    n, x0, x1, steps, barrier = args
    sys.path.insert(0, HERE)
    import build_ref
    mod = build_ref.load("tgv3d")
    f = _slab_state(n, x0, x1)
    fnew = np.empty_like(f)
    nx, ny, nz = f.shape[:3]
    _halo(f)
    mod.one_time_step(f, fnew, nx, ny, nz)  # warm-up
    barrier.wait()
    t0 = time.perf_counter()
    for _ in range(steps):
        _halo(f)
        mod.one_time_step(f, fnew, nx, ny, nz)
        f, fnew = fnew, f
    dt = time.perf_counter() - t0
    return (x1 - x0) * n * n * steps, dt


def reference_available():
    sys.path.insert(0, HERE)
    import build_ref
    try:
        return build_ref.compile_ref("tgv3d") is not None
    except Exception:
        return False


def reference_mlups(n=256, steps=10, procs=None):
    """MLUPS of the reference's generated kernel on ``procs`` processes."""
    procs = procs or os.cpu_count() or 1
    procs = min(procs, n)
    bounds = np.linspace(0, n, procs + 1).astype(int)
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        barrier = mgr.Barrier(procs)
        with ctx.Pool(procs) as pool:
            res = pool.map(_worker, [(n, int(bounds[i]), int(bounds[i + 1]), steps, barrier) for i in range(procs)])
    nodes = sum(r[0] for r in res)
    tmax = max(r[1] for r in res)
    return {"value": nodes / tmax / 1e6, "unit": "MLUPS", "cores": procs, "kind": "reference",
            "sample": f"D3Q19 TGV {n}^3, {steps} steps, float64: pylbm's generated Cython one_time_step "
                      f"(oracle/_ref) on {procs} processes, one x-slab each"}


def oracle_mlups(n=256, steps=4, threads=None):
    """MLUPS of the C oracle (restated algorithm, OpenMP)."""
    sys.path.insert(0, HERE)
    sys.path.insert(0, ROOT)
    from oracle import OracleSimulation
    from pylbm_gb300 import workloads as W

    threads = threads or os.cpu_count() or 1
    o = OracleSimulation(W.tgv3d(n=n), nthreads=threads)
    o.initialize()
    o.one_time_step()
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    return {"value": n ** 3 * steps / dt / 1e6, "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"D3Q19 TGV {n}^3, {steps} steps, float64, C oracle with OpenMP over {threads} threads"}


def cpu_baseline(n=256, steps=10):
    if reference_available():
        return reference_mlups(n=n, steps=steps)
    return oracle_mlups(n=n, steps=max(2, steps // 3))
