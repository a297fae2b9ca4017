"""CPU baseline: the reference's generated one_time_step on every host core.

TEST INFRASTRUCTURE ONLY (the CPU legs of bench.py).

pylbm runs on several cores through MPI domain decomposition
(pylbm/mpi_topology.py, one slab per rank, ghost exchange in
pylbm/storage.py:307-367).  Here P spawned processes each own one x-slab of
the D3Q19 Taylor-Green grid in pylbm's Cython layout f[x, y, z, k]
(pylbm/container.py:75-90) and, every step, refresh their ghost layers as
pylbm's Array.update does: the x faces come from the neighbouring slabs
(through shared memory, double-buffered by step parity, one barrier per
step), then the y and z ghosts by periodic copies within the slab; then they
call the reference's generated ``one_time_step(f, fnew, nx, ny, nz)``
(oracle/_ref, built by oracle/build_ref.py).  The processes therefore advance
the one global periodic grid, as pylbm's ranks would.  What is not timed is
pylbm's per-step Python orchestration around the kernel
(Simulation.one_time_step, the Array.update bookkeeping): leaving it out
favours the reference.  All processes start together; the rate is total node
updates / slowest process.  When oracle/_ref is missing, the C oracle
(float64, OpenMP) is timed instead.
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


def _halo_yz(f):
    f[:, 0] = f[:, -2]
    f[:, -1] = f[:, 1]
    f[:, :, 0] = f[:, :, -2]
    f[:, :, -1] = f[:, :, 1]


class _Faces:
    """Shared x faces of every slab: faces[parity, slab, side] = plane (y, z, k)."""

    def __init__(self, name, procs, plane_shape, create=False):
        from multiprocessing import shared_memory
        count = 2 * procs * 2 * int(np.prod(plane_shape))
        self.shm = shared_memory.SharedMemory(name=name, create=create, size=8 * count)
        self.a = np.ndarray((2, procs, 2) + tuple(plane_shape), dtype=np.float64, buffer=self.shm.buf)

    def close(self, unlink=False):
        del self.a
        self.shm.close()
        if unlink:
            self.shm.unlink()


def _exchange(f, faces, rank, procs, parity, barrier):
    """pylbm's x exchange (neighbouring slabs, periodic), then y and z in the slab."""
    faces.a[parity, rank, 0] = f[1]
    faces.a[parity, rank, 1] = f[-2]
    barrier.wait()
    f[0] = faces.a[parity, (rank - 1) % procs, 1]
    f[-1] = faces.a[parity, (rank + 1) % procs, 0]
    _halo_yz(f)


def _worker(n, x0, x1, steps, rank, procs, shm_name, barrier, results, keep_state):
    sys.path.insert(0, HERE)
    import build_ref
    mod = build_ref.load("tgv3d")
    f = _slab_state(n, x0, x1)
    fnew = np.empty_like(f)
    nx, ny, nz = f.shape[:3]
    faces = _Faces(shm_name, procs, f.shape[1:])
    # one untimed step (warm-up), then the timed ones; the step count is the
    # same on every rank, so the exchanges pair up
    _exchange(f, faces, rank, procs, 0, barrier)
    mod.one_time_step(f, fnew, nx, ny, nz)
    f, fnew = fnew, f
    barrier.wait()
    t0 = time.perf_counter()
    for s in range(steps):
        _exchange(f, faces, rank, procs, (s + 1) % 2, barrier)
        mod.one_time_step(f, fnew, nx, ny, nz)
        f, fnew = fnew, f
    dt = time.perf_counter() - t0
    state = np.array(f[1:-1, 1:-1, 1:-1]) if keep_state else None
    faces.close()
    results.put((rank, (x1 - x0) * n * n * steps, dt, state))


def run_slabs(n=256, steps=10, procs=None, keep_state=False):
    """Run the reference's kernel on ``procs`` slab processes; returns
    (node updates, slowest time, interior populations f[x, y, z, k] after
    1 + steps steps or None)."""
    procs = procs or os.cpu_count() or 1
    procs = min(procs, n)
    bounds = np.linspace(0, n, procs + 1).astype(int)
    ctx = mp.get_context("spawn")
    name = f"lbm_ref_faces_{os.getpid()}"
    faces = _Faces(name, procs, (n + 2, n + 2, 19), create=True)
    try:
        barrier = ctx.Barrier(procs)
        results = ctx.Queue()
        ps = [ctx.Process(target=_worker, args=(n, int(bounds[i]), int(bounds[i + 1]), steps, i, procs, name,
                                                barrier, results, keep_state)) for i in range(procs)]
        for p in ps:
            p.start()
        res = [results.get(timeout=3600) for _ in ps]
        for p in ps:
            p.join()
        if any(p.exitcode for p in ps):
            raise RuntimeError("a reference slab process failed")
    finally:
        faces.close(unlink=True)
    res.sort(key=lambda r: r[0])
    nodes = sum(r[1] for r in res)
    tmax = max(r[2] for r in res)
    state = np.concatenate([r[3] for r in res]) if keep_state else None
    return nodes, tmax, state


def reference_available():
    sys.path.insert(0, HERE)
    import build_ref
    try:
        return build_ref.compile_ref("tgv3d") is not None
    except Exception:
        return False


def reference_mlups(n=256, steps=10, procs=None):
    """MLUPS of the reference's generated kernel on ``procs`` processes."""
    nodes, tmax, _ = run_slabs(n=n, steps=steps, procs=procs)
    procs = min(procs or os.cpu_count() or 1, n)
    return {"value": nodes / tmax / 1e6, "unit": "MLUPS", "cores": procs, "kind": "reference",
            "sample": f"D3Q19 TGV {n}^3 (the whole grid), {steps} steps, float64: pylbm's generated Cython "
                      f"one_time_step (oracle/_ref) on {procs} processes, one x-slab each, x faces exchanged "
                      "between slabs every step as pylbm's MPI ranks do; pylbm's per-step Python orchestration "
                      "is not timed (favours the reference)"}


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
