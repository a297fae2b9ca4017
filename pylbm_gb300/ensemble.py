"""Batched ensembles: many independent periodic simulations in one launch per step.

pylbm runs one ``Simulation`` per process.  An ``Ensemble`` holds N
independent periodic simulations of one scheme -- each with its own grid size,
initial state and run-time parameters (e.g. the shear relaxation rate as a
free symbol ``omega``) -- in a single device arena, and advances all of them
with one persistent kernel launch per time step (``lbm_ensemble_step``): the
thread blocks stride over a list of tiles that covers every instance, so
small and large grids share the GPU without per-instance launches.  Two
steps are captured in a CUDA graph and replayed.  The tile shape (threads per
block, rows per tile, number of resident blocks) is chosen by ``autotune``,
which times the candidates on the ensemble itself and caches the winner.

Each instance computes exactly what a single ``Simulation`` of the same
dictionary, storage type and parameters computes (same generated module,
same per-node arithmetic), so single-instance runs check the ensemble.
"""
import ctypes
import hashlib
import json
import os
import types

import numpy as np
import sympy as sp

from . import runtime
from .codegen import SchemeSource
from .domain import Domain
from .scheme import Scheme
from .simulation import from_storage, RAW_DTYPE

TILE_BLOCKS = (32, 64, 128, 256)
TILE_ROWS = (1, 2, 4, 8, 16)
GRID_PER_SM = (0, 4, 8, 16)   # 0: one block per tile


class Ensemble:
    """N periodic simulations of one scheme.

    Parameters
    ----------
    dicos : list of dict
        pylbm dictionaries; same scheme (velocities, polynomials, equilibrium,
        relaxation rates as numbers or the same free symbols), box periodic
        along every axis.
    params : list of dict
        run-time parameter values per instance ({symbol or name: value}).
    dtype : str
        storage type ("float32", "float16", "bfloat16" shifted; "float64").
    tile : (block, rows_per_tile, grid) or None
        fixed tile shape; None runs the autotuner.
    pairs : bool or None
        threads update two neighbouring nodes (lbm_gb300.h,
        LBM_INSTANCE_PAIRS); default: on for 16-bit storage.
    """

    def __init__(self, dicos, params=None, dtype="float16", tile=None, c0=None, pairs=None):
        if not dicos:
            raise ValueError("an ensemble needs at least one instance")
        params = params or [{} for _ in dicos]
        if len(params) != len(dicos):
            raise ValueError("one parameter dict per instance")
        self.storage = dtype
        self.compute = "float64" if dtype == "float64" else "float32"
        self.shifted = dtype != "float64"
        self.pairs = (dtype in ("float16", "bfloat16")) if pairs is None else bool(pairs)
        self.scheme = Scheme(dicos[0])
        self.dicos = dicos
        self.params = [{str(k): float(v) for k, v in p.items()} for p in params]
        names = [str(s) for s in self.scheme.free_symbols]
        if len(names) > runtime.LBM_MAX_PRM:
            raise ValueError("too many run-time parameters for an ensemble")
        self.domains = []
        for i, d in enumerate(dicos):
            dom = Domain(d, self.scheme.stencil, with_flags=False)
            # time step of the source-term integrator: the instance's dx / la
            self.params[i].setdefault("dt", dom.dx / self.scheme.la_float)
            missing = [n for n in names if n not in self.params[i]]
            if missing:
                raise ValueError(f"missing run-time parameters {missing}")
            if dom.dim != self.scheme.dim:
                raise ValueError("dimension mismatch between instances")
            self.domains.append(dom)
        self._check_same_scheme()
        if c0 is None:
            c0 = [1.0] + [0.0] * (self.scheme.nconsm - 1) if self.shifted else None
        src = SchemeSource(self.scheme, self.shifted, c0, simplify_frame=self.compute == "float32")
        self.module = runtime.SchemeModule(src, dtype, self.compute)
        self._core = runtime.core()
        s = ctypes.c_void_p()
        runtime.check(self._core.lbm_stream_create(ctypes.byref(s)))
        self._stream = s
        es = runtime.DTYPE_SIZE[dtype]
        self.lats = []
        self.mlats = []
        offsets = []
        cursor = 0
        for dom in self.domains:
            lat = runtime.lattice(dom.dim, self.scheme.nv, dtype, dom.shape_in, [int(h) for h in dom.halo],
                                  shift=self.module.shift)
            self.lats.append(lat)
            self.mlats.append(runtime.lattice(dom.dim, self.scheme.nv, "float64", dom.shape_in,
                                              [int(h) for h in dom.halo]))
            offsets.append((cursor, cursor + lat.elements))
            cursor += 2 * lat.elements
        self.offsets = offsets
        self.arena = runtime.DeviceBuffer(cursor * es)
        self.arena.zero(self._stream)
        self.nodes = [int(np.prod(dom.shape_in)) for dom in self.domains]
        self.total_nodes = int(sum(self.nodes))
        self.parity = 0
        self.nt = 0
        self._graph = None
        self._graph_parity = None
        self._tables = {}
        self.tile = tuple(tile) if tile is not None else autotune(self)
        self._initialize()

    def _check_same_scheme(self):
        first = self.dicos[0]
        key = (str(first["schemes"]), str(first.get("parameters")), str(first["scheme_velocity"]))
        for d in self.dicos[1:]:
            if (str(d["schemes"]), str(d.get("parameters")), str(d["scheme_velocity"])) == key:
                continue
            sc = Scheme(d)
            if sc.nv != self.scheme.nv or sc.M_frac != self.scheme.M_frac or \
                    [str(e) for e in sc.EQ] != [str(e) for e in self.scheme.EQ] or \
                    [str(r) for r in sc.s] != [str(r) for r in self.scheme.s]:
                raise ValueError("all ensemble instances must share one scheme")

    # ------------------------------------------------------------------ tables
    def _table(self, block, rows):
        """Device instance descriptors and tile map for a tile shape."""
        key = (block, rows)
        if key in self._tables:
            return self._tables[key]
        L = self.scheme.dim - 1
        insts = (runtime.Instance * len(self.domains))()
        tile_map = []
        for i, (dom, lat) in enumerate(zip(self.domains, self.lats)):
            I = insts[i]
            I.offset[0], I.offset[1] = self.offsets[i]
            for d in range(3):
                I.n[d] = lat.n[d]
                I.halo[d] = lat.halo[d]
                I.stride[d] = lat.stride[d]
            I.vstride = lat.vstride
            I.origin = lat.origin
            I.rows = int(np.prod([lat.n[d] for d in range(L)])) if L > 0 else 1
            even = [lat.n[L], lat.origin + lat.halo[L], lat.vstride, *self.offsets[i]]
            even += [lat.stride[d] for d in range(L)]
            I.flags = runtime.LBM_INSTANCE_PAIRS if self.pairs and all(x % 2 == 0 for x in even) else 0
            span = 2 * block if I.flags else block
            I.col_tiles = -(-lat.n[L] // span)
            row_tiles = -(-I.rows // rows)
            I.tile_begin = len(tile_map)
            tile_map.extend([i] * (row_tiles * I.col_tiles))
            for j, name in enumerate(str(s) for s in self.scheme.free_symbols):
                I.prm[j] = self.params[i][name]
        dinst = runtime.DeviceBuffer(ctypes.sizeof(insts))
        runtime.check(self._core.lbm_memcpy(dinst.handle, ctypes.cast(insts, ctypes.c_void_p), ctypes.sizeof(insts),
                                            runtime.H2D, self._stream))
        tmap = np.asarray(tile_map, dtype=np.int32)
        dtiles = runtime.DeviceBuffer(max(tmap.nbytes, 4))
        dtiles.upload(tmap, stream=self._stream)
        self.synchronize()
        self._tables[key] = (dinst, dtiles, len(tile_map), insts)
        return self._tables[key]

    # ------------------------------------------------------------------ init
    def _initialize(self):
        sc = self.scheme
        es = runtime.DTYPE_SIZE[self.storage]
        biggest = max(m.elements for m in self.mlats)
        mbuf = runtime.DeviceBuffer(biggest * 8)
        for i, (d, dom) in enumerate(zip(self.dicos, self.domains)):
            lat, mlat = self.lats[i], self.mlats[i]
            coords = np.meshgrid(*dom.coords_halo, sparse=True, indexing="ij")
            plane = np.zeros(mlat.vstride)
            view = np.lib.stride_tricks.as_strided(plane[mlat.origin:], shape=dom.shape_halo,
                                                   strides=[mlat.stride[k] * 8 for k in range(dom.dim)])
            for key, val in (d.get("init") or {}).items():
                idx = sc.consm[key] if isinstance(key, (sp.Symbol, sp.IndexedBase)) else int(key)
                view[...] = 0.0
                if isinstance(val, tuple):
                    view[...] = val[0](*(tuple(coords) + (tuple(val[1]) if len(val) == 2 else ())))
                elif isinstance(val, types.FunctionType):
                    view[...] = val(*coords)
                else:
                    view[...] = val
                mbuf.upload(plane, offset=idx * mlat.vstride * 8, stream=self._stream)
            prm = np.array([self.params[i][str(s)] for s in sc.free_symbols] + [0.0])
            pp = prm.ctypes.data_as(ctypes.c_void_p)
            f0 = ctypes.c_void_p(self.arena.ptr + self.offsets[i][0] * es)
            f1 = ctypes.c_void_p(self.arena.ptr + self.offsets[i][1] * es)
            # equilibrium then m2f, in one pass (as Simulation initialises)
            self.module.call(self.module.lib.lbm_init_conserved(mbuf.handle, ctypes.byref(mlat), f0,
                                                                ctypes.byref(lat), pp, self._stream))
            runtime.check(self._core.lbm_memcpy(f1, f0, lat.elements * es, runtime.D2D, self._stream))
            self.synchronize()
        mbuf.free()
        self.parity = 0
        self.nt = 0

    # ------------------------------------------------------------------ steps
    def _enqueue(self, parity, tile=None):
        block, rows, grid = tile or self.tile
        dinst, dtiles, ntiles, insts = self._table(block, rows)
        # every instance on the two-node path: the kernel without the one-node path
        pairs_only = all(I.flags & runtime.LBM_INSTANCE_PAIRS for I in insts)
        entry = self.module.lib.lbm_ensemble_step_pairs if pairs_only else self.module.lib.lbm_ensemble_step
        self.module.call(entry(self.arena.handle, dinst.handle, dtiles.handle, ntiles, rows, block, grid, parity,
                               self._stream))

    def one_time_step(self):
        self._enqueue(self.parity)
        self.parity ^= 1
        self.nt += 1

    def run(self, nsteps, graph=True):
        nsteps = int(nsteps)
        if not graph or nsteps < 2:
            for _ in range(nsteps):
                self.one_time_step()
            return
        if self._graph is None or self._graph_parity != self.parity:
            self._drop_graph()
            self._table(*self.tile[:2])  # allocations must happen before the capture
            runtime.check(self._core.lbm_graph_begin(self._stream))
            try:
                self._enqueue(self.parity)
                self._enqueue(self.parity ^ 1)
            finally:
                g = ctypes.c_void_p()
                rc = self._core.lbm_graph_end(self._stream, ctypes.byref(g))
            runtime.check(rc)
            self._graph = g
            self._graph_parity = self.parity
        for _ in range(nsteps // 2):
            runtime.check(self._core.lbm_graph_launch(self._graph, self._stream))
        self.nt += 2 * (nsteps // 2)
        if nsteps % 2:
            self.one_time_step()

    def _drop_graph(self):
        if self._graph is not None:
            self._core.lbm_graph_destroy(self._graph)
        self._graph = None
        self._graph_parity = None

    def synchronize(self):
        runtime.check(self._core.lbm_stream_synchronize(self._stream))

    # ------------------------------------------------------------------ access
    def moments(self, i, keys=None):
        """Interior moments (nv or len(keys), *shape) of instance ``i`` in float64."""
        lat, mlat, dom = self.lats[i], self.mlats[i], self.domains[i]
        es = runtime.DTYPE_SIZE[self.storage]
        mbuf = runtime.DeviceBuffer(mlat.elements * 8)
        f = ctypes.c_void_p(self.arena.ptr + self.offsets[i][self.parity] * es)
        self.module.call(self.module.lib.lbm_f2m(f, ctypes.byref(lat), mbuf.handle, ctypes.byref(mlat), self._stream))
        keys = range(self.scheme.nv) if keys is None else keys
        out = []
        inner = tuple(slice(int(h), -int(h)) for h in dom.halo)
        for k in keys:
            k = self.scheme.consm[k] if isinstance(k, (sp.Symbol, sp.IndexedBase)) else int(k)
            plane = np.empty(mlat.vstride)
            mbuf.download(plane, offset=k * mlat.vstride * 8, stream=self._stream)
            v = np.lib.stride_tricks.as_strided(plane[mlat.origin:], shape=dom.shape_halo,
                                                strides=[mlat.stride[d] * 8 for d in range(dom.dim)])
            out.append(np.array(v[inner]))
        mbuf.free()
        return np.array(out)

    def population_sums(self, i):
        """FP64 interior sums of every population of instance ``i`` and the NaN/Inf count."""
        lat = self.lats[i]
        es = runtime.DTYPE_SIZE[self.storage]
        f = ctypes.c_void_p(self.arena.ptr + self.offsets[i][self.parity] * es)
        size = ctypes.c_size_t()
        runtime.check(self._core.lbm_population_sums_scratch_bytes(ctypes.byref(lat), ctypes.byref(size)))
        scratch = runtime.DeviceBuffer(size.value)
        out = runtime.DeviceBuffer(8 * (self.scheme.nv + 1))
        runtime.check(self._core.lbm_population_sums(f, ctypes.byref(lat), out.handle,
                                                     ctypes.c_void_p(out.ptr + 8 * self.scheme.nv), scratch.handle,
                                                     size.value, self._stream))
        host = np.empty(self.scheme.nv + 1)
        out.download(host, stream=self._stream)
        return host[:self.scheme.nv], int(np.frombuffer(host[self.scheme.nv:].tobytes()[:4], np.int32)[0])

    def free(self):
        self._drop_graph()
        self.arena.free()
        for dinst, dtiles, _, _ in self._tables.values():
            dinst.free()
            dtiles.free()
        self._tables = {}
        if self._stream:
            self._core.lbm_stream_destroy(self._stream)
            self._stream = None


# ---------------------------------------------------------------------- tuner
def _cache_path():
    return os.path.join(runtime.JIT_DIR, "autotune.json")


def _signature(ens):
    sm, name = runtime.device_info()
    sizes = sorted(tuple(lat.n[d] for d in range(3)) for lat in ens.lats)
    text = json.dumps([name, sm, ens.module.key, ens.storage, ens.pairs, sizes])
    return hashlib.sha256(text.encode()).hexdigest()[:20], sm


def autotune(ens, steps=4, candidates=None):
    """Pick (block, rows_per_tile, grid) by timing each candidate on ``ens``.

    Runs on the arena before initialisation (zero deviations = the rest
    state, so every candidate does the same work); the winner is cached per
    device, module, storage type and set of grid sizes.
    """
    sig, sm = _signature(ens)
    path = _cache_path()
    cache = {}
    if os.path.exists(path):
        try:
            with open(path) as fh:
                cache = json.load(fh)
        except (OSError, ValueError):
            cache = {}
    if sig in cache:
        return tuple(cache[sig]["tile"])
    cands = candidates or [(b, r, g * sm) for b in TILE_BLOCKS for r in TILE_ROWS for g in GRID_PER_SM]
    results = []
    for cand in cands:
        ens._enqueue(0, cand)  # warm-up (also builds the tables)
        ens.synchronize()
        e0, e1 = runtime.Event(), runtime.Event()
        e0.record(ens._stream)
        for s in range(steps):
            ens._enqueue(s & 1, cand)
        e1.record(ens._stream)
        results.append((e0.elapsed_ms(e1) / steps, cand))
    best_ms, best = min(results)
    ens.arena.zero(ens._stream)
    cache[sig] = {"tile": list(best), "ms_per_step": best_ms,
                  "timings": [[list(c), t] for t, c in sorted(results)[:8]]}
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + f".{os.getpid()}.tmp"
    with open(tmp, "w") as fh:
        json.dump(cache, fh, indent=1)
    os.replace(tmp, path)
    return tuple(best)


def shear_ensemble(count=512, sides=tuple(range(64, 513, 32)), nu_range=(5e-4, 5e-2), seed=0, dtype="float16",
                   tile=None):
    """The batched double-shear-layer workload: ``count`` instances, sides drawn
    uniformly from ``sides``, viscosity log-uniform in ``nu_range``."""
    from . import workloads as W

    rng = np.random.default_rng(seed)
    omega = sp.Symbol("omega")
    sides = np.asarray(sides)
    n = rng.choice(sides, size=count)
    nu = np.exp(rng.uniform(np.log(nu_range[0]), np.log(nu_range[1]), size=count))
    dicos = [W.shear_layer(n=int(s), omega=omega, seed=int(seed * 100003 + i)) for i, s in enumerate(n)]
    params = [{"omega": W.omega_from_nu(float(v))} for v in nu]
    return Ensemble(dicos, params, dtype=dtype, tile=tile), n, nu


def main(argv=None):
    """Time the batched shear-layer workload: ``python -m pylbm_gb300.ensemble``."""
    import argparse

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--count", type=int, default=512)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--dtype", default="float16", choices=["float64", "float32", "float16", "bfloat16"])
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args(argv)
    ens, sides, _ = shear_ensemble(count=args.count, seed=args.seed, dtype=args.dtype)
    ens.run(4)
    ens.synchronize()
    e0, e1 = runtime.Event(), runtime.Event()
    e0.record(ens._stream)
    ens.run(args.steps)
    e1.record(ens._stream)
    ms = e0.elapsed_ms(e1)
    nodes = ens.total_nodes
    print(json.dumps({"instances": len(sides), "nodes_per_step": nodes, "steps": args.steps, "tile": list(ens.tile),
                      "ms_per_step": ms / args.steps, "MLUPS": nodes * args.steps / (ms / 1e3) / 1e6}))
    ens.free()


if __name__ == "__main__":
    main()
