"""``Simulation`` with ``generator='cuda'``: pylbm's time loop on one GB300.

The public surface follows pylbm/simulation.py:33: ``Simulation(dico, sorder,
dtype, check_inverse, initialize)``, ``one_time_step()`` (:393-420),
``boundary_condition()`` (:374-390), ``m[...]``/``F[...]`` item access
(:216-256), ``t``, ``nt``, ``dt``, ``extra_parameters``.  The populations live
on the device in the padded structure-of-arrays layout of the C ABI; a step is

    lbm_update_halo(F)                       periodic ghost refresh
    lbm_<method>(F, iload0, istore, rhs)     every boundary method in order
    lbm_one_time_step(F, Fnew)               fused pull-stream + collide
    swap(F, Fnew)

and a domain that is periodic along every axis skips the first two and uses
``lbm_one_time_step_periodic``, which wraps the pull inside the interior.
``run(n)`` replays a captured CUDA graph of two steps (the buffers are back in
place after two swaps), so a step costs one graph launch instead of one
Python call and 2 + nmethods kernel launches.

``dtype`` selects the storage type: "float64" (FP64 storage and arithmetic,
the parity path) or "float32"/"float16"/"bfloat16" (values stored as
deviations f - feq(c0) from the equilibrium of a reference state c0 of the
conserved moments, arithmetic in FP32).
"""
import ctypes
import types

import numpy as np
import sympy as sp

from . import runtime
from .boundary import Boundary, batch_entries, box_wall_table, observed_ghost_copies
from .codegen import SchemeSource
from .domain import Domain
from .scheme import Scheme

_STORAGES = ("float64", "float32", "float16", "bfloat16")


class _ItemAccess:
    """``sim.m[key]`` / ``sim.m[key] = value`` helper (pylbm/utils.py:26-81).

    With a box reader, ``sim.m[key, i0, i1, ...]`` (ints and slices over the
    interior nodes) copies only the selected nodes from the device."""

    def __init__(self, getter, setter=None, box=None):
        self._get = getter
        self._set = setter
        self._box = box

    def __getitem__(self, key):
        if isinstance(key, tuple) and self._box is not None:
            return self._box(key[0], key[1:])
        return self._get(key)

    def __setitem__(self, key, value):
        if self._set is None:
            raise AttributeError("read-only item access")
        self._set(key, value)


def _round_reference(values):
    """Reference value of a conserved moment: its mean, to 4 significant digits."""
    mean = float(np.mean(values))
    scale = float(np.max(np.abs(values))) if values.size else 0.0
    if scale == 0.0 or abs(mean) <= 1e-6 * scale:
        return 0.0
    return float(f"{mean:.4g}")


def to_storage(host, dtype):
    """float64 numpy -> raw storage array of ``dtype`` (bfloat16 as uint16 bits)."""
    if dtype == "float64":
        return np.ascontiguousarray(host, dtype=np.float64)
    if dtype == "float32":
        return np.ascontiguousarray(host, dtype=np.float32)
    if dtype == "float16":
        return np.ascontiguousarray(host, dtype=np.float16)
    # bfloat16: round-to-nearest-even on the float32 bit pattern
    b = np.ascontiguousarray(host, dtype=np.float32).view(np.uint32)
    rounding = ((b >> 16) & 1) + 0x7FFF
    return ((b + rounding) >> 16).astype(np.uint16)


def from_storage(raw, dtype):
    if dtype == "bfloat16":
        return (raw.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    return raw.astype(np.float64)


RAW_DTYPE = {"float64": np.float64, "float32": np.float32, "float16": np.float16, "bfloat16": np.uint16}


def flat_slots(rows, lat, dim):
    """int32 element offsets k * vstride + node offset of (k, i0, ...) rows of
    a lattice (lbm_bc_method with LBM_BC_FLAT)."""
    rows = np.asarray(rows, dtype=np.int64).reshape(-1, dim + 1)
    off = rows[:, 0] * lat.vstride + lat.origin
    for d in range(dim):
        off = off + rows[:, 1 + d] * lat.stride[d]
    return np.ascontiguousarray(off, dtype=np.int32)


def float_form_constants(kind, iload, istore, rhs, dist, shift):
    """Per-link FP32 constant of LBM_BC_FLOAT_FORM: the shifts of the load and
    store populations folded into the right-hand side, in float64, rounded
    once, so that the link computes on stored deviations g = f - shift:
    g_s = +/- g_0 + c, or ((1 - d) g_1 +/- d g_0) + c for Bouzidi links."""
    shift = np.asarray(shift, dtype=np.float64)
    s0 = shift[np.asarray(iload[0])[:, 0]]
    ss = shift[np.asarray(istore)[:, 0]]
    rhs = np.zeros(len(ss)) if kind == "neumann" else np.asarray(rhs, dtype=np.float64)
    if kind.startswith("bouzidi"):
        s1 = shift[np.asarray(iload[1])[:, 0]]
        t0 = dist * s0
        c = (1.0 - dist) * s1 + (-t0 if kind == "bouzidi_anti_bounce_back" else t0)
    else:
        c = -s0 if kind == "anti_bounce_back" else s0
    return np.ascontiguousarray(c + rhs - ss, dtype=np.float32)


class Simulation:
    """A pylbm simulation whose hot path runs on the GPU.

    Parameters
    ----------
    dico : dict
        pylbm scheme dictionary; ``generator`` must be 'cuda' (or absent).
    sorder : ignored
        kept for signature compatibility: the device layout is fixed.
    dtype : str
        storage type, one of "float64", "float32", "float16", "bfloat16".
    initialize : bool
        initialise the populations now (else on the first step).
    shifted : bool or None
        store deviations from feq(c0); default: every type but float64.
    parity : bool
        float64 only: evaluate the per-node algebra in the reference
        generator's printed form (refforms), compiled without FMA, so results
        track pylbm's Cython code; False uses the faster exact-constant form.
    node_pairs : bool
        16-bit storage on periodic domains: one thread updates two
        neighbouring nodes with packed FP32x2 arithmetic (bit-identical to
        one node per thread, fewer instructions per node).
    c0 : sequence of float or None
        reference state of the conserved moments for shifted storage
        (default: the mean of the initial fields, 4 significant digits).
    device_domain : bool
        build the fluid/solid map, wall distances and boundary link lists on
        the GPU (identical to the host construction; for large obstacle
        sets); ``domain.in_or_out``/``distance``/``flag`` then stay on the
        device (``domain.download_arrays()``).
    halo : str
        "observed" (default): the ghost refresh copies only the ghost
        populations that a later read observes (an interior pull or a
        boundary load that no boundary store precedes), as extra links of the
        boundary launch where the lists allow it; interior results are those
        of the full refresh bit for bit, ghost populations nothing reads
        keep stale values.  "full": pylbm's refresh of every ghost
        population of every axis.
    """

    def __init__(self, dico, sorder=None, dtype="float64", check_inverse=False, initialize=True,
                 shifted=None, parity=True, node_pairs=True, c0=None, device_domain=False, halo="observed"):
        gen = str(dico.get("generator", "cuda")).upper()
        if gen != "CUDA":
            raise ValueError(f"pylbm_gb300 implements generator='cuda', not {gen!r}")
        if dtype not in _STORAGES:
            raise ValueError(f"dtype must be one of {_STORAGES}")
        self.parity = bool(parity)
        self.node_pairs = bool(node_pairs)
        if halo not in ("observed", "full"):
            raise ValueError("halo must be 'observed' or 'full'")
        self.halo = halo
        self.c0 = None if c0 is None else [float(c) for c in c0]
        self.dico = dico
        self.scheme = Scheme(dico)
        lab = dico["box"].get("label", -1)
        lab = [lab] if isinstance(lab, (int, np.integer)) else list(lab)
        all_periodic = all(int(l) == -1 for l in lab) and not dico.get("elements")
        # wall distances and flags only matter where some boundary method needs them
        self.domain = Domain(dico, self.scheme.stencil, with_flags=not all_periodic, device=device_domain)
        if self.domain.dim != self.scheme.dim:
            raise ValueError("the dimension of the domain and of the scheme are not the same")
        self.dim = self.domain.dim
        self.storage = dtype
        self.compute = "float64" if dtype == "float64" else "float32"
        self.shifted = (dtype != "float64") if shifted is None else bool(shifted)
        self.t = 0.0
        self.nt = 0
        self._dt = self.domain.dx / self.scheme.la_float
        self.extra_parameters = {}
        self.init_type = dico.get("inittype", "moments")
        self.init_data = dico.get("init", None)
        self.periodic = all(l == -1 for l in self.domain.box_label) and not self.domain.elements

        self.bc = Boundary(self.domain, dico)
        for meth in self.bc.methods:
            meth.set_iload()

        self._core = runtime.core()
        shape_in = self.domain.shape_in
        halo = [int(h) for h in self.domain.halo]
        self._lat = runtime.lattice(self.dim, self.scheme.nv, dtype, shape_in, halo)
        self._mlat = runtime.lattice(self.dim, self.scheme.nv, "float64", shape_in, halo)
        es = runtime.DTYPE_SIZE[dtype]
        s = ctypes.c_void_p()
        runtime.check(self._core.lbm_stream_create(ctypes.byref(s)))
        self._stream = s
        self._F = runtime.DeviceBuffer(self._lat.elements * es)
        self._Fnew = runtime.DeviceBuffer(self._lat.elements * es)
        for buf in (self._F, self._Fnew):  # row and plane padding stays zero (host reads whole planes)
            buf.zero(self._stream)
        self._M = None
        self.module = None
        self._m_cache = {}
        self._update_m = True
        self._m_partial = False     # only the conserved planes of the moment array are current
        self._eq_pending = False    # the other planes are the equilibrium of the conserved ones, not yet computed
        self._bc_dev = []
        self._bc_batch = None
        self._ghost = None          # observed ghost copies: (istore, iload) device lists
        self._ghost_alone = None    # their one-entry batch table when they cannot join the methods
        self._batch_bufs = []       # device lists made for the batch table
        self._batch_rhs = []        # (device array, method index, host builder) of batch right-hand sides that follow time_bc
        self._full_halo = True
        self.batch_boundary = True  # one launch for all boundary methods where the lists allow it
        # bounce-back box walls applied in the pull where the links allow it
        # (cube 256^3 per step: FP32 0.396 against 0.430 ms with the boundary
        # launch, FP16 0.249 against 0.256, BF16 0.250 against 0.253)
        self.fold_walls = True
        self._walls = None          # (constants nv x 27, opposite populations) of lbm_one_time_step_walls
        self._graph = None
        self._graph_key = None
        self._need_init = True
        if initialize:
            self._initialize()

    # ------------------------------------------------------------------ setup
    @property
    def dt(self):
        return self._dt

    def extra_parameters_str(self):
        return {str(k): v for k, v in self.extra_parameters.items()}

    def _prm(self, for_init=False):
        """Run-time parameter vector (free symbols of the scheme, sorted by name).

        Initialisation only evaluates the equilibrium, so it needs only the
        symbols that appear there (as pylbm, which takes ``extra_parameters``
        after construction); a step needs them all.
        """
        vals = dict(self.extra_parameters_str())
        vals.setdefault("dt", self.dt)  # time step of the source-term integrator
        names = [str(s) for s in self.scheme.free_symbols]
        needed = set(names)
        if for_init:
            needed = {str(s) for e in self.scheme.EQ for s in e.free_symbols} & needed
        missing = [n for n in names if n not in vals and n in needed]
        if missing:
            raise ValueError(f"extra_parameters must give values for {missing}")
        return np.array([float(vals.get(n, 0.0)) for n in names] + [0.0], dtype=np.float64)

    def feq_host(self, cons):
        """Equilibrium populations of boundary values on the host.

        In the float64 parity form they come from the reference generator's
        printed equilibrium and m2f routines, so boundary right-hand sides
        equal pylbm's; otherwise from the exact-constant matrices.
        """
        params = self.extra_parameters_str()
        if self.module is not None and self.module.src.style == "reference":
            prm = [float(params.get(str(s), 0.0)) for s in self.scheme.free_symbols]
            return self.module.src.reference_forms().feq_host(cons, prm)
        return self.scheme.feq_numpy(cons, params)

    def _mbuf(self):
        if self._M is None:
            self._M = runtime.DeviceBuffer(self._mlat.elements * 8)
        return self._M

    def _plane_view(self, plane, lat):
        """(shape_halo) view of one population plane of a padded buffer."""
        es = plane.itemsize
        return np.lib.stride_tricks.as_strided(plane[lat.origin:], shape=self.domain.shape_halo,
                                               strides=[lat.stride[d] * es for d in range(self.dim)])

    def _initialize(self):
        sc = self.scheme
        nv = sc.nv
        coords = np.meshgrid(*self.domain.coords_halo, sparse=True, indexing="ij")
        shape = self.domain.shape_halo
        if self.init_type not in ("moments", "distributions"):
            raise ValueError("inittype must be 'moments' or 'distributions'")
        # only the conserved moments are given for a moment initialisation;
        # the device computes the others (equilibrium) and the populations
        nplanes = sc.nconsm if self.init_type == "moments" else nv
        arr = np.zeros([nplanes] + shape)
        if self.init_data is not None:
            for key, val in self.init_data.items():
                if self.init_type == "moments":
                    idx = sc.consm[key] if isinstance(key, (sp.Symbol, sp.IndexedBase)) else int(key)
                else:
                    idx = int(key)
                if idx >= nplanes:
                    raise ValueError(f"initial value given for non-conserved moment {key}")
                if isinstance(val, tuple):
                    fargs = tuple(coords) + (tuple(val[1]) if len(val) == 2 else ())
                    arr[idx] = val[0](*fargs)
                elif isinstance(val, types.FunctionType):
                    arr[idx] = val(*coords)
                else:
                    arr[idx] = val
        if self.init_type == "distributions":
            arr = np.einsum("ij,j...->i...", sc.M, arr)
        inner = tuple(slice(int(h), -int(h)) for h in self.domain.halo)
        c0 = None
        if self.shifted:
            c0 = self.c0 if self.c0 is not None else [_round_reference(arr[c][inner]) for c in range(sc.nconsm)]
        # the printed-form parity style covers the plain MRT step; schemes with a
        # relative velocity or source terms use the exact-constant form
        plain = sc.Tu is None and not sc.source_terms
        style = "reference" if (self.storage == "float64" and not self.shifted and self.parity and plain) else "fast"
        src = SchemeSource(sc, self.shifted, c0, style=style, node_pairs=self.node_pairs,
                           simplify_frame=self.compute == "float32")
        self.module = runtime.SchemeModule(src, self.storage, self.compute)
        for k in range(nv):
            self._lat.shift[k] = float(self.module.shift[k])
        mbuf = self._mbuf()
        plane = np.zeros(self._mlat.vstride, dtype=np.float64)
        for c in range(nplanes):
            self._plane_view(plane, self._mlat)[...] = arr[c]
            mbuf.upload(plane, offset=c * self._mlat.vstride * 8, stream=self._stream)
        del arr
        prm = self._prm(for_init=True)
        pp = prm.ctypes.data_as(ctypes.c_void_p)
        if self.init_type == "moments":  # equilibrium then m2f, in one pass
            self.module.call(self.module.lib.lbm_init_conserved(mbuf.handle, ctypes.byref(self._mlat), self._F.handle,
                                                                ctypes.byref(self._lat), pp, self._stream))
        else:
            self.module.call(self.module.lib.lbm_m2f(mbuf.handle, ctypes.byref(self._mlat), self._F.handle,
                                                     ctypes.byref(self._lat), self._stream))
        runtime.check(self._core.lbm_memcpy(self._Fnew.handle, self._F.handle, self._F.nbytes, runtime.D2D,
                                            self._stream))
        self.synchronize()
        for meth in self.bc.methods:
            meth.prepare_rhs(self)
            meth.fix_iload()
            meth.set_rhs()
        self._upload_bc()
        self._update_m = True
        self._m_cache = {}
        self._drop_graph()
        self._need_init = False

    def _device_array(self, a, itemsize):
        buf = runtime.DeviceBuffer(max(a.nbytes, itemsize))
        buf.upload(a, stream=self._stream)
        return buf

    def _check_links(self, meth):
        """Every slot of the method's lists lies in the halo box (no device-side check)."""
        hi = np.array([self.scheme.nv] + [n + 2 * int(h) for n, h in zip(self.domain.shape_in, self.domain.halo)])
        for lst in [meth.istore] + list(meth.iload):
            if lst.size and (lst.min() < 0 or np.any(lst.max(axis=0) >= hi)):
                raise ValueError(f"{type(meth).__name__}: link list outside the lattice")

    def _upload_bc(self):
        self._free_bc()
        for meth in self.bc.methods:
            self._check_links(meth)
            dev = {"iload": [self._device_array(il, 4) for il in meth.iload],
                   "istore": self._device_array(meth.istore, 4),
                   "rhs": self._device_array(meth.rhs, 8),
                   "ordered": 0 if self._links_independent(meth) else 1}
            if meth.kind.startswith("bouzidi"):
                dev["dist"] = self._device_array(np.ascontiguousarray(meth.s, dtype=np.float64), 8)
                # copy semantics of the bounce-back: compute every link before storing
                dev["scratch"] = runtime.DeviceBuffer(8 * max(meth.ncond, 1)) if dev["ordered"] else None
            self._bc_dev.append((meth, dev))
        self._upload_ghost()
        self._bc_batch = self._batch_table()
        self._walls = self._wall_table()

    def _wall_table(self):
        """Constants of the bounce-back box walls folded into the step, or None."""
        if self.periodic or self._full_halo or self._ghost is not None or self.dim > 3:
            return None
        if any(m.kind != "bounce_back" for m in self.bc.methods):
            return None
        float_form = self.storage != "float64"
        if not float_form and any(self._lat.shift[k] for k in range(self.scheme.nv)):
            return None
        if float_form:
            consts = [self._float_constants(m.kind, m.iload, m.istore, m.rhs, None) for m in self.bc.methods]
        else:
            consts = [np.asarray(m.rhs, dtype=np.float64) for m in self.bc.methods]
        table = box_wall_table(self.bc.methods, self.domain.shape_in, self.domain.halo,
                               self.scheme.stencil.get_all_velocities(), consts)
        if table is None:
            return None
        sym = np.ascontiguousarray(self.scheme.stencil.get_symmetric(), dtype=np.int32)
        return np.ascontiguousarray(table.reshape(-1), dtype=np.float64), sym

    def _upload_ghost(self):
        """The ghost copies a step observes (``halo='observed'``), else the full refresh."""
        self._full_halo = True
        if self.halo != "observed":
            return
        copies = observed_ghost_copies(self.domain.shape_in, self.domain.halo,
                                       self.scheme.stencil.get_all_velocities(), self.bc.methods)
        if copies is None:
            return
        self._full_halo = False
        istore, iload = copies
        if len(istore):
            self._ghost = {"istore_host": istore, "iload_host": iload, "ncond": int(len(istore)),
                           "istore": self._device_array(istore, 4), "iload": self._device_array(iload, 4),
                           "joined": False}
            entry = (runtime.LBM_BC_KIND["ghost_copy"], len(istore), self._ghost["iload"].ptr, None,
                     self._ghost["istore"].ptr, None, None)
            self._ghost_alone = self._table([entry])

    def _slot_keys(self, lst):
        """int64 key of each [k, i_0, ...] slot of a link list."""
        ext = [self.scheme.nv] + [n + 2 * int(h) for n, h in zip(self.domain.shape_in, self.domain.halo)]
        lst = np.asarray(lst, dtype=np.int64).reshape(-1, len(ext))
        return np.ravel_multi_index(tuple(lst.T), tuple(ext))

    def _links_independent(self, meth):
        """True when no link reads a slot another link of the method writes."""
        st = self._slot_keys(meth.istore)
        return not any(np.isin(self._slot_keys(il), st).any() for il in meth.iload)

    def _table(self, entries):
        """Device lbm_bc_method table of (kind, ncond, iload0, iload1, istore, rhs, dist[, flags]) entries."""
        table = (runtime.BcMethod * len(entries))()
        first = 0
        for t, e in zip(table, entries):
            kind, ncond, il0, il1, st, rhs, dist = e[:7]
            t.kind, t.ncond, t.first, t.flags = kind, ncond, first, (e[7] if len(e) > 7 else 0)
            t.iload0, t.iload1, t.istore, t.rhs, t.dist = il0, il1, st, rhs, dist
            first += ncond
        buf = runtime.DeviceBuffer(ctypes.sizeof(table))
        runtime.check(self._core.lbm_memcpy(buf.handle, ctypes.cast(table, ctypes.c_void_p), ctypes.sizeof(table),
                                            runtime.H2D, self._stream))
        self.synchronize()
        return buf, len(entries), first

    def _batch_table(self):
        """Device table of every method (and the observed ghost copies) for
        one lbm_boundary_batch launch, or None when the links cannot all read
        the populations as they are before the launch (then the ghost copies
        and the methods run one after the other, as pylbm applies them).

        Every link of a batch reads the state before the launch.  Two kinds of
        load see a value another link writes in the sequential order, and are
        rewritten: a load of a copied ghost slot reads the copy's source, and a
        Neumann link whose load slot another method stores (the outflow's corner
        links reading a wall's ghosts) takes that method's formula for the slot
        and stores its result (the value the copy would have moved)."""
        self._batch_rhs = []   # (device array, method index, host builder) refreshed with time_bc
        self._batch_bufs = []  # device lists made for the table
        g = self._ghost
        ghost = (g["istore_host"], g["iload_host"]) if g is not None else None
        ext = [self.scheme.nv] + [n + 2 * int(h) for n, h in zip(self.domain.shape_in, self.domain.halo)]
        plan = batch_entries([m for m, _ in self._bc_dev], ext, ghost)
        if plan is None:
            return None
        entries, joined = plan
        if g is not None:
            g["joined"] = joined
        rows = []
        # shifted storage: the links compute in FP32 on the stored deviations,
        # with the shifts folded into one per-link constant (LBM_BC_FLOAT_FORM)
        float_form = self.storage != "float64"
        # one int32 element offset per slot instead of a (k, i0, ...) row when
        # the kernel needs no population index (LBM_BC_FLAT)
        unshifted = not any(self._lat.shift[k] for k in range(self.scheme.nv))
        flat = (float_form or unshifted) and self._lat.elements < 2 ** 31
        flags = (runtime.LBM_BC_FLOAT_FORM if float_form else 0) | (runtime.LBM_BC_FLAT if flat else 0)
        if g is not None and g["joined"]:
            if flat:
                gl, gs = (self._device_array(self._flat_slots(a), 4) for a in (g["iload_host"], g["istore_host"]))
                self._batch_bufs += [gl, gs]
            else:
                gl, gs = g["iload"], g["istore"]
            rows.append((runtime.LBM_BC_KIND["ghost_copy"], g["ncond"], gl.ptr, None, gs.ptr, None, None,
                         runtime.LBM_BC_FLAT if flat else 0))
        for e in entries:
            i, links = e["method"], e["links"]
            m, dev = self._bc_dev[i]
            if flat:
                il = [self._device_array(self._flat_slots(a), 4) for a in e["iload"]]
                st = self._device_array(self._flat_slots(e["istore"]), 4)
                self._batch_bufs += il + [st]
            elif links is None and all(a is b for a, b in zip(e["iload"], m.iload)):
                il = dev["iload"]
                st = dev["istore"]
            else:
                il = [self._device_array(np.ascontiguousarray(a, dtype=np.int32), 4) for a in e["iload"]]
                st = self._device_array(np.ascontiguousarray(e["istore"], dtype=np.int32), 4)
                self._batch_bufs += il + [st]
            sel = slice(None) if links is None else links
            dist_host = np.asarray(m.s, dtype=np.float64)[sel] if hasattr(m, "s") else None
            if float_form:
                def rhs_of(meth, e=e, sel=sel, d=dist_host):
                    return self._float_constants(e["kind"], e["iload"], e["istore"], np.asarray(meth.rhs)[sel], d)
                rhs = self._device_array(rhs_of(m), 4)
                self._batch_rhs.append((rhs, i, rhs_of))
                self._batch_bufs.append(rhs)
                dist = None
                if dist_host is not None:
                    dist = self._device_array(np.ascontiguousarray(dist_host, dtype=np.float32), 4)
                    self._batch_bufs.append(dist)
            else:
                rhs, dist = dev["rhs"], dev.get("dist")
                if links is not None:
                    def rhs_of(meth, sel=sel):
                        return np.ascontiguousarray(np.asarray(meth.rhs)[sel], dtype=np.float64)
                    rhs = self._device_array(rhs_of(m), 8)
                    self._batch_rhs.append((rhs, i, rhs_of))
                    self._batch_bufs.append(rhs)
                    if dist is not None:
                        dist = self._device_array(np.ascontiguousarray(dist_host), 8)
                        self._batch_bufs.append(dist)
            rows.append((runtime.LBM_BC_KIND[e["kind"]], int(len(e["istore"])), il[0].ptr,
                         il[1].ptr if len(il) > 1 else None, st.ptr, rhs.ptr, dist.ptr if dist is not None else None,
                         flags))
        if len(rows) < (1 if float_form else 2):
            if g is not None:
                g["joined"] = False
            return None
        return self._table(rows)

    def _flat_slots(self, rows):
        return flat_slots(rows, self._lat, self.dim)

    def _float_constants(self, kind, iload, istore, rhs, dist):
        return float_form_constants(kind, iload, istore, rhs, dist, self.module.shift)

    # ------------------------------------------------------------------ step
    def _enqueue_boundary(self, F):
        lat = ctypes.byref(self._lat)
        batch = self._bc_batch is not None and self.batch_boundary
        if self._full_halo:
            runtime.check(self._core.lbm_update_halo(F.handle, lat, self._stream))
        elif self._ghost is not None and not (batch and self._ghost["joined"]):
            buf, nmeth, total = self._ghost_alone
            runtime.check(self._core.lbm_boundary_batch(F.handle, lat, buf.handle, nmeth, total, self._stream))
        if batch:
            buf, nmeth, total = self._bc_batch
            runtime.check(self._core.lbm_boundary_batch(F.handle, lat, buf.handle, nmeth, total, self._stream))
            return
        for meth, dev in self._bc_dev:
            il, st, rhs, ordered = dev["iload"], dev["istore"].handle, dev["rhs"].handle, dev["ordered"]
            if meth.kind == "bounce_back":
                rc = self._core.lbm_bounce_back(F.handle, il[0].handle, st, meth.ncond, rhs, lat, ordered,
                                                self._stream)
            elif meth.kind == "anti_bounce_back":
                rc = self._core.lbm_anti_bounce_back(F.handle, il[0].handle, st, meth.ncond, rhs, lat, ordered,
                                                     self._stream)
            elif meth.kind == "bouzidi_bounce_back":
                scratch = dev["scratch"].handle if dev["scratch"] is not None else None
                rc = self._core.lbm_bouzidi_bounce_back(F.handle, il[0].handle, il[1].handle, st, meth.ncond, rhs,
                                                        dev["dist"].handle, lat, scratch, self._stream)
            elif meth.kind == "bouzidi_anti_bounce_back":
                rc = self._core.lbm_bouzidi_anti_bounce_back(F.handle, il[0].handle, il[1].handle, st, meth.ncond,
                                                             rhs, dev["dist"].handle, lat, ordered, self._stream)
            else:
                rc = self._core.lbm_neumann(F.handle, il[0].handle, st, meth.ncond, lat, ordered, self._stream)
            runtime.check(rc)

    def set_closure(self, model):
        """Use a learned collision closure (closure.ClosureModel) from the next step on.

        Periodic domains only; ``None`` returns to the plain relaxation.
        """
        if model is not None and not self.periodic:
            raise ValueError("the learned closure runs on periodic domains")
        if model is not None and (self.scheme.Tu is not None or self.scheme.source_terms):
            raise ValueError("the learned closure corrects the plain MRT relaxation only")
        self.closure = model
        if not hasattr(self, "closure_kernel"):
            # "tc": tcgen05 MMAs, 128 nodes per block; "warp": mma.sync, 32 nodes
            # per warp; "auto": the tensor-core step from 2^20 interior nodes on
            # (measured with the trained rate-form model, us per step, warp /
            # tc: 256^2 10.3 / 14.4, 512^2 23.0 / 26.0, 768^2 45.8 / 46.0,
            # 1024^2 75.2 / 73.3, 1536^2 162 / 152; on smaller grids a
            # block's set-up is spread over too few tiles)
            self.closure_kernel = "auto"
        if model is not None and getattr(self, "_fallbacks", None) is None:
            self._fallbacks = runtime.DeviceBuffer(4)
        if model is not None:
            self._fallbacks.zero(self._stream)
        self._drop_graph()

    def closure_fallbacks(self):
        """Node updates since set_closure() at which the closure's guard kept the
        plain MRT collision (corrections not finite, or far beyond the
        relaxation's own change)."""
        if getattr(self, "_fallbacks", None) is None:
            return 0
        out = np.zeros(1, dtype=np.int32)
        self._fallbacks.download(out, stream=self._stream)
        return int(out[0])

    def _launch_step(self, F, Fnew, pp):
        model = getattr(self, "closure", None)
        if model is not None and self._closure_on_tensor_cores():
            # the MLP on the 5th-generation tensor cores, one node per thread
            self.module.call(self.module.lib.lbm_one_time_step_periodic_closure_tc(
                F.handle, Fnew.handle, ctypes.byref(self._lat), pp, model.mlp.p.handle, model.norm_ptr(),
                model.guard_ptr(), model.rate_ptr(), self._fallbacks.handle, self._stream))
            return
        if model is not None:
            self.module.call(self.module.lib.lbm_one_time_step_periodic_closure(
                F.handle, Fnew.handle, ctypes.byref(self._lat), pp, model.mlp.w.handle, model.mlp.p.handle,
                model.norm_ptr(), model.guard_ptr(), model.rate_ptr(), self._fallbacks.handle, model.grid,
                self._stream))
            return
        fn = self.module.lib.lbm_one_time_step_periodic if self.periodic else self.module.lib.lbm_one_time_step
        self.module.call(fn(F.handle, Fnew.handle, ctypes.byref(self._lat), pp, self._stream))

    def _closure_on_tensor_cores(self):
        kernel = getattr(self, "closure_kernel", "auto")
        if kernel not in ("auto", "tc", "warp"):
            raise ValueError(f"closure_kernel: {kernel!r} (auto, tc or warp)")
        if kernel == "auto":
            return int(np.prod(self.domain.shape_in)) >= 1 << 20
        return kernel == "tc"

    def launches_per_step(self):
        """Kernel launches of one step: ghost refresh, boundary methods, step."""
        if self.periodic or self._folded():
            return 1
        batch = self._bc_batch is not None and self.batch_boundary
        n = 1
        if self._full_halo or (self._ghost is not None and not (batch and self._ghost["joined"])):
            n += 1
        if batch:
            return n + 1
        for meth, dev in self._bc_dev:
            n += 2 if meth.kind == "bouzidi_bounce_back" and dev["ordered"] else 1
        return n

    def _folded(self):
        return self._walls is not None and self.fold_walls and getattr(self, "closure", None) is None

    def _launch_walls_step(self, F, Fnew, pp):
        table, sym = self._walls
        self.module.call(self.module.lib.lbm_one_time_step_walls(
            F.handle, Fnew.handle, ctypes.byref(self._lat), pp, table.ctypes.data_as(ctypes.c_void_p),
            sym.ctypes.data_as(ctypes.c_void_p), self._stream))

    def _enqueue_step(self, F, Fnew, prm):
        if self._folded():
            self._launch_walls_step(F, Fnew, prm.ctypes.data_as(ctypes.c_void_p))
            return
        if not self.periodic:
            self._enqueue_boundary(F)
        self._launch_step(F, Fnew, prm.ctypes.data_as(ctypes.c_void_p))

    def boundary_condition(self):
        """Ghost refresh then every boundary method (pylbm/simulation.py:374-390)."""
        if self._need_init:
            self._initialize()
        if self.periodic:
            # the periodic step wraps inside the interior; the ghost layer is
            # refreshed here for the phase-by-phase routines (transport)
            runtime.check(self._core.lbm_update_halo(self._F.handle, ctypes.byref(self._lat), self._stream))
            return
        for i, (meth, dev) in enumerate(self._bc_dev):
            if meth.update_feq(self):
                meth.set_rhs()
                dev["rhs"].upload(meth.rhs, stream=self._stream)
                for buf, j, rhs_of in self._batch_rhs:
                    if j == i:
                        buf.upload(rhs_of(meth), stream=self._stream)
        self._enqueue_boundary(self._F)

    def one_time_step(self):
        """One time step (pylbm/simulation.py:393-420)."""
        if self._need_init:
            self._initialize()
        self._update_m = True
        self._eq_pending = False
        self._m_cache = {}
        prm = self._prm()
        if self._folded():
            self._launch_walls_step(self._F, self._Fnew, prm.ctypes.data_as(ctypes.c_void_p))
        else:
            if not self.periodic:
                self.boundary_condition()
            self._launch_step(self._F, self._Fnew, prm.ctypes.data_as(ctypes.c_void_p))
        self._F, self._Fnew = self._Fnew, self._F
        self.t += self.dt
        self.nt += 1

    # ---------------------------------------------------- phase by phase
    # pylbm's routines for users who split the step themselves
    # (pylbm/simulation.py:258-372): each runs one C-ABI kernel on the
    # device populations F / Fnew and the float64 moment array m.
    def initialization(self):
        """Populations from the dictionary's initial values (pylbm/simulation.py:258-320)."""
        self._initialize()
        self.t = 0.0
        self.nt = 0

    def _moments_ready(self):
        if self._need_init:
            self._initialize()
        self._m_cache = {}

    def transport(self):
        """Fnew = pulled F, ghost layer included as it is (pylbm/simulation.py:322-327)."""
        self._moments_ready()
        self.module.call(self.module.lib.lbm_transport(self._F.handle, self._Fnew.handle, ctypes.byref(self._lat),
                                                       self._stream))

    def f2m(self):
        """m = M F on the whole box (pylbm/simulation.py:344-350)."""
        self._moments_ready()
        self.module.call(self.module.lib.lbm_f2m(self._F.handle, ctypes.byref(self._lat), self._mbuf().handle,
                                                 ctypes.byref(self._mlat), self._stream))
        self._update_m = False
        self._m_partial = False

    def m2f(self):
        """F = M^-1 m on the whole box (pylbm/simulation.py:352-358).  After
        ``equilibrium()`` the populations come from the conserved moments in
        one pass (lbm_init_conserved), without the equilibrium planes."""
        self._moments_ready()
        if self._eq_pending and not self._update_m:
            prm = self._prm(for_init=True)
            self.module.call(self.module.lib.lbm_init_conserved(
                self._mbuf().handle, ctypes.byref(self._mlat), self._F.handle, ctypes.byref(self._lat),
                prm.ctypes.data_as(ctypes.c_void_p), self._stream))
            return
        self._moments_for(None)
        self.module.call(self.module.lib.lbm_m2f(self._mbuf().handle, ctypes.byref(self._mlat), self._F.handle,
                                                 ctypes.byref(self._lat), self._stream))

    def equilibrium(self):
        """Non-conserved moments of m set to their equilibrium values
        (pylbm/simulation.py:360-372).  They are computed when first read; a
        following ``m2f()`` needs only the conserved ones."""
        self._moments_ready()
        self._moments_for(0)
        self._eq_pending = True
        self._m_partial = False
        self._update_m = False

    def _materialize_equilibrium(self):
        """Write the pending equilibrium planes into the moment array."""
        self._eq_pending = False
        prm = self._prm(for_init=True)
        self.module.call(self.module.lib.lbm_equilibrium(self._mbuf().handle, ctypes.byref(self._mlat),
                                                         prm.ctypes.data_as(ctypes.c_void_p), self._stream))

    def relaxation(self):
        """m relaxed toward the equilibrium at the scheme's rates (pylbm/simulation.py:329-334)."""
        self._moments_ready()
        self._moments_for(None)
        prm = self._prm()
        self.module.call(self.module.lib.lbm_relaxation(self._mbuf().handle, ctypes.byref(self._mlat),
                                                        prm.ctypes.data_as(ctypes.c_void_p), self._stream))

    def source_term(self, fraction_of_time_step=1.0):
        """Source terms over half a time step on the moments of the interior
        (pylbm/simulation.py:336-341: the generated routine integrates
        m_c += dt/2 S_c(m), pylbm/algorithm/ode.py:11-16, and
        ``fraction_of_time_step`` is accepted and not used, as there)."""
        if not self.scheme.source_terms:
            raise ValueError("the scheme has no source terms")
        self._moments_ready()
        self._moments_for(None)
        prm = self._prm()
        self.module.call(self.module.lib.lbm_source_term(self._mbuf().handle, ctypes.byref(self._mlat),
                                                         prm.ctypes.data_as(ctypes.c_void_p), self._stream))

    def _plane_range(self, key):
        """(first, count, is_slice) of the moment planes a key names: an index,
        a conserved-moment symbol, or a slice of consecutive planes."""
        if isinstance(key, slice):
            r = range(*key.indices(self.scheme.nv))
            if len(r) == 0 or r.step != 1:
                raise IndexError("moment planes must be a non-empty run of consecutive indices")
            return r.start, len(r), True
        idx = self.scheme.consm[key] if isinstance(key, (sp.Symbol, sp.IndexedBase)) else int(key)
        if not 0 <= idx < self.scheme.nv:
            raise IndexError(f"moment {idx} of {self.scheme.nv}")
        return idx, 1, False

    def _stage(self, nbytes):
        """Dense device staging buffer of at least ``nbytes`` (kept between calls)."""
        cur = getattr(self, "_stage_buf", None)
        if cur is None or cur.nbytes < nbytes:
            if cur is not None:
                self.synchronize()
                cur.free()
            self._stage_buf = cur = runtime.DeviceBuffer(nbytes)
        return cur

    def _set_moment_halo(self, key, value):
        """The named plane(s) of the moment array take ``value`` (broadcast to
        the halo box); the other planes stay as they are (pylbm/simulation.py:
        210-213).  The dense array crosses to the device in one copy (at the
        link's full rate from pinned memory, ``runtime.pinned_empty``) and a
        kernel writes it into the padded layout."""
        if self._need_init:
            self._initialize()
        if self._eq_pending and not self._update_m:  # the other planes as pylbm's equilibrium() left them
            self._moments_for(None)
        first, count, many = self._plane_range(key)
        shape = ((count,) if many else ()) + tuple(self.domain.shape_halo)
        src = value if isinstance(value, np.ndarray) else np.asarray(value)
        if src.dtype != np.float64 or src.shape != shape or not src.flags["C_CONTIGUOUS"]:
            src = np.ascontiguousarray(np.broadcast_to(src.astype(np.float64, copy=False), shape))
        direct = runtime.mapped_device_pointer(src)
        if direct is None:  # one contiguous copy to the device, then into the layout
            stage = self._stage(src.nbytes)
            runtime.check(self._core.lbm_memcpy(stage.handle, src.ctypes.data_as(ctypes.c_void_p), src.nbytes,
                                                runtime.H2D, self._stream))
            direct = stage.handle
        # page-locked arrays are read by the kernel itself over the host link
        runtime.check(self._core.lbm_copy_planes(self._mbuf().handle, ctypes.byref(self._mlat), first, count, 1,
                                                 direct, 1, self._stream))
        self.synchronize()  # ``value`` may be a temporary
        for i in range(first, first + count):
            self._m_cache.pop(i, None)
        self._update_m = False
        self._m_partial = False

    def _drop_graph(self):
        if self._graph is not None:
            self._core.lbm_graph_destroy(self._graph)
        self._graph = None
        self._graph_key = None

    def _capture(self, prm):
        """Capture two steps (F -> Fnew -> F) into one executable graph."""
        self._drop_graph()
        runtime.check(self._core.lbm_graph_begin(self._stream))
        try:
            self._enqueue_step(self._F, self._Fnew, prm)
            self._enqueue_step(self._Fnew, self._F, prm)
        finally:
            g = ctypes.c_void_p()
            rc = self._core.lbm_graph_end(self._stream, ctypes.byref(g))
        runtime.check(rc)
        self._graph = g
        self._graph_key = (self._F.ptr, self._Fnew.ptr, tuple(prm), self._folded(), self.batch_boundary,
                           getattr(self, "closure_kernel", None))

    def run(self, nsteps, graph=True):
        """Advance ``nsteps`` time steps (same result as calling one_time_step)."""
        if self._need_init:
            self._initialize()
        nsteps = int(nsteps)
        timed = any(meth._timed for meth in self.bc.methods)
        if not graph or timed or nsteps < 2:
            for _ in range(nsteps):
                self.one_time_step()
            return
        prm = self._prm()
        if self._graph_key != (self._F.ptr, self._Fnew.ptr, tuple(prm), self._folded(), self.batch_boundary,
                               getattr(self, "closure_kernel", None)):
            self._capture(prm)
        for _ in range(nsteps // 2):
            runtime.check(self._core.lbm_graph_launch(self._graph, self._stream))
            self.t += self.dt
            self.t += self.dt
            self.nt += 2
        self._update_m = True
        self._eq_pending = False
        self._m_cache = {}
        if nsteps % 2:
            self.one_time_step()

    def synchronize(self):
        runtime.check(self._core.lbm_stream_synchronize(self._stream))

    # ------------------------------------------------------------------ access
    def _moments_for(self, idx):
        """Bring the device moment array up to date for plane ``idx`` (every
        plane when None): the conserved planes alone when only they are read."""
        need_all = idx is None or idx >= self.scheme.nconsm
        if self._update_m:
            self._eq_pending = False
        elif self._eq_pending and need_all:
            self._m_cache = {}
            self._materialize_equilibrium()
        if self._update_m or (need_all and self._m_partial):
            self._m_cache = {}
            entry = self.module.lib.lbm_f2m if need_all else self.module.lib.lbm_f2m_conserved
            self.module.call(entry(self._F.handle, ctypes.byref(self._lat), self._mbuf().handle,
                                   ctypes.byref(self._mlat), self._stream))
            self._update_m = False
            self._m_partial = not need_all

    def _moment_halo(self, key):
        idx = self.scheme.consm[key] if isinstance(key, (sp.Symbol, sp.IndexedBase)) else int(key)
        self._moments_for(idx)
        if idx not in self._m_cache:
            # the conserved moments (what users and writers read) come in one
            # device-to-host copy; other moments one plane at a time
            first, count = (0, self.scheme.nconsm) if idx < self.scheme.nconsm else (idx, 1)
            planes = np.empty(count * self._mlat.vstride, dtype=np.float64)
            self._mbuf().download(planes, offset=first * self._mlat.vstride * 8, stream=self._stream)
            for j in range(count):
                if first + j not in self._m_cache:
                    plane = planes[j * self._mlat.vstride:(j + 1) * self._mlat.vstride]
                    self._m_cache[first + j] = np.array(self._plane_view(plane, self._mlat))
        return self._m_cache[idx]

    def fields(self, out=None):
        """Conserved moments on the interior, {name: array}.

        One launch computes the conserved moments, one gathers their interior
        nodes into a dense device array, and one device-to-host copy brings
        them over: into ``out`` when given (float64, shape (nconsm, *interior),
        C-contiguous; page-locked memory from ``runtime.pinned_empty`` copies
        at the link's full rate), else into a new array.
        """
        if self._need_init:
            self._initialize()
        nc = self.scheme.nconsm
        shape = (nc,) + tuple(self.domain.shape_in)
        if out is None:
            out = np.empty(shape, dtype=np.float64)
        elif out.shape != shape or out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError(f"fields(out=...) needs a C-contiguous float64 array of shape {shape}")
        # page-locked arrays are written by the kernel itself over the host link
        direct = runtime.mapped_device_pointer(out)
        dst = direct if direct is not None else self._stage(out.nbytes).handle
        if self._update_m:
            # straight from the populations, without the moment array
            self.module.call(self.module.lib.lbm_f2m_conserved_dense(self._F.handle, ctypes.byref(self._lat), dst,
                                                                     self._stream))
        else:  # the moment array holds values the user set: read those
            runtime.check(self._core.lbm_copy_planes(self._mbuf().handle, ctypes.byref(self._mlat), 0, nc, 0,
                                                     dst, 0, self._stream))
        if direct is None:
            runtime.check(self._core.lbm_memcpy(out.ctypes.data_as(ctypes.c_void_p), dst, out.nbytes,
                                                runtime.D2H, self._stream))
        self.synchronize()
        names = sorted(self.scheme.consm.items(), key=lambda kv: kv[1])
        return {str(c): out[i] for c, i in names}

    def write_h5(self, filename, path="", timestep=None, vectors=None):
        """Write the conserved moments (and {name: [moment names]} vectors) as
        HDF5 + XDMF (pylbm/hdf5.py H5File, as used by the demos' ``save``)."""
        from .output import H5File

        h5 = H5File(None, filename, path, timestep)
        h5.set_grid(*self.domain.coords)
        fields = self.fields()
        used = set()
        for name, comps in (vectors or {}).items():
            h5.add_vector(name, [fields[c] for c in comps])
            used.update(comps)
        for name, arr in fields.items():
            if name not in used:
                h5.add_scalar(name, arr)
        h5.save()
        return h5

    def _inner(self):
        return tuple(slice(int(h), -int(h)) for h in self.domain.halo)

    @property
    def m_halo(self):
        """Moments on the whole box; assignment writes the device moment array
        (pylbm/simulation.py:200-213), which m2f turns into populations."""
        return _ItemAccess(self._moment_halo, self._set_moment_halo)

    @property
    def m(self):
        """Moments on the interior nodes (pylbm/simulation.py:216-224);
        ``sim.m[key, i0, ...]`` reads only the selected nodes."""
        return _ItemAccess(lambda key: self._moment_halo(key)[self._inner()], box=self._moment_box)

    def _box_args(self, index):
        """(start, count, step, squeeze axes) of interior indices (ints / slices)."""
        n = list(self.domain.shape_in)
        if len(index) > self.dim:
            raise IndexError(f"{len(index)} indices for a {self.dim}-D field")
        index = tuple(index) + (slice(None),) * (self.dim - len(index))
        start, count, step, squeeze = [], [], [], []
        for d, ix in enumerate(index):
            if isinstance(ix, slice):
                r = range(*ix.indices(n[d]))
                if len(r) == 0:
                    raise IndexError(f"empty selection on axis {d}")
                start.append(r.start)
                count.append(len(r))
                step.append(r.step)
            else:
                i = int(ix)
                if i < -n[d] or i >= n[d]:
                    raise IndexError(f"index {i} out of range for axis {d} of size {n[d]}")
                start.append(i % n[d])
                count.append(1)
                step.append(1)
                squeeze.append(d)
        return start, count, step, tuple(squeeze)

    def _gather(self, buf, lat, plane, index, raw_dtype):
        start, count, step, squeeze = self._box_args(index)
        total = int(np.prod(count))
        out = runtime.DeviceBuffer(total * np.dtype(raw_dtype).itemsize)
        a = [np.array(v + [0] * (3 - len(v)), dtype=np.int32) for v in (start, count, step)]
        runtime.check(self._core.lbm_gather(buf.handle, ctypes.byref(lat), int(plane),
                                            *[x.ctypes.data_as(ctypes.c_void_p) for x in a],
                                            out.handle, self._stream))
        host = np.empty(total, dtype=raw_dtype)
        out.download(host, stream=self._stream)
        out.free()
        return host.reshape(count).squeeze(axis=squeeze) if squeeze else host.reshape(count)

    def _moment_box(self, key, index):
        idx = self.scheme.consm[key] if isinstance(key, (sp.Symbol, sp.IndexedBase)) else int(key)
        self._moments_for(idx)
        return self._gather(self._mbuf(), self._mlat, idx, index, np.float64)

    def _population_box(self, k, index):
        raw = self._gather(self._F, self._lat, int(k), index, RAW_DTYPE[self.storage])
        return from_storage(raw, self.storage) + float(self._lat.shift[int(k)])

    def _population_halo(self, k):
        k = int(k)
        es = runtime.DTYPE_SIZE[self.storage]
        raw = np.empty(self._lat.vstride, dtype=RAW_DTYPE[self.storage])
        self._F.download(raw, offset=k * self._lat.vstride * es, stream=self._stream)
        vals = from_storage(raw, self.storage)
        return np.array(self._plane_view(vals, self._lat)) + float(self._lat.shift[k])

    def _set_population_halo(self, k, value):
        k = int(k)
        cur = self._population_halo(k)
        cur[...] = value
        es = runtime.DTYPE_SIZE[self.storage]
        plane = np.zeros(self._lat.vstride, dtype=np.float64)
        self._plane_view(plane, self._lat)[...] = cur - float(self._lat.shift[k])
        self._F.upload(to_storage(plane, self.storage), offset=k * self._lat.vstride * es, stream=self._stream)
        self._update_m = True
        self._m_cache = {}

    @property
    def F_halo(self):
        return _ItemAccess(self._population_halo, self._set_population_halo)

    @property
    def F(self):
        """Populations on the interior nodes (pylbm/simulation.py:248-256)."""
        return _ItemAccess(lambda k: self._population_halo(k)[self._inner()], box=self._population_box)

    # ------------------------------------------------------------------ checks
    def population_sums(self):
        """FP64 sum of every population over the interior, and the NaN/Inf count."""
        size = ctypes.c_size_t()
        runtime.check(self._core.lbm_population_sums_scratch_bytes(ctypes.byref(self._lat), ctypes.byref(size)))
        scratch = runtime.DeviceBuffer(size.value)
        out = runtime.DeviceBuffer(8 * self.scheme.nv + 8)
        runtime.check(self._core.lbm_population_sums(self._F.handle, ctypes.byref(self._lat), out.handle,
                                                     ctypes.c_void_p(out.ptr + 8 * self.scheme.nv), scratch.handle,
                                                     size.value, self._stream))
        host = np.empty(self.scheme.nv + 1, dtype=np.float64)
        out.download(host, stream=self._stream)
        sums = host[:self.scheme.nv]
        bad = int(np.frombuffer(host[self.scheme.nv:].tobytes()[:4], dtype=np.int32)[0])
        return sums, bad

    def conserved_sums(self):
        """FP64 totals of the conserved moments (mass, momentum, ...)."""
        sums, bad = self.population_sums()
        if bad:
            raise FloatingPointError(f"non-finite populations detected ({bad} blocks)")
        return self.scheme.M[:self.scheme.nconsm] @ sums

    def free(self):
        self._drop_graph()
        for b in (self._F, self._Fnew, self._M, getattr(self, "_stage_buf", None), getattr(self, "_fallbacks", None)):
            if b is not None:
                b.free()
        self._free_bc()
        if self._stream:
            self._core.lbm_stream_destroy(self._stream)
            self._stream = None

    def _free_bc(self):
        for dev in [d for _, d in self._bc_dev] + ([self._ghost] if self._ghost else []):
            for val in dev.values():
                for b in (val if isinstance(val, list) else [val]):
                    if isinstance(b, runtime.DeviceBuffer):
                        b.free()
        self._bc_dev = []
        self._ghost = None
        for tab in (self._bc_batch, self._ghost_alone):
            if tab is not None:
                tab[0].free()
        self._bc_batch = None
        self._ghost_alone = None
        for b in self._batch_bufs:
            b.free()
        self._batch_bufs = []
        self._batch_rhs = []

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
