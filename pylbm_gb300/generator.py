"""``generator.module`` for pylbm's backend 'CUDA': the routines pylbm calls by name.

pylbm compiles one module per scheme and calls its routines through
``call_genfunction`` (pylbm/symbolic.py:288-299), which reads the routine's
parameter names with ``inspect.getfullargspec`` and passes the values of the
same names from ``BaseAlgorithm._get_args`` (pylbm/algorithm/base.py:630-667)
or ``BoundaryMethod._get_args`` (pylbm/boundary.py:358-376).  ``CudaModule``
exposes those routines with the names and parameter names of the reference's
generated Cython module (recorded in tests/golden/ref_signatures.json) and
runs each through the C ABI of ``liblbm_gb300.so`` and the scheme's
``lbm_scheme_<hash>.so``:

=========================  ==========================================  =============================
routine                    reference (pylbm/...)                        C ABI
=========================  ==========================================  =============================
one_time_step              algorithm/base.py:551-600, pull.py:11-59     lbm_one_time_step
f2m / m2f                  algorithm/base.py:336-360                    lbm_f2m / lbm_m2f
equilibrium / relaxation   algorithm/base.py:298-335,361-402            lbm_equilibrium / lbm_relaxation
source_term                algorithm/base.py:439-504                    lbm_source_term
transport                  algorithm/base.py:403-428                    lbm_transport
bounce_back                boundary.py:400-469                          lbm_bounce_back
anti_bounce_back           boundary.py:626-684                          lbm_anti_bounce_back
neumann, neumannx/y/z      boundary.py:763-895                          lbm_neumann
Bouzidi_bounce_back        boundary.py:472-623                          lbm_bouzidi_bounce_back
Bouzidi_anti_bounce_back   boundary.py:687-760                          lbm_bouzidi_anti_bounce_back
update_x / _y / _z         storage.py:307-420 (one axis each)           lbm_update_halo_axis
=========================  ==========================================  =============================

The arrays pylbm passes (``Array.array`` of the containers, and the boundary
lists after ``move2gpu``) are ``DeviceArray`` / ``LinkArray`` objects: device
memory plus the shape and layout metadata the C ABI needs.  ``nx, ny, nz``
are pylbm's sizes with the ghost layers (``Array.nspace``) and are checked
against the arrays.  A link list whose loads read slots it also stores is
applied in link order, as pylbm's generated loop does; the Bouzidi
bounce-back reads a copy of f (``fcopy``), which the kernel reproduces with a
scratch of one value per link, so ``fcopy`` is accepted and not read.
"""
import ctypes
import inspect

import numpy as np

from . import runtime
from .codegen import SchemeSource
from .scheme import Scheme
from .simulation import RAW_DTYPE, from_storage, to_storage

_SPACE = ("nx", "ny", "nz")
_KW = inspect.Parameter.POSITIONAL_OR_KEYWORD


def _arg_name(symbol_name):
    """pylbm passes the parameter 'lambda' as 'lambda_' (base.py:660-662)."""
    return "lambda_" if symbol_name == "lambda" else symbol_name


def routine_signatures(scheme):
    """{routine: parameter names} of the module of ``scheme`` (a ``Scheme``).

    The boundary routines depend only on the dimension; the algorithm
    routines take the run-time parameters their expressions use: the
    equilibrium those of m_eq, the relaxation those of m_eq and the rates,
    the step all of them (``dt`` with source terms)."""
    space = list(_SPACE[:scheme.dim])
    names = [str(s) for s in scheme.free_symbols]
    eq = {str(s) for e in scheme.EQ for s in getattr(e, "free_symbols", ())}
    rates = {str(s) for r in scheme.s for s in getattr(r, "free_symbols", ())}

    def prm(keep):
        return [_arg_name(n) for n in names if n in keep]

    links = ["f", "iload0", "istore", "ncond"] + space
    sig = {
        "one_time_step": ["f", "fnew"] + space + prm(set(names)),
        "f2m": ["f", "m"] + space,
        "m2f": ["f", "m"] + space,
        "equilibrium": ["m"] + space + prm(eq),
        "relaxation": ["m"] + space + prm(eq | rates),
        "transport": ["f", "fnew"] + space,
        "bounce_back": links + ["rhs"],
        "anti_bounce_back": links + ["rhs"],
        "neumann": list(links),
        "Bouzidi_bounce_back": ["dist", "f", "fcopy", "iload0", "iload1", "istore", "ncond"] + space + ["rhs"],
        "Bouzidi_anti_bounce_back": ["dist", "f", "iload0", "iload1", "istore", "ncond"] + space + ["rhs"],
    }
    if scheme.source_terms:
        # pylbm generates source_term only for schemes with sources (base.py:616-617)
        src = {"dt"} | {str(s) for _, e in scheme.source_terms for s in getattr(e, "free_symbols", ())}
        sig["source_term"] = ["m"] + space + prm(src)
    for a in space:
        sig["neumann" + a[1]] = list(links)
        sig["update_" + a[1]] = ["f"] + space + ["nv"]
    return sig


class DeviceArray:
    """Populations or moments on the device: pylbm's ``Array.array`` for 'CUDA'.

    ``nspace`` counts the ghost layers (pylbm's ``Array.nspace``); the layout
    is structure of arrays with padded rows (``lbm_lattice_init``).  Stored
    populations of a shifted module are deviations from the module's
    reference equilibrium; ``get``/``set`` convert from and to float64 values
    of shape ``(nv, *nspace)``."""

    def __init__(self, nv, nspace, vmax, dtype="float64", shift=None):
        self.nv = int(nv)
        self.nspace = [int(n) for n in nspace]
        # one ghost width per axis, or one for every axis (pylbm passes 0 for
        # the boundary-value arrays of prepare_rhs, boundary.py:276-281)
        self.vmax = [int(v) for v in np.broadcast_to(np.atleast_1d(vmax), (len(self.nspace),))]
        self.dim = len(self.nspace)
        self.dtype = dtype
        shape_in = [n - 2 * h for n, h in zip(self.nspace, self.vmax)]
        if min(shape_in) < 1:
            raise ValueError(f"nspace {self.nspace} leaves no interior with vmax {self.vmax}")
        self.lattice = runtime.lattice(self.dim, self.nv, dtype, shape_in, self.vmax, shift=shift)
        self.shape = (self.nv, *self.nspace)
        self._es = runtime.DTYPE_SIZE[dtype]
        self.buffer = runtime.DeviceBuffer(max(self.lattice.elements * self._es, 8))
        runtime.check(runtime.core().lbm_memset(self.buffer.handle, 0, self.buffer.nbytes, None))

    @property
    def ptr(self):
        return self.buffer.handle

    def _view(self, raw):
        lat = self.lattice
        es = raw.itemsize
        return np.lib.stride_tricks.as_strided(
            raw[lat.origin:], shape=(self.nv, *self.nspace),
            strides=[lat.vstride * es] + [lat.stride[d] * es for d in range(self.dim)])

    def get(self):
        raw = np.empty(self.lattice.elements, dtype=RAW_DTYPE[self.dtype])
        self.buffer.download(raw)
        vals = np.array(self._view(from_storage(raw, self.dtype)))
        shift = np.array([self.lattice.shift[k] for k in range(self.nv)])
        return vals + shift.reshape((-1,) + (1,) * self.dim)

    def set(self, values):
        values = np.broadcast_to(np.asarray(values, dtype=np.float64), self.shape)
        shift = np.array([self.lattice.shift[k] for k in range(self.nv)])
        plane = np.zeros(self.lattice.elements, dtype=np.float64)
        self._view(plane)[...] = values - shift.reshape((-1,) + (1,) * self.dim)
        self.buffer.upload(to_storage(plane, self.dtype))

    @property
    def size(self):
        return int(np.prod(self.shape))

    def copy(self):
        """A new device array with the same values (pylbm's Bouzidi methods
        pass ``fcopy = f.copy()``, boundary.py:549; the kernels keep the copy
        semantics themselves and do not read it)."""
        out = DeviceArray(self.nv, self.nspace, self.vmax, self.dtype,
                          shift=[self.lattice.shift[k] for k in range(self.nv)])
        out[:] = self
        return out

    def __getitem__(self, key):
        """``a[:]`` is the whole array (pylbm copies F into Fnew with
        ``Fnew.array[:] = F.array[:]``, simulation.py:320)."""
        if key == slice(None) or key is Ellipsis:
            return self
        return self.get()[key]

    def __setitem__(self, key, value):
        if not (key == slice(None) or key is Ellipsis):
            host = self.get()
            host[key] = value
            self.set(host)
        elif isinstance(value, DeviceArray):
            if value.shape != self.shape or value.dtype != self.dtype:
                raise ValueError("device copy between arrays of different shape or type")
            runtime.check(runtime.core().lbm_memcpy(self.buffer.handle, value.buffer.handle,
                                                    self.buffer.nbytes, runtime.D2D, None))
            runtime.check(runtime.core().lbm_device_synchronize())
        else:
            self.set(value)

    def free(self):
        self.buffer.free()


class LinkArray:
    """A boundary list (iload, istore: int32 (ncond, dim+1); rhs, dist:
    float64 (ncond)) on the device, keeping its host copy."""

    def __init__(self, host):
        host = np.ascontiguousarray(host)
        if host.dtype.kind in "iu":
            host = np.ascontiguousarray(host, dtype=np.int32)
        else:
            host = np.ascontiguousarray(host, dtype=np.float64)
        self.host = host
        self.shape = host.shape
        self.dtype = host.dtype
        self.buffer = runtime.DeviceBuffer(max(host.nbytes, 8))
        if host.size:
            self.buffer.upload(host)

    @property
    def ptr(self):
        return self.buffer.handle

    def set(self, host):
        host = np.ascontiguousarray(host, dtype=self.dtype)
        if host.shape != self.shape:
            raise ValueError(f"shape {host.shape} != {self.shape}")
        self.host = host
        if host.size:
            self.buffer.upload(host)

    def get(self):
        return self.host.copy()

    def __getitem__(self, key):
        """Read the host copy (pylbm's set_rhs reads istore[:, 0] after move2gpu)."""
        return self.host[key]

    def __setitem__(self, key, value):
        """Write the host copy and upload it (pylbm's set_rhs assigns rhs[:] every step)."""
        host = self.host.copy()
        host[key] = value
        self.set(host)

    def free(self):
        self.buffer.free()


def to_device(array):
    """Upload a boundary list (what pylbm's ``move2gpu`` does for LOOPY)."""
    return array if isinstance(array, LinkArray) else LinkArray(array)


class CudaModule:
    """The generated module of one scheme for backend 'CUDA'.

    ``dico`` is a pylbm dictionary (or a ``Scheme``); ``storage`` the
    population type ("float64" computes in FP64; the others store shifted
    values and compute in FP32).  Routines are plain functions whose
    ``inspect.getfullargspec(...).args`` are the reference's parameter names,
    so ``call_genfunction`` can call them unchanged."""

    def __init__(self, dico, storage="float64", parity=True, c0=None):
        sc = dico if isinstance(dico, Scheme) else Scheme(dico)
        self.scheme = sc
        self.storage = storage
        self.compute = "float64" if storage == "float64" else "float32"
        shifted = storage != "float64"
        plain = sc.Tu is None and not sc.source_terms
        style = "reference" if (storage == "float64" and parity and plain) else "fast"
        if shifted and c0 is None:
            c0 = [1.0] + [0.0] * (sc.nconsm - 1)
        self.source = SchemeSource(sc, shifted, c0 if shifted else None, style=style,
                                   simplify_frame=self.compute == "float32")
        self.module = runtime.SchemeModule(self.source, storage, self.compute)
        self.core = runtime.core()
        self.params = [str(s) for s in sc.free_symbols]
        self.vmax = [int(v) for v in np.abs(sc.stencil.get_all_velocities()).max(axis=0)]
        self.signatures = routine_signatures(sc)
        self._scratch = {}
        self._order_cache = {}
        impl = {
            "one_time_step": self._one_time_step, "f2m": self._f2m, "m2f": self._m2f,
            "equilibrium": self._equilibrium, "relaxation": self._relaxation, "transport": self._transport,
            "source_term": self._source_term,
            "bounce_back": self._bounce_back, "anti_bounce_back": self._anti_bounce_back,
            "Bouzidi_bounce_back": self._bouzidi_bounce_back,
            "Bouzidi_anti_bounce_back": self._bouzidi_anti_bounce_back,
        }
        for name, args in self.signatures.items():
            if name.startswith("neumann"):
                fn = self._neumann
            elif name.startswith("update_"):
                fn = self._updater("xyz".index(name[-1]))
            else:
                fn = impl[name]
            setattr(self, name, _routine(name, args, fn))

    # ---------------------------------------------------------------- arrays
    def populations(self, nspace):
        """Zeroed population array (pylbm's F / Fnew) with halo width vmax."""
        return DeviceArray(self.scheme.nv, nspace, self.vmax, self.storage, shift=self.module.shift)

    def moments(self, nspace):
        """Zeroed float64 moment array (pylbm's m)."""
        return DeviceArray(self.scheme.nv, nspace, self.vmax, "float64")

    # --------------------------------------------------------------- helpers
    def _prm(self, kw):
        vals = [float(kw.get(_arg_name(n), 0.0)) for n in self.params]
        return np.array(vals + [0.0], dtype=np.float64)

    def _check(self, a, kw, what="f"):
        if not isinstance(a, DeviceArray):
            raise TypeError(f"{what} must be a DeviceArray, got {type(a).__name__}")
        for d, key in enumerate(_SPACE[:a.dim]):
            if key in kw and int(kw[key]) != a.nspace[d]:
                raise ValueError(f"{key}={kw[key]} but {what} has {a.nspace[d]} points on axis {d}")
        return ctypes.byref(a.lattice)

    def _links(self, f, kw, *names):
        out = []
        for n in names:
            a = kw[n]
            if not isinstance(a, LinkArray):
                a = LinkArray(a)
                kw[n] = a
            out.append(a)
        ncond = int(kw["ncond"])
        for a in out:
            if a.shape[0] < ncond:
                raise ValueError(f"list of {a.shape[0]} links for ncond={ncond}")
            if a.dtype == np.int32 and a.host.size:
                hi = np.array([f.nv] + f.nspace)
                if a.host.min() < 0 or np.any(a.host[:ncond].max(axis=0) >= hi):
                    raise ValueError("link list outside the lattice")
        return out

    def _ordered(self, istore, *loads):
        """1 when a load of the list reads a slot the list stores (link order matters)."""
        key = (id(istore),) + tuple(id(il) for il in loads)
        hit = self._order_cache.get(key)
        if hit is None or hit[0] is not istore:
            lists = [istore.host.astype(np.int64)] + [il.host.astype(np.int64) for il in loads]
            width = lists[0].shape[1]
            full = [a for a in lists if a.size]
            ext = tuple(int(e) + 1 for e in np.max([a.max(axis=0) for a in full], axis=0)) if full else (1,) * width

            def flat(a):
                return np.ravel_multi_index(tuple(a.T), ext) if a.size else np.zeros(0, np.int64)
            stored = flat(lists[0])
            ordered = int(any(np.isin(flat(a), stored).any() for a in lists[1:]))
            hit = self._order_cache[key] = (istore, ordered)
        return hit[1]

    # -------------------------------------------------------------- routines
    def _one_time_step(self, **kw):
        f, fnew = kw["f"], kw["fnew"]
        lat = self._check(f, kw)
        self._check(fnew, kw, "fnew")
        prm = self._prm(kw)
        self.module.call(self.module.lib.lbm_one_time_step(f.ptr, fnew.ptr, lat,
                                                           prm.ctypes.data_as(ctypes.c_void_p), None))

    def _f2m(self, **kw):
        f, m = kw["f"], kw["m"]
        self.module.call(self.module.lib.lbm_f2m(f.ptr, self._check(f, kw), m.ptr, self._check(m, kw, "m"), None))

    def _m2f(self, **kw):
        f, m = kw["f"], kw["m"]
        self.module.call(self.module.lib.lbm_m2f(m.ptr, self._check(m, kw, "m"), f.ptr, self._check(f, kw), None))

    def _equilibrium(self, **kw):
        m = kw["m"]
        prm = self._prm(kw)
        self.module.call(self.module.lib.lbm_equilibrium(m.ptr, self._check(m, kw, "m"),
                                                         prm.ctypes.data_as(ctypes.c_void_p), None))

    def _relaxation(self, **kw):
        m = kw["m"]
        prm = self._prm(kw)
        self.module.call(self.module.lib.lbm_relaxation(m.ptr, self._check(m, kw, "m"),
                                                        prm.ctypes.data_as(ctypes.c_void_p), None))

    def _source_term(self, **kw):
        m = kw["m"]
        prm = self._prm(kw)
        self.module.call(self.module.lib.lbm_source_term(m.ptr, self._check(m, kw, "m"),
                                                         prm.ctypes.data_as(ctypes.c_void_p), None))

    def _transport(self, **kw):
        f, fnew = kw["f"], kw["fnew"]
        self._check(fnew, kw, "fnew")
        self.module.call(self.module.lib.lbm_transport(f.ptr, fnew.ptr, self._check(f, kw), None))

    def _bounce_back(self, **kw):
        self._signed(kw, self.core.lbm_bounce_back)

    def _anti_bounce_back(self, **kw):
        self._signed(kw, self.core.lbm_anti_bounce_back)

    def _signed(self, kw, entry):
        f = kw["f"]
        lat = self._check(f, kw)
        il, st, rhs = self._links(f, kw, "iload0", "istore", "rhs")
        runtime.check(entry(f.ptr, il.ptr, st.ptr, int(kw["ncond"]), rhs.ptr, lat, self._ordered(st, il), None))

    def _neumann(self, **kw):
        f = kw["f"]
        lat = self._check(f, kw)
        il, st = self._links(f, kw, "iload0", "istore")
        runtime.check(self.core.lbm_neumann(f.ptr, il.ptr, st.ptr, int(kw["ncond"]), lat, self._ordered(st, il),
                                            None))

    def _bouzidi_bounce_back(self, **kw):
        f = kw["f"]
        lat = self._check(f, kw)
        il0, il1, st, rhs, dist = self._links(f, kw, "iload0", "iload1", "istore", "rhs", "dist")
        ncond = int(kw["ncond"])
        scratch = None
        if self._ordered(st, il0, il1):
            buf = self._scratch.get(ncond)
            if buf is None:
                buf = self._scratch[ncond] = runtime.DeviceBuffer(8 * max(ncond, 1))
            scratch = buf.handle
        runtime.check(self.core.lbm_bouzidi_bounce_back(f.ptr, il0.ptr, il1.ptr, st.ptr, ncond, rhs.ptr, dist.ptr,
                                                        lat, scratch, None))

    def _bouzidi_anti_bounce_back(self, **kw):
        f = kw["f"]
        lat = self._check(f, kw)
        il0, il1, st, rhs, dist = self._links(f, kw, "iload0", "iload1", "istore", "rhs", "dist")
        runtime.check(self.core.lbm_bouzidi_anti_bounce_back(f.ptr, il0.ptr, il1.ptr, st.ptr, int(kw["ncond"]),
                                                             rhs.ptr, dist.ptr, lat, self._ordered(st, il0, il1),
                                                             None))

    def _updater(self, axis):
        def update(**kw):
            f = kw["f"]
            runtime.check(self.core.lbm_update_halo_axis(f.ptr, self._check(f, kw), axis, None))
        return update


def _routine(name, args, impl):
    """A plain function named ``name`` whose parameters (as ``inspect`` sees
    them) are ``args``; it forwards them to ``impl`` by keyword."""
    def routine(**kw):
        missing = [a for a in args if a not in kw]
        if missing:
            raise TypeError(f"{name}() missing {missing}")
        return impl(**kw)
    routine.__name__ = routine.__qualname__ = name
    routine.__signature__ = inspect.Signature([inspect.Parameter(a, _KW) for a in args])
    return routine
