"""Host stand-in for the device of pylbm_gb300.plugin (test infrastructure).

``HostDevice`` offers what ``plugin.CudaDevice`` offers -- the scheme's
module, the arrays, the list uploads -- with numpy arrays in the device
layout [nv, x, y(, z)] and every routine computed by the C oracle.  The
module's routines have the names and parameter names of
``generator.CudaModule`` (``routine_signatures``), so pylbm's own
``call_genfunction`` binds them exactly as it binds the CUDA module; every
call is recorded (routine, argument names) for the dispatch checks.
"""
import numpy as np

from oracle import _p, equilibrium_table, lib
from pylbm_gb300.generator import _routine, routine_signatures
from pylbm_gb300.scheme import Scheme


class HostArray:
    """numpy stand-in for generator.DeviceArray."""

    def __init__(self, nv, nspace, vmax):
        self.nv = int(nv)
        self.nspace = [int(n) for n in nspace]
        self.dim = len(self.nspace)
        self.vmax = [int(v) for v in np.broadcast_to(np.atleast_1d(vmax), (self.dim,))]
        self.shape = (self.nv, *self.nspace)
        self.data = np.zeros(self.shape)

    @property
    def n(self):
        return np.array([s - 2 * v for s, v in zip(self.nspace, self.vmax)] + [1] * (3 - self.dim), dtype=np.int32)

    @property
    def h(self):
        return np.array(self.vmax + [0] * (3 - self.dim), dtype=np.int32)

    def get(self):
        return self.data.copy()

    def copy(self):
        out = HostArray(self.nv, self.nspace, self.vmax)
        out.data[...] = self.data
        return out

    def set(self, values):
        self.data[...] = np.broadcast_to(values, self.shape)

    def __getitem__(self, key):
        if key == slice(None):
            return self
        return self.data[key]

    def __setitem__(self, key, value):
        if key == slice(None) and isinstance(value, HostArray):
            self.data[...] = value.data
        else:
            self.data[key] = value


class HostList:
    """numpy stand-in for generator.LinkArray."""

    def __init__(self, host):
        host = np.ascontiguousarray(host)
        self.host = np.ascontiguousarray(host, dtype=np.int32 if host.dtype.kind in "iu" else np.float64)
        self.shape = self.host.shape
        self.dtype = self.host.dtype

    def get(self):
        return self.host.copy()

    def __getitem__(self, key):
        return self.host[key]

    def __setitem__(self, key, value):
        self.host[key] = value


class HostModule:
    def __init__(self, dico, calls):
        sc = Scheme(dico)
        self.scheme = sc
        self.calls = calls
        self.params = [str(s) for s in sc.free_symbols]
        v = np.zeros((sc.nv, 3), dtype=np.int32)
        v[:, :sc.dim] = sc.stencil.get_all_velocities()
        self.vel = v
        self.M = np.ascontiguousarray(sc.M)
        self.invM = np.ascontiguousarray(sc.invM)
        impl = {"one_time_step": self._step, "f2m": self._f2m, "m2f": self._m2f, "equilibrium": self._equilibrium,
                "bounce_back": lambda **kw: self._boundary(kw, 1.0),
                "anti_bounce_back": lambda **kw: self._boundary(kw, -1.0),
                "Bouzidi_bounce_back": lambda **kw: self._bouzidi(kw, 0),
                "Bouzidi_anti_bounce_back": lambda **kw: self._bouzidi(kw, 1)}
        for name, args in routine_signatures(sc).items():
            if name.startswith("neumann"):
                fn = lambda **kw: self._boundary(kw, 0.0)  # noqa: E731
            elif name.startswith("update_"):
                fn = self._updater("xyz".index(name[-1]))
            elif name in impl:
                fn = impl[name]
            else:
                fn = self._not_used(name)
            setattr(self, name, _routine(name, args, self._recorded(name, fn)))

    def _recorded(self, name, fn):
        def call(**kw):
            self.calls.append((name, tuple(sorted(kw))))
            return fn(**kw)
        return call

    @staticmethod
    def _not_used(name):
        def fn(**kw):
            raise NotImplementedError(f"{name} is not exercised by these tests")
        return fn

    def _extra(self, kw):
        return {n: float(kw[n if n != "lambda" else "lambda_"]) for n in self.params}

    def _tables(self, kw):
        sc = self.scheme
        extra = self._extra(kw)
        return (np.ascontiguousarray(sc.rates_numpy(extra)),) + equilibrium_table(sc, extra)

    def _step(self, **kw):
        f, fnew = kw["f"], kw["fnew"]
        s, rows, coefs, expos = self._tables(kw)
        sc = self.scheme
        lib().oracle_one_time_step(_p(f.data), _p(fnew.data), sc.dim, sc.nv, sc.nconsm, _p(f.n), _p(f.h),
                                   _p(self.vel), _p(self.M), _p(self.invM), _p(s), len(rows), _p(rows), _p(coefs),
                                   _p(expos), 1)

    def _f2m(self, **kw):
        f, m = kw["f"], kw["m"]
        lib().oracle_f2m(_p(f.data), _p(m.data), f.dim, f.nv, _p(f.n), _p(f.h), _p(self.M))

    def _m2f(self, **kw):
        f, m = kw["f"], kw["m"]
        lib().oracle_m2f(_p(m.data), _p(f.data), f.dim, f.nv, _p(f.n), _p(f.h), _p(self.invM))

    def _equilibrium(self, **kw):
        m = kw["m"]
        _, rows, coefs, expos = self._tables(kw)
        lib().oracle_equilibrium(_p(m.data), m.dim, m.nv, self.scheme.nconsm, _p(m.n), _p(m.h), len(rows),
                                 _p(rows), _p(coefs), _p(expos))

    def _boundary(self, kw, sign):
        f = kw["f"]
        rhs = kw.get("rhs")
        lib().oracle_boundary(_p(f.data), f.dim, f.nv, _p(f.n), _p(f.h), _p(kw["iload0"].host),
                              _p(kw["istore"].host), int(kw["ncond"]), _p(rhs.host) if sign else None,
                              sign if sign else 1.0)

    def _bouzidi(self, kw, anti):
        f = kw["f"]
        lib().oracle_bouzidi(_p(f.data), f.dim, f.nv, _p(f.n), _p(f.h), _p(kw["iload0"].host),
                             _p(kw["iload1"].host), _p(kw["istore"].host), int(kw["ncond"]), _p(kw["rhs"].host),
                             _p(kw["dist"].host), anti)

    @staticmethod
    def _updater(axis):
        def update(**kw):
            f = kw["f"]
            a = f.data
            v = f.vmax[axis]
            n = f.nspace[axis]
            lo = [slice(None)] * a.ndim
            src = [slice(None)] * a.ndim
            lo[1 + axis], src[1 + axis] = slice(0, v), slice(n - 2 * v, n - v)
            a[tuple(lo)] = a[tuple(src)]
            lo[1 + axis], src[1 + axis] = slice(n - v, n), slice(v, 2 * v)
            a[tuple(lo)] = a[tuple(src)]
        return update


class HostDevice:
    """plugin device whose module, arrays and lists live on the host."""

    def __init__(self):
        self.calls = []
        self.modules = []

    def module(self, dico):
        mod = HostModule(dico, self.calls)
        self.modules.append(mod)
        return mod

    @staticmethod
    def array(nv, nspace, vmax):
        return HostArray(nv, nspace, vmax)

    @staticmethod
    def to_device(host):
        return host if isinstance(host, HostList) else HostList(host)
