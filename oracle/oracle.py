"""Python driver of the C oracle (oracle/lbm_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of bench.py to check and time the GPU path.  The
pylbm_gb300 package never imports it.

``OracleSimulation`` replays pylbm's time step on the CPU in float64 with the
reference's own order of operations (pylbm/simulation.py:374-420):
periodic ghost exchange of every axis, boundary methods in list order, pull
step on the interior, swap.  Scheme constants, domain and boundary lists come
from pylbm_gb300's host code, which the golden fixtures pin against the
reference separately.
"""
import ctypes
import os
import subprocess

import numpy as np
import sympy as sp

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liblbm_oracle.so")
SRC = os.path.join(HERE, "lbm_oracle.c")


def build(force=False):
    """Compile the oracle with gcc (OpenMP) into oracle/_build/."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-o", tmp, SRC, "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P, I = ctypes.c_void_p, ctypes.c_int
        L.oracle_update_halo.argtypes = [P, I, I, P, P]
        L.oracle_boundary.argtypes = [P, I, I, P, P, P, P, I, P, ctypes.c_double]
        L.oracle_bouzidi.argtypes = [P, I, I, P, P, P, P, P, I, P, P, I]
        L.oracle_one_time_step.argtypes = [P, P, I, I, I, P, P, P, P, P, P, I, P, P, P, I]
        L.oracle_f2m.argtypes = [P, P, I, I, P, P, P]
        L.oracle_m2f.argtypes = [P, P, I, I, P, P, P]
        L.oracle_equilibrium.argtypes = [P, I, I, I, P, P, I, P, P, P]
        for fn in ("oracle_update_halo", "oracle_boundary", "oracle_bouzidi", "oracle_one_time_step", "oracle_f2m",
                   "oracle_m2f", "oracle_equilibrium"):
            getattr(L, fn).restype = None
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def equilibrium_table(scheme, params=None):
    """Monomial table (rows, coefs, exponents) of the scheme's equilibria."""
    params = {str(k): v for k, v in (params or {}).items()}
    cons = list(scheme.consm.keys())
    rows, coefs, expos = [], [], []
    for k in range(scheme.nconsm, scheme.nv):
        e = scheme.EQ[k]
        e = e.subs({s: params[str(s)] for s in e.free_symbols if str(s) in params})
        e = sp.expand(e)
        for term in sp.Add.make_args(e):
            if term == 0:
                continue
            coef, facs = term.as_coeff_mul()
            ex = [0] * len(cons)
            c = float(coef)
            for fac in facs:
                base, p = fac.as_base_exp()
                if base in cons and p.is_Integer:
                    ex[cons.index(base)] += int(p)
                elif not fac.free_symbols:
                    c *= float(fac)
                else:
                    raise ValueError(f"equilibrium term {term} is not a monomial of the conserved moments")
            rows.append(k)
            coefs.append(c)
            expos.append(ex)
    return (np.array(rows, dtype=np.int32), np.array(coefs, dtype=np.float64),
            np.ascontiguousarray(np.array(expos, dtype=np.int32).reshape(len(rows), len(cons))))


class OracleSimulation:
    """CPU float64 replay of a pylbm simulation (same dictionary)."""

    def __init__(self, dico, nthreads=1):
        from pylbm_gb300.boundary import Boundary
        from pylbm_gb300.domain import Domain
        from pylbm_gb300.scheme import Scheme

        self.scheme = Scheme(dico)
        self.domain = Domain(dico, self.scheme.stencil)
        self.dim = self.domain.dim
        self.nthreads = int(nthreads)
        self.extra_parameters = {}
        self.n = np.array(self.domain.shape_in, dtype=np.int32)
        self.h = np.array(self.domain.halo, dtype=np.int32)
        sc = self.scheme
        v = np.zeros((sc.nv, 3), dtype=np.int32)
        v[:, :self.dim] = sc.stencil.get_all_velocities()
        self.vel = v
        self.M = np.ascontiguousarray(sc.M)
        self.invM = np.ascontiguousarray(sc.invM)
        shape = [sc.nv] + self.domain.shape_halo
        self.f = np.zeros(shape)
        self.fnew = np.zeros(shape)
        self.dico = dico
        self.bc = Boundary(self.domain, dico)
        for meth in self.bc.methods:
            meth.set_iload()
        self.t = 0.0
        self.nt = 0
        self.dt = self.domain.dx / sc.la_float
        self.after_halo = None
        self.boundary_phase = None
        self._ready = False

    def extra_parameters_str(self):
        return {str(k): v for k, v in self.extra_parameters.items()}

    def _tables(self):
        sc = self.scheme
        s = sc.rates_numpy(self.extra_parameters_str())
        rows, coefs, expos = equilibrium_table(sc, self.extra_parameters_str())
        return np.ascontiguousarray(s), rows, coefs, expos

    def initialize(self):
        sc = self.scheme
        coords = np.meshgrid(*self.domain.coords_halo, sparse=True, indexing="ij")
        m = np.zeros_like(self.f)
        init_type = self.dico.get("inittype", "moments")
        for key, val in (self.dico.get("init") or {}).items():
            idx = sc.consm[key] if init_type == "moments" and isinstance(key, sp.Basic) else int(key)
            if isinstance(val, tuple):
                m[idx] = val[0](*(tuple(coords) + (tuple(val[1]) if len(val) == 2 else ())))
            elif callable(val):
                m[idx] = val(*coords)
            else:
                m[idx] = val
        if init_type == "moments":
            if self._monomial_equilibrium():
                s, rows, coefs, expos = self._tables()
                lib().oracle_equilibrium(_p(m), self.dim, sc.nv, sc.nconsm, _p(self.n), _p(self.h), len(rows),
                                         _p(rows), _p(coefs), _p(expos))
            else:  # equilibrium of the whole halo box from the conserved moments (NumPy)
                cons = m[:sc.nconsm].reshape(sc.nconsm, -1)
                m = sc.equilibrium_numpy(cons, self.extra_parameters_str()).reshape(m.shape)
                m = np.ascontiguousarray(m)
            lib().oracle_m2f(_p(m), _p(self.f), self.dim, sc.nv, _p(self.n), _p(self.h), _p(self.invM))
        else:
            self.f[...] = m
        self.fnew[...] = self.f
        for meth in self.bc.methods:
            meth.prepare_rhs(self)
            meth.fix_iload()
            meth.set_rhs()
        self._ready = True

    def one_time_step(self):
        if not self._ready:
            self.initialize()
        sc = self.scheme
        L = lib()
        if self.boundary_phase is not None:  # tests: an alternative ghost refresh + boundary phase
            self.boundary_phase(self.f)
            methods = []
        else:
            L.oracle_update_halo(_p(self.f), self.dim, sc.nv, _p(self.n), _p(self.h))
            methods = self.bc.methods
        if self.after_halo is not None:  # tests: observe the populations after the refresh
            self.after_halo(self.f)
        for meth in methods:
            if meth.update_feq(self):
                meth.set_rhs()
            if meth.kind.startswith("bouzidi"):
                dist = np.ascontiguousarray(meth.s, dtype=np.float64)
                L.oracle_bouzidi(_p(self.f), self.dim, sc.nv, _p(self.n), _p(self.h), _p(meth.iload[0]),
                                 _p(meth.iload[1]), _p(meth.istore), meth.ncond, _p(meth.rhs), _p(dist),
                                 1 if meth.kind == "bouzidi_anti_bounce_back" else 0)
                continue
            sign = -1.0 if meth.kind == "anti_bounce_back" else 1.0
            rhs = meth.rhs if meth.kind != "neumann" else None
            L.oracle_boundary(_p(self.f), self.dim, sc.nv, _p(self.n), _p(self.h), _p(meth.iload[0]),
                              _p(meth.istore), meth.ncond, _p(rhs) if rhs is not None else None, sign)
        if sc.Tu is not None or sc.source_terms or not self._monomial_equilibrium():
            self._frame_step()
        else:
            s, rows, coefs, expos = self._tables()
            L.oracle_one_time_step(_p(self.f), _p(self.fnew), self.dim, sc.nv, sc.nconsm, _p(self.n), _p(self.h),
                                   _p(self.vel), _p(self.M), _p(self.invM), _p(s), len(rows), _p(rows), _p(coefs),
                                   _p(expos), self.nthreads)
        self.f, self.fnew = self.fnew, self.f
        self.t += self.dt
        self.nt += 1

    def run(self, nsteps):
        for _ in range(int(nsteps)):
            self.one_time_step()

    def _monomial_equilibrium(self):
        """The C step takes the equilibrium as monomials with integer exponents;
        others (e.g. u^(-2/3) of the p-system) go through the NumPy step."""
        if not hasattr(self, "_monomial"):
            try:
                equilibrium_table(self.scheme, self.extra_parameters_str())
                self._monomial = True
            except ValueError:
                self._monomial = False
        return self._monomial

    # ---------------------------------------------------------------- relative velocity / sources
    def _frame_functions(self):
        """NumPy functions of the conserved moments, u and m (built once per parameter set)."""
        from pylbm_gb300.scheme import DT
        sc = self.scheme
        key = tuple(sorted(self.extra_parameters_str().items()))
        if getattr(self, "_frame_key", None) == key:
            return self._frame
        vals = dict(self.extra_parameters_str())
        vals["dt"] = self.dt
        prm = {sym: vals[str(sym)] for sym in sc.free_symbols}
        cons = list(sc.consm.keys())
        msym = sp.symbols(f"m0:{sc.nv}")
        u = list(sc.rel_vel_symbols)
        to_m = dict(zip(cons, msym[:sc.nconsm]))
        args = list(msym) + u

        def fn(exprs):
            exprs = [sp.sympify(e).subs(prm).subs(to_m) for e in exprs]
            return [sp.lambdify(args, e, "numpy") for e in exprs]

        out = {"rel": fn(sc.rel_vel) if sc.Tu is not None else None}
        eq = sp.Matrix(sc.EQ)
        if sc.Tu is not None:
            out["to_rel"] = fn([sum(sc.Tu[k, l] * msym[l] for l in range(sc.nv)) for k in range(sc.nv)])
            out["back"] = fn([sum(sc.Tmu[k, l] * msym[l] for l in range(sc.nv)) for k in range(sc.nv)])
            eq = sc.Tu * eq
        out["eq"] = fn(list(eq))
        out["src"] = [(k, f) for (k, _), f in zip(sc.source_terms,
                                                   fn([cons[k] + DT / 2 * rhs for k, rhs in sc.source_terms]))]
        out["s"] = sc.rates_numpy(self.extra_parameters_str())
        self._frame, self._frame_key = out, key
        return out

    def _frame_step(self):
        """PullAlgorithm.one_time_step_local (pylbm/algorithm/pull.py:11-59) with
        a relative velocity (base.py f2m_local :298-334, relaxation_local
        :404-428, restore_conserved_moments :255-263, m2f_local :346-369)
        and/or source terms (source_term_local :439-495): conserved moments
        M f, u = rel_vel(m), non-conserved moments T(u) M f, sources over
        dt/2, relaxation towards T(u) m_eq, conserved moments replaced by
        (T(u) M f)_c, sources over dt/2, f = M^-1 T(-u) m.  Float64 NumPy,
        whole interior at once."""
        sc = self.scheme
        fn = self._frame_functions()
        nv, nc, dim = sc.nv, sc.nconsm, self.dim
        h, n = self.h, self.n
        pulled = np.empty((nv,) + tuple(int(x) for x in n))
        for k in range(nv):
            sl = tuple(slice(int(h[d]) - int(self.vel[k, d]), int(h[d]) - int(self.vel[k, d]) + int(n[d]))
                       for d in range(dim))
            pulled[k] = self.f[(k,) + sl]
        m = np.tensordot(self.M, pulled, axes=1)
        zero = np.zeros_like(m[0])
        u = [zero + f(*m, *([zero] * dim)) for f in fn["rel"]] if fn["rel"] else []
        rel = None
        if u:
            rel = [zero + f(*m, *u) for f in fn["to_rel"]]
            for k in range(nc, nv):
                m[k] = rel[k]
        u_args = u if u else [zero] * dim

        def sources():
            new = [(k, zero + f(*m, *u_args)) for k, f in fn["src"]]
            for k, v in new:
                m[k] = v

        sources()
        eq = [zero + f(*m, *u_args) for f in fn["eq"]]
        for k in range(nv):
            if fn["s"][k] != 0.0:
                m[k] = m[k] + fn["s"][k] * (eq[k] - m[k])
        if rel is not None:  # restore_conserved_moments (pylbm/algorithm/base.py:255-263, pull.py:48-49)
            for k in range(nc):
                m[k] = rel[k]
        sources()
        if u:
            m = np.array([zero + f(*m, *u) for f in fn["back"]])
        inner = tuple(slice(int(h[d]), int(h[d]) + int(n[d])) for d in range(dim))
        self.fnew[(slice(None),) + inner] = np.tensordot(self.invM, m, axes=1)

    def source_term(self, m):
        """pylbm's standalone source_term (pylbm/algorithm/base.py:439-504,
        ode.py:11-16) on a halo-box moment array m[nv, ...]: every conserved
        moment with a source gets m_c + dt/2 S_c(m) on the interior nodes, from
        the moments as they were; returns a new array."""
        fn = self._frame_functions()
        out = np.array(m, dtype=np.float64)
        inner = tuple(slice(int(self.h[d]), int(self.h[d]) + int(self.n[d])) for d in range(self.dim))
        mi = [out[(k,) + inner] for k in range(self.scheme.nv)]
        zero = np.zeros_like(mi[0])
        new = [(k, zero + f(*mi, *([zero] * self.dim))) for k, f in fn["src"]]
        for k, v in new:
            out[(k,) + inner] = v
        return out

    def moments_halo(self):
        sc = self.scheme
        m = np.zeros_like(self.f)
        lib().oracle_f2m(_p(self.f), _p(m), self.dim, sc.nv, _p(self.n), _p(self.h), _p(self.M))
        return m

    def moments(self):
        inner = (slice(None),) + tuple(slice(int(h), -int(h)) for h in self.h)
        return self.moments_halo()[inner]

    # boundary methods call back into these (prepare_rhs / update_feq)
    @property
    def _mlist(self):
        return None
