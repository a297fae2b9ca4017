"""Scheme constants from a pylbm scheme dictionary.

A pylbm scheme is described symbolically (pylbm/scheme.py:70 ``Scheme``):
moment polynomials P_i(X, Y, Z), equilibrium values of every moment as
functions of the conserved moments, relaxation rates s_i and the conserved
moments.  The hot path needs their numeric form:

* ``M[i, j] = P_i(v_j * la)`` (pylbm/scheme.py:464-532), built per elementary
  scheme and assembled block-diagonally, and its inverse.  Both are computed
  here in exact rational arithmetic after the parameters are substituted, then
  rounded once to float64.
* the conserved moments moved to the front by the same sequence of row swaps
  the reference applies (pylbm/scheme.py:225-241), so moment indices match
  ``sim.m[...]`` of the reference.
* the equilibrium of every moment as a sympy expression of the conserved
  moments (and of free symbols, which become run-time parameters, like the
  reference's ``extra_parameters``, pylbm/algorithm/base.py:663-666).
* the relaxation rates, numbers or free symbols.
"""
from collections import OrderedDict
from fractions import Fraction

import numpy as np
import sympy as sp

from .stencil import Stencil


class SchemeError(ValueError):
    """Raised for scheme dictionaries the CUDA backend does not handle."""


# velocity of the moving frame (pylbm/symbolic.py rel_ux, rel_uy, rel_uz) and
# the time step of the source-term integrator (pylbm/algorithm/ode.py:15)
REL_U = sp.symbols("rel_ux, rel_uy, rel_uz")
DT = sp.Symbol("dt")


def _box_dim(dico):
    if "dim" in dico and dico["dim"]:
        return int(dico["dim"])
    box = dico["box"]
    dim = 1
    if box.get("y") is not None:
        dim += 1
        if box.get("z") is not None:
            dim += 1
    return dim


def to_fraction(value):
    """Exact rational of a number or a numeric sympy expression."""
    if isinstance(value, Fraction):
        return value
    if isinstance(value, (int, np.integer)):
        return Fraction(int(value))
    if isinstance(value, (float, np.floating)):
        return Fraction(float(value))
    expr = sp.sympify(value)
    if expr.is_Integer:
        return Fraction(int(expr))
    if expr.is_Rational:
        return Fraction(int(expr.p), int(expr.q))
    if expr.is_Float:
        return Fraction(float(expr))
    expr = sp.nsimplify(expr, rational=True) if expr.free_symbols == set() else expr
    if expr.is_Rational:
        return Fraction(int(expr.p), int(expr.q))
    val = complex(sp.N(expr, 30))
    if val.imag != 0:
        raise SchemeError(f"non-real constant {expr}")
    return Fraction(val.real)


def exact_inverse(mat):
    """Gauss-Jordan inverse of a square matrix of Fractions."""
    n = len(mat)
    a = [list(row) + [Fraction(int(i == j)) for j in range(n)] for i, row in enumerate(mat)]
    for col in range(n):
        piv = next((r for r in range(col, n) if a[r][col] != 0), None)
        if piv is None:
            raise SchemeError("the moment matrix M is singular")
        a[col], a[piv] = a[piv], a[col]
        p = a[col][col]
        a[col] = [x / p for x in a[col]]
        for r in range(n):
            if r != col and a[r][col] != 0:
                fac = a[r][col]
                a[r] = [x - fac * y for x, y in zip(a[r], a[col])]
    return [row[n:] for row in a]


class Scheme:
    """Numeric description of a pylbm scheme dictionary.

    Attributes
    ----------
    stencil : Stencil
    nv : int                     total number of populations (sum over schemes)
    M_frac, invM_frac : list     exact M and M^-1 (conserved moments in front)
    M, invM : ndarray            float64 copies
    consm : OrderedDict          conserved symbol -> moment index (0..nconsm-1)
    EQ : list of sympy exprs     equilibrium of every moment, in conserved symbols
    s : list                     relaxation rates (floats or sympy symbols)
    free_symbols : list          symbols that are run-time parameters
    """

    def __init__(self, dico):
        self.dico = dico
        self.dim = _box_dim(dico)
        schemes = dico["schemes"]
        self.stencil = Stencil.from_dico(dico, self.dim)
        self.nv = self.stencil.nvtot
        self.param = dict(dico.get("parameters", {}) or {})
        la = dico["scheme_velocity"]
        self.la_expr = sp.sympify(la)
        la_val = self.la_expr.subs(list(self.param.items()))
        self.la = to_fraction(la_val)
        self.la_float = float(self.la)
        for s in schemes:
            if "feq" in s and s["feq"]:
                raise SchemeError("'feq' equilibria are not supported; give 'equilibrium'")
            if "M" in s:
                raise SchemeError("explicit 'M' matrices are not supported; give 'polynomials'")
        coords = [self.param.get(k, sp.Symbol(n)) for k, n in
                  (("space_x", "X"), ("space_y", "Y"), ("space_z", "Z"))]
        self.symb_coord = coords

        # moment matrix, block diagonal over elementary schemes
        nv = self.nv
        mfrac = [[Fraction(0)] * nv for _ in range(nv)]
        polys = []
        self.rel_vel_symbols = list(REL_U[:self.dim])
        rel_vel = dico.get("relative_velocity")
        mu_rows = [[sp.Integer(0)] * nv for _ in range(nv)] if rel_vel is not None else None
        la_sym = sp.Rational(self.la.numerator, self.la.denominator)
        for isch, s in enumerate(schemes):
            v = [self._vel(n) for n in self.stencil.num(isch)]
            base = int(self.stencil.nv_ptr[isch])
            plist = list(s["polynomials"])
            if len(plist) != len(v):
                raise SchemeError(f"scheme {isch}: {len(plist)} polynomials for {len(v)} velocities")
            for i, p in enumerate(plist):
                p = sp.sympify(p).subs(list(self.param.items()))
                polys.append(p)
                for j, vj in enumerate(v):
                    subs = {coords[d]: sp.Rational(vj[d]) * sp.Rational(self.la.numerator, self.la.denominator)
                            for d in range(self.dim)}
                    # substitute by name as well, as the reference does (str keys)
                    subs_named = [(str(coords[d]), subs[coords[d]]) for d in range(self.dim)]
                    val = p.subs(subs_named)
                    mfrac[base + i][base + j] = to_fraction(sp.nsimplify(val, rational=True))
                    if mu_rows is not None:
                        # moments of the populations seen from a frame moving at u
                        # (pylbm/scheme.py:494-500): P_i(v_j la - u)
                        pr = sp.nsimplify(p, rational=True)
                        shifted = [(str(coords[d]), sp.Rational(vj[d]) * la_sym - REL_U[d]) for d in range(self.dim)]
                        mu_rows[base + i][base + j] = sp.expand(pr.subs(shifted))
        self.polynomials = polys

        eq = []
        for isch, s in enumerate(schemes):
            eqs = list(s["equilibrium"])
            if len(eqs) != self.stencil.nv[isch]:
                raise SchemeError(f"scheme {isch}: wrong number of equilibrium values")
            eq.extend(sp.sympify(e) for e in eqs)
        rates = []
        for isch, s in enumerate(schemes):
            rr = list(s["relaxation_parameters"])
            if len(rr) != self.stencil.nv[isch]:
                raise SchemeError(f"scheme {isch}: wrong number of relaxation parameters")
            rates.extend(rr)

        # conserved moments: index of the moment whose equilibrium is the symbol itself
        consm = OrderedDict()
        for isch, s in enumerate(schemes):
            cm = s.get("conserved_moments")
            if cm is None:
                continue
            if isinstance(cm, (sp.Symbol, sp.IndexedBase, str)):
                cm = [cm]
            leq = eq[self.stencil.nv_ptr[isch]:self.stencil.nv_ptr[isch + 1]]
            for c in cm:
                c = sp.Symbol(c) if isinstance(c, str) else c
                consm[c] = int(self.stencil.nv_ptr[isch]) + leq.index(c)

        # move the conserved moments in front with the reference's swap sequence
        perm = list(range(nv))
        for ic, c in enumerate(list(consm.values())):
            perm[ic], perm[c] = perm[c], perm[ic]
            eq[ic], eq[c] = eq[c], eq[ic]
            rates[ic], rates[c] = rates[c], rates[ic]
            mfrac[ic], mfrac[c] = mfrac[c], mfrac[ic]
            if mu_rows is not None:
                mu_rows[ic], mu_rows[c] = mu_rows[c], mu_rows[ic]
        for ic, c in enumerate(list(consm.keys())):
            consm[c] = ic
        self.consm = consm
        self.nconsm = len(consm)
        self.moment_perm = perm

        self.M_frac = mfrac
        self.invM_frac = exact_inverse(mfrac)
        self.M = np.array([[float(x) for x in row] for row in mfrac])
        self.invM = np.array([[float(x) for x in row] for row in self.invM_frac])
        psubs = list(self.param.items())

        # relative velocity (pylbm/scheme.py:149, :494-532): T(u) maps the
        # moments M f to the moments P_i(v la - u) f of a frame moving at u;
        # with M and M^-1 already permuted, T(u) = M_u M^-1 is permuted alike
        self.Tu = self.Tmu = self.rel_vel = None
        if mu_rows is not None:
            inv = sp.Matrix([[sp.Rational(x.numerator, x.denominator) for x in row] for row in self.invM_frac])
            tu = (sp.Matrix(mu_rows) * inv).applyfunc(sp.expand)
            self.Tu = tu
            self.Tmu = tu.subs(list(zip(REL_U, [-u for u in REL_U])), simultaneous=True).applyfunc(sp.expand)
            if len(rel_vel) != self.dim:
                raise SchemeError("relative_velocity needs one expression per space dimension")
            self.rel_vel = [sp.nsimplify(sp.sympify(e).subs(psubs), rational=True) for e in rel_vel]

        # source terms (pylbm/algorithm/base.py:141-150, :439-495): conserved
        # moment -> right-hand side, integrated by explicit Euler over dt/2
        # before and after the relaxation
        self.source_terms = []
        for isch, s in enumerate(schemes):
            for key, val in (s.get("source_terms") or {}).items():
                key = sp.Symbol(key) if isinstance(key, str) else key
                if key not in consm:
                    raise SchemeError(f"source term on {key}, which is not a conserved moment")
                rhs = sp.sympify(val).subs(psubs)
                rhs = rhs if rhs.free_symbols else sp.nsimplify(rhs, rational=True)
                bad = rhs.free_symbols & ({c for c in coords if isinstance(c, sp.Symbol)} | {sp.Symbol("t")})
                if bad:
                    raise SchemeError(f"source terms depending on {sorted(map(str, bad))} are not supported")
                self.source_terms.append((consm[key], rhs))

        # equilibrium and rates with parameters substituted
        self.EQ = [sp.nsimplify(sp.sympify(e).subs(psubs)) if sp.sympify(e).subs(psubs).free_symbols
                   else sp.nsimplify(sp.sympify(e).subs(psubs), rational=True) for e in eq]
        self.s = []
        for r in rates:
            r = sp.sympify(r).subs(psubs)
            if r.free_symbols:
                self.s.append(r)
            else:
                self.s.append(float(r))
        cons_syms = set(consm.keys())
        free = set()
        for e in self.EQ:
            free |= e.free_symbols
        for r in self.s:
            if isinstance(r, sp.Expr):
                free |= r.free_symbols
        for e in (self.rel_vel or []):
            free |= e.free_symbols
        for _, e in self.source_terms:
            free |= e.free_symbols
        if self.source_terms:
            free.add(DT)
        coord_syms = {c for c in coords if isinstance(c, sp.Symbol)}
        if free & coord_syms:
            raise SchemeError("space-dependent equilibria are not supported by the CUDA backend")
        self.free_symbols = sorted(free - cons_syms, key=lambda x: x.name)
        for k in range(self.nconsm):
            if self.EQ[k] != list(consm.keys())[k]:
                raise SchemeError("conserved moment equilibrium mismatch")

    def _vel(self, num):
        from .stencil import velocity
        return velocity(self.dim, int(num))

    # -- host-side evaluation (float64), used for boundary values and checks --
    def equilibrium_numpy(self, cons, params=None):
        """Equilibrium moments (nv, n) from conserved moments ``cons`` (nconsm, n)."""
        params = params or {}
        cons = np.asarray(cons, dtype=np.float64)
        n = cons.shape[1]
        syms = list(self.consm.keys()) + list(self.free_symbols)
        needed = set().union(*(e.free_symbols for e in self.EQ))

        def value(s):
            if s not in needed:  # e.g. the time step of source terms: not in the equilibrium
                return np.zeros(n)
            return np.full(n, float(params[str(s)] if str(s) in params else params[s]))

        vals = [cons[i] for i in range(self.nconsm)] + [value(s) for s in self.free_symbols]
        out = np.empty((self.nv, n))
        for k, e in enumerate(self.EQ):
            f = sp.lambdify(syms, e, "numpy")
            out[k] = np.broadcast_to(np.asarray(f(*vals), dtype=np.float64), (n,))
        return out

    def feq_numpy(self, cons, params=None):
        """Equilibrium populations ``invM . meq(cons)``, shape (nv, n)."""
        return self.invM @ self.equilibrium_numpy(cons, params)

    def rates_numpy(self, params=None):
        params = params or {}
        out = np.empty(self.nv)
        for k, r in enumerate(self.s):
            if isinstance(r, sp.Expr):
                out[k] = float(r.subs({s: params[str(s)] if str(s) in params else params[s] for s in r.free_symbols}))
            else:
                out[k] = r
        return out
