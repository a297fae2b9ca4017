"""Reference-faithful float64 forms of the per-node algebra.

pylbm's Cython generator does not evaluate M f, the relaxation and M^-1 m
with exact constants: it prints sympy expressions as C, where rationals are
printed with 16 significant digits and floats (every constant that went
through a float parameter such as ``la = 1.0``) with 15
(pylbm/generator/printing/cython.py:72-210), and the relaxation is printed in
the factored form produced by ``alltogether`` (expand, together, factor;
pylbm/symbolic.py:259-275, pylbm/algorithm/base.py:404-428).  The generated
scheme is therefore a slightly perturbed version of the exact one, and two
float64 codes with different constants drift apart by ~1e-12 in a thousand
steps of a high-Reynolds flow.

The float64 parity module is generated from these forms: the same symbolic
pipeline (moment matrix in the scheme velocity, its inverse, conserved moments
moved in front, parameters substituted, relaxation factored), printed by a
sympy code printer with the same number formatting and the same term and
factor order, then compiled without fused multiply-adds.  Its arithmetic is
then the reference's arithmetic.
"""
import numpy as np
import sympy as sp
from sympy.printing.c import C99CodePrinter
from sympy.printing.str import StrPrinter

from .stencil import velocity

# the names pylbm's generator gives its loop indices and sizes
_nx, _ny, _nz, _nv = sp.symbols("nx, ny, nz, nv", integer=True)
_ix_, _iy_, _iz_ = sp.symbols("ix_, iy_, iz_", integer=True)


def _alltogether(M, nsimplify=False):
    for i in range(M.shape[0]):
        for j in range(M.shape[1]):
            e = M[i, j].expand().together().factor()
            M[i, j] = e.nsimplify() if nsimplify else e


def _recursive_sub(expr, replace):
    new = expr
    for _ in range(len(replace)):
        new = expr.subs(replace)
        if new == expr:
            return new
        expr = new
    return new


def _set_order(array, priority):
    return [array[p] for p in np.argsort(priority)]


class _Printer(C99CodePrinter):
    """C printer with the reference printer's number and power conventions."""

    def __init__(self, names):
        super().__init__({"full_prec": "auto", "precision": 16})
        self._names = names

    def _print_Float(self, expr):
        return StrPrinter._print_Float(self, expr)

    def _print_Rational(self, expr):
        return self._print(expr.evalf(16))

    def _print_Integer(self, expr):
        return StrPrinter._print_Integer(self, expr)

    def _print_Pow(self, expr):
        prec = sp.printing.precedence.precedence(expr)
        if expr.exp == -1:
            return "1.0/%s" % self.parenthesize(expr.base, prec)
        if expr.exp == 0.5:
            return "sqrt(%s)" % self._print(expr.base)
        if expr.exp > 0 and expr.exp.is_integer:
            b = self.parenthesize(expr.base, prec)
            return "(%s)" % "*".join([b] * int(expr.exp))
        return "pow(%s, %s)" % (self._print(expr.base), self._print(expr.exp))

    def _print_Indexed(self, expr):
        key = self._names.get(expr)
        if key is None:
            raise KeyError(f"unmapped indexed object {expr}")
        return key

    def _print_MatrixElement(self, expr):
        key = self._names.get(expr)
        if key is None:
            raise KeyError(f"unmapped matrix element {expr}")
        return key

    def _print_Symbol(self, expr):
        if expr in self._names:
            return self._names[expr]
        return super()._print_Symbol(expr)


class ReferenceForms:
    """Per-node expressions of the reference generator for one dictionary."""

    def __init__(self, dico, free_symbols=()):
        self.dim = self._dim(dico)
        schemes = dico["schemes"]
        param = dict(dico.get("parameters", {}) or {})
        la = sp.sympify(dico["scheme_velocity"])
        coords = [param.get(k, sp.Symbol(n)) for k, n in (("space_x", "X"), ("space_y", "Y"), ("space_z", "Z"))]
        nums = [list(s["velocities"]) for s in schemes]
        nvs = [len(n) for n in nums]
        ptr = np.concatenate([[0], np.cumsum(nvs)]).astype(int)
        ns = int(ptr[-1])
        self.ns = ns

        # moment matrices per elementary scheme (pylbm/scheme.py:464-532)
        M = sp.zeros(ns, ns)
        invM = sp.zeros(ns, ns)
        P = [p for s in schemes for p in s["polynomials"]]
        for isch in range(len(schemes)):
            v = [velocity(self.dim, n) for n in nums[isch]]
            p = P[ptr[isch]:ptr[isch + 1]]
            lv = len(v)
            Mk = sp.zeros(lv, lv)
            for i in range(lv):
                for j in range(lv):
                    sub = [(str(coords[d]), sp.Integer(v[j][d]) * la) for d in range(self.dim)]
                    Mk[i, j] = sp.sympify(p[i]).subs(sub)
            invk = Mk.inv()
            for i in range(lv):
                for j in range(lv):
                    M[ptr[isch] + i, ptr[isch] + j] = Mk[i, j]
                    invM[ptr[isch] + i, ptr[isch] + j] = invk[i, j]
        _alltogether(M, nsimplify=True)
        _alltogether(invM, nsimplify=True)

        EQ = sp.Matrix([sp.sympify(e) for s in schemes for e in s["equilibrium"]])
        S = sp.Matrix([sp.sympify(r) for s in schemes for r in s["relaxation_parameters"]])
        consm = []
        for isch, s in enumerate(schemes):
            cm = s.get("conserved_moments")
            if cm is None:
                continue
            cm = [cm] if isinstance(cm, (sp.Symbol, sp.IndexedBase)) else list(cm)
            leq = list(EQ[ptr[isch]:ptr[isch + 1]])
            for c in cm:
                consm.append((c, int(ptr[isch]) + leq.index(c)))
        for ic, (_, c) in enumerate(consm):
            EQ.row_swap(ic, c)
            S.row_swap(ic, c)
            M.row_swap(ic, c)
            invM.col_swap(ic, c)
        self.nconsm = len(consm)
        cons_syms = [c for c, _ in consm]

        # algorithm level (pylbm/algorithm/base.py:90-190)
        psubs = list(param.items())
        self.M = M.subs(psubs)
        self.invM = invM.subs(psubs)
        self.mv = sp.MatrixSymbol("m", ns, 1)
        local = sp.symbols("xx, yy, zz")
        to_subs = list(zip(coords, local)) + psubs
        to_subs_full = to_subs + [(c, self.mv[i, 0]) for i, c in enumerate(cons_syms)]
        self.eq = _recursive_sub(EQ, to_subs_full)
        _alltogether(self.eq, nsimplify=True)
        self.s = _recursive_sub(S, to_subs_full)
        _alltogether(self.s)
        self.free = list(free_symbols)

        # storage order of the Cython container: velocities last (AoS)
        self.sorder = [self.dim] + list(range(self.dim))
        self.vel = np.array([velocity(self.dim, n) for nn in nums for n in nn], dtype=np.int64)

    @staticmethod
    def _dim(dico):
        box = dico["box"]
        return 1 + (box.get("y") is not None) + (box.get("y") is not None and box.get("z") is not None)

    # ------------------------------------------------------------------ objects
    def _space_idx(self, inner):
        vmax = np.abs(self.vel).max(axis=0)
        sizes = [_nx, _ny, _nz]
        idxs = [_ix_, _iy_, _iz_]
        out = []
        for d in range(3):
            vm = int(vmax[d]) if d < self.dim else 0
            rng = (sp.Integer(vm), sizes[d] - vm) if inner else (sp.Integer(0), sizes[d])
            out.append(sp.Idx(idxs[d], rng))
        return _set_order(out, self.sorder[1:])

    def _indexed(self, name, space_index, shifts=None):
        base = sp.IndexedBase(name, _set_order([sp.Integer(self.ns), _nx, _ny, _nz], self.sorder))
        out = []
        for k in range(self.ns):
            ind = list(space_index)
            if shifts is not None:
                ind = [ind[d] + int(shifts[k][d]) for d in range(self.dim)]
            out.append(base[tuple(_set_order([k] + ind, self.sorder))])
        return out

    def _printer(self, names):
        for i, s in enumerate(self.free):
            names[s] = f"prm[{i}]"
        return _Printer(names)

    # ------------------------------------------------------------------ forms
    def moments_pull(self, src="g", dst="m"):
        """m = M f with f pulled (one_time_step, pylbm/algorithm/pull.py:11-59)."""
        f = self._indexed("f", self._space_idx(True), shifts=-self.vel)
        names = {f[k]: f"{src}[{k}]" for k in range(self.ns)}
        pr = self._printer(names)
        mf = self.M * sp.Matrix(f)
        return [f"{dst}[{i}] = {pr.doprint(mf[i])};" for i in range(self.ns) if mf[i] != 0]

    def moments_full(self, src="g", dst="m"):
        """m = M f on the whole box (routine f2m, pylbm/algorithm/base.py:336-344)."""
        f = self._indexed("f", self._space_idx(False))
        names = {f[k]: f"{src}[{k}]" for k in range(self.ns)}
        pr = self._printer(names)
        mf = self.M * sp.Matrix(f)
        return [f"{dst}[{i}] = {pr.doprint(mf[i])};" if mf[i] != 0 else f"{dst}[{i}] = 0.0;"
                for i in range(self.ns)]

    def relaxation(self, m="m"):
        """Relaxation with the local moment vector (pylbm/algorithm/base.py:404-428)."""
        names = {self.mv[i, 0]: f"{m}[{i}]" for i in range(self.ns)}
        pr = self._printer(names)
        eq = self.eq
        relax = sp.Matrix([(1 - self.s[i]) * self.mv[i, 0] + self.s[i] * eq[i] for i in range(self.ns)])
        _alltogether(relax)
        lines = []
        for i in range(self.ns):
            if sp.simplify(relax[i] - self.mv[i, 0]) == 0:
                continue
            lines.append(f"{m}[{i}] = {pr.doprint(relax[i])};")
        return lines

    def populations(self, src="m", dst="g"):
        """f = M^-1 m inside one_time_step, local moment vector (pylbm/algorithm/base.py:346-379)."""
        names = {self.mv[i, 0]: f"{src}[{i}]" for i in range(self.ns)}
        pr = self._printer(names)
        fm = self.invM * sp.Matrix([self.mv[i, 0] for i in range(self.ns)])
        return [f"{dst}[{k}] = {pr.doprint(fm[k])};" for k in range(self.ns)]

    def populations_routine(self, src="m", dst="g"):
        """f = M^-1 m of the standalone m2f routine, whose moments are indexed
        arrays: sympy orders their terms by the printed index (m[..., 10]
        before m[..., 3]), unlike the local vector of one_time_step."""
        mi = self._indexed("m", self._space_idx(False))
        names = {mi[k]: f"{src}[{k}]" for k in range(self.ns)}
        pr = self._printer(names)
        fm = self.invM * sp.Matrix(mi)
        return [f"{dst}[{k}] = {pr.doprint(fm[k])};" for k in range(self.ns)]

    def feq_host(self, cons, prm=()):
        """Equilibrium populations (ns, n) of conserved moments (nconsm, n),
        computed on the host with the printed equilibrium and m2f routines
        (the reference's BoundaryMethod.prepare_rhs runs exactly those,
        pylbm/boundary.py:238-305).  Every printed line is also a valid
        Python expression, evaluated here in IEEE float64."""
        if not hasattr(self, "_feq_code"):
            body = []
            for line in self.equilibrium("m")[1:] + self.populations_routine("m", "g"):
                body.append(line.rstrip(";"))
            self._feq_code = compile("\n".join(body), "<reference equilibrium>", "exec")
        cons = np.asarray(cons, dtype=np.float64)
        n = cons.shape[1]
        m = [np.zeros(n) for _ in range(self.ns)]
        for c in range(self.nconsm):
            m[c] = cons[c].copy()
        ns = {"m": m, "__in": [x.copy() for x in m], "g": [None] * self.ns, "prm": list(prm),
              "sqrt": np.sqrt, "pow": np.power}
        exec(self._feq_code, ns)
        return np.array([np.broadcast_to(np.asarray(x, dtype=np.float64), (n,)) for x in ns["g"]])

    def relaxation_routine(self, m="m"):
        """Relaxation of the standalone relaxation routine (indexed moments)."""
        mi = self._indexed("m", self._space_idx(False))
        names = {mi[k]: f"__in[{k}]" for k in range(self.ns)}
        pr = self._printer(names)
        eq = self.eq.subs(list(zip(self.mv, mi)))
        relax = sp.Matrix([(1 - self.s[i]) * mi[i] + self.s[i] * eq[i] for i in range(self.ns)])
        _alltogether(relax)
        lines = [f"const double __in[{self.ns}] = {{" + ", ".join(f"{m}[{k}]" for k in range(self.ns)) + "};"]
        for i in range(self.ns):
            if sp.simplify(relax[i] - mi[i]) == 0:
                continue
            lines.append(f"{m}[{i}] = {pr.doprint(relax[i])};")
        return lines

    def equilibrium(self, m="m"):
        """Equilibrium of every moment (routine equilibrium, pylbm/algorithm/base.py:381-402)."""
        mi = self._indexed("m", self._space_idx(False))
        names = {mi[k]: f"__in[{k}]" for k in range(self.ns)}
        pr = self._printer(names)
        eq = self.eq.subs(list(zip(self.mv, mi)))
        lines = [f"const double __in[{self.ns}] = {{" + ", ".join(f"{m}[{k}]" for k in range(self.ns)) + "};"]
        for k in range(self.nconsm, self.ns):
            lines.append(f"{m}[{k}] = {pr.doprint(eq[k])};")
        return lines
