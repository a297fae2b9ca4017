"""Per-scheme CUDA source generation.

pylbm turns a scheme into code at run time (pylbm/generator/, ``Generator``
generator.py:9; Cython printer pylbm/generator/printing/cython.py:72) and
compiles it into a module whose routines are named ``one_time_step``,
``f2m``, ``m2f``, ``equilibrium``, ``relaxation`` and ``transport``
(pylbm/algorithm/base.py:603-628).  The CUDA backend keeps that split: the
kernels are hand-written templates (``csrc/scheme_kernels.cuh``) and only the
per-node algebra is generated here, as straight-line device functions:

* ``lbm_moments``: m = M g.  Opposite velocities k, k' share the sum
  g_k + g_k' (for moments even in v) or the difference g_k - g_k' (odd
  moments); equal coefficients are grouped so each row costs one multiply per
  distinct coefficient.
* ``lbm_populations``: g = M^-1 m through the even/odd split
  g_k = E_k + O_k, g_k' = E_k - O_k.
* ``lbm_relax``: the non-conserved moments relax toward equilibrium,
  m <- m + s (meq - m)  (pylbm/algorithm/base.py:404-428 writes it as
  (1 - s) m + s meq).

In the shifted-storage form the device holds g = f - feq(c0) for a fixed
reference state c0 of the conserved moments, and the equilibrium is emitted
as meq(c0 + dc) - meq(c0) expanded symbolically, so the large constant parts
cancel exactly before any rounding.
"""
import hashlib
from fractions import Fraction

import numpy as np
import sympy as sp

from .scheme import REL_U, SchemeError, to_fraction


def _lit(x):
    """A typed literal: exact float64 repr converted to the compute type at compile time."""
    f = float(x)
    if f == int(f) and abs(f) < 2**31:
        return f"LBM_R({int(f)})"
    return f"LBM_R({repr(f)})"


class ExprPrinter:
    """Prints +, *, integer powers and numbers of a sympy expression as C."""

    def __init__(self, names):
        self.names = names
        self.products = {}  # shared-product symbol -> its product (see _cse)

    def __call__(self, e):
        return self.p(sp.sympify(e))

    def p(self, e):
        if e in self.names:
            return self.names[e]
        if e.is_Number:
            fr = to_fraction(e)
            return _lit(fr) if fr >= 0 else f"(-{_lit(-fr)})"
        if e.is_Symbol:
            raise SchemeError(f"unbound symbol {e} in generated expression")
        if e.is_Add:
            # every product term is an explicit multiply-add: the plain terms
            # are summed first, then c*x -> fma(c, x, acc), x*y*z -> fma(x, y*z, acc),
            # -x*y -> fma(-x, y, acc), x^n -> fma(x, x^(n-1), acc); no product
            # ever feeds an addition, so there is nothing left to contract
            plain, prods = [], []
            for a in e.args:
                (prods if self._fusable(a) else plain).append(a)
            if plain:
                acc = self.p(plain[0])
                for a in plain[1:]:
                    coef, rest = a.as_coeff_Mul()
                    acc = f"({acc} - {self.p(rest)})" if coef == -1 else f"({acc} + {self.p(a)})"
            else:
                acc, prods = self.p(prods[0]), prods[1:]
            for a in prods:
                acc = self._fma_term(a, acc)
            return "(" + acc + ")"
        if e.is_Mul:
            coef, rest = e.as_coeff_Mul()
            if coef == -1:  # a negation, not a multiplication
                return f"(-{self.p(rest)})"
            num, den = self._mul_parts(e)
            s = "*".join(num) if num else "LBM_R(1)"
            if den:
                s = f"({s})/({'*'.join(den)})"
            return "(" + s + ")"
        if e.is_Pow:
            if e.exp.is_Integer:
                n = int(e.exp)
                b = self.p(e.base)
                if n == 0:
                    return "LBM_R(1)"
                if n > 0:
                    return "(" + "*".join([b] * n) + ")"
                return "(LBM_R(1)/(" + "*".join([b] * (-n)) + "))"
            if e.exp == sp.Rational(1, 2):
                return f"lbm_sqrt({self.p(e.base)})"
            if e.exp.is_Number:  # real power (e.g. the p-system's u^(-2/3))
                return f"lbm_pow({self.p(e.base)}, {_lit(to_fraction(e.exp))})"
            raise SchemeError(f"unsupported power {e}")
        raise SchemeError(f"unsupported expression {e} ({type(e).__name__})")

    def _mul_parts(self, e):
        """Printed numerator and denominator factors of a product."""
        num, den = [], []
        for a in e.args:
            if a.is_Pow and a.exp.is_Integer and a.exp < 0:
                den.append(self.p(a.base) if a.exp == -1 else self.p(sp.Pow(a.base, -a.exp)))
            elif a.is_Rational and not a.is_Integer and a.p == 1:
                den.append(_lit(a.q))
            else:
                num.append(self.p(a))
        return num, den

    def _splittable(self, e):
        num, den = self._mul_parts(e)
        return not den and len(num) >= 2

    def _fusable(self, a):
        """A term c*x, x*y*..., x^n, or a shared product, that folds into a multiply-add."""
        coef, rest = a.as_coeff_Mul()
        if coef.is_Number and coef not in (1, -1) and rest != 1:
            return True
        if rest in self.products:
            return self._fusable(self.products[rest])
        if rest.is_Mul and self._splittable(rest):
            return True
        return bool(rest.is_Pow and rest.exp.is_Integer and rest.exp >= 2)

    def _fma_term(self, a, acc):
        coef, rest = a.as_coeff_Mul()
        if coef in (1, -1) and rest in self.products:  # t + z with t = x*y: fma(x, y, z)
            return self._fma_term(coef * self.products[rest], acc)
        if coef.is_Number and coef not in (1, -1) and rest != 1:
            return f"lbm_fma<R>({self.p(coef)}, {self.p(rest)}, {acc})"
        if rest.is_Mul:
            first, tail = self._split(rest)
        else:
            first, tail = self.p(rest.base), self.p(sp.Pow(rest.base, rest.exp - 1))
        lead = first if coef == 1 else f"(-{first})"
        return f"lbm_fma<R>({lead}, {tail}, {acc})"

    def _split(self, e):
        """x*y*z -> ("x", "(y*z)") for a product without divisions."""
        num, _ = self._mul_parts(e)
        return num[0], "(" + "*".join(num[1:]) + ")"


def _cse(exprs, prefix, printer=None):
    """Common subexpressions, with shared products known to the printer.

    A shared product t = x*y reaching an addition as a plain value (t + z) is
    a pattern the compiler may or may not fuse into one multiply-add, and in
    practice fuses for packed FP32x2 operations even when both are written
    with an explicit rounding mode.  The printer is told which symbols are
    products (``printer.products``) and writes such a term as
    lbm_fma(x, y, z) instead, so the scalar and the two-node kernels round
    identically; elsewhere the product is computed once.
    """
    repl, red = sp.cse(exprs, symbols=sp.numbered_symbols(prefix), optimizations="basic")
    if printer is not None:
        for sym, val in repl:
            if val.is_Mul or val.is_Pow:
                printer.products[sym] = val
    return repl, red


def _pairs(scheme):
    """(k, ksym) pairs with k < ksym, and self-symmetric indices (v = 0)."""
    ksym = scheme.stencil.get_symmetric()
    pairs, selfs = [], []
    for k in range(scheme.nv):
        if ksym[k] == k:
            selfs.append(k)
        elif k < ksym[k]:
            pairs.append((k, int(ksym[k])))
    return pairs, selfs


def _row_parity(row, pairs, selfs):
    """'even', 'odd' or None for one row of M (coefficients over populations)."""
    even = all(row[a] == row[b] for a, b in pairs)
    odd = all(row[a] == -row[b] for a, b in pairs) and all(row[k] == 0 for k in selfs)
    if even:
        return "even"
    if odd:
        return "odd"
    return None


def _emit_combo(terms):
    """sum of coef*var, grouped by |coef|.

    Each group of equal |coef| is summed first; groups are then accumulated
    with explicit multiply-adds, lbm_fma(c2, (x2 + ...), c1*(x1 + ...)), which
    the compiler contracts for scalars and which map to the packed FP32x2 FMA
    when two nodes are updated together.
    """
    groups = {}
    order = []
    for c, v in terms:
        if c == 0:
            continue
        key = abs(c)
        if key not in groups:
            groups[key] = []
            order.append(key)
        groups[key].append(("+" if c > 0 else "-", v))
    if not order:
        return "LBM_R(0)"
    if 1 in groups:  # the unit group starts the accumulator (no multiply)
        order.remove(1)
        order.insert(0, 1)
    acc = None
    for key in order:
        items = groups[key]
        inner = ""
        for i, (sg, v) in enumerate(items):
            if i == 0:
                inner = v if sg == "+" else f"-{v}"
            else:
                inner += f" {sg} {v}"
        if acc is None:
            acc = f"({inner})" if key == 1 else f"{_lit(key)}*({inner})"
        else:
            acc = f"lbm_fma<R>({_lit(key)}, ({inner}), {acc})"
    return acc


def _cheaper(a, b):
    """The expression of the two with fewer operations (a on ties)."""
    return b if sp.count_ops(b) < sp.count_ops(a) else a


class SchemeSource:
    """Generated device code for one scheme and one storage form.

    Parameters
    ----------
    scheme : Scheme
    shifted : bool
        True: storage holds f - feq(c0) and the relaxation works on deviations.
    c0 : sequence of float
        reference values of the conserved moments (used only when shifted).
    style : "fast" or "reference"
        "fast": exact constants, shared pair sums, grouped coefficients.
        "reference" (unshifted float64 only): the reference generator's
        printed expressions (refforms.ReferenceForms), compiled without fused
        multiply-adds, for parity with pylbm's generated code.
    node_pairs : bool
        16-bit storage, fast style: update two nodes of a row per thread with
        packed FP32x2 arithmetic where the lattice allows it.
    """

    def __init__(self, scheme, shifted, c0=None, style="fast", node_pairs=True, simplify_frame=False):
        self.scheme = scheme
        self.node_pairs = bool(node_pairs)
        # relative-velocity schemes: write the moving-frame equilibrium T(u) m_eq
        # with u replaced by its definition and simplified (for the usual
        # u = q / rho it reduces to constants times rho); equal up to rounding
        self.simplify_frame = bool(simplify_frame)
        self.shifted = bool(shifted)
        if style not in ("fast", "reference"):
            raise SchemeError(f"unknown style {style!r}")
        if style == "reference" and self.shifted:
            raise SchemeError("the reference style is the unshifted float64 form")
        if style == "reference" and (scheme.Tu is not None or scheme.source_terms):
            raise SchemeError("the reference style covers schemes without relative velocity or source terms")
        self.style = style
        # no implicit contraction: every fused multiply-add is an explicit
        # lbm_fma in the generated source, so all kernels of a module (and the
        # one- and two-node forms) round identically
        self.nvcc_flags = ["-fmad=false"]
        self._ref = None
        nv, nc = scheme.nv, scheme.nconsm
        self.c0 = [to_fraction(c) for c in (c0 if c0 is not None else [0] * nc)]
        if len(self.c0) != nc:
            raise SchemeError("one reference value per conserved moment is needed")
        self.params = list(scheme.free_symbols)
        cons = list(scheme.consm.keys())
        c0s = [sp.Rational(c.numerator, c.denominator) for c in self.c0]
        # absolute equilibrium at the reference state
        ref = dict(zip(cons, c0s))
        self.meq_ref = []
        for e in scheme.EQ:
            # unshifted storage has no reference state (and c0 = 0 may be singular, e.g. u^(-2/3))
            v = e.subs(ref) if self.shifted else sp.Integer(0)
            self.meq_ref.append(v)
        if any(v.free_symbols for v in self.meq_ref):
            if self.shifted:
                raise SchemeError("shifted storage needs an equilibrium at rest free of run-time parameters")
        self.meq_ref_frac = [to_fraction(v) if not v.free_symbols else Fraction(0) for v in self.meq_ref]
        if self.shifted:
            shift = [sum((scheme.invM_frac[k][j] * self.meq_ref_frac[j] for j in range(nv)), Fraction(0))
                     for k in range(nv)]
        else:
            shift = [Fraction(0)] * nv
        self.shift = shift
        self.mref = [sum((scheme.M_frac[i][k] * shift[k] for k in range(nv)), Fraction(0)) for i in range(nv)]
        self.pairs, self.selfs = _pairs(scheme)
        self.parity = [_row_parity(scheme.M_frac[i], self.pairs, self.selfs) for i in range(nv)]

    @property
    def shift_float(self):
        return np.array([float(x) for x in self.shift])

    @property
    def mref_float(self):
        return np.array([float(x) for x in self.mref])

    # ---------------------------------------------------------------
    def _moments_code(self, src, dst, indent="  "):
        """dst_i = (M src)_i using pair sums/differences."""
        sc = self.scheme
        lines = []
        use_pairs = any(p is not None for p in self.parity)
        if use_pairs:
            for a, b in self.pairs:
                lines.append(f"{indent}const R {src}_a{a} = {src}[{a}] + {src}[{b}];")
                lines.append(f"{indent}const R {src}_b{a} = {src}[{a}] - {src}[{b}];")
        for i in range(sc.nv):
            row = sc.M_frac[i]
            par = self.parity[i]
            terms = []
            if par == "even":
                for k in self.selfs:
                    terms.append((row[k], f"{src}[{k}]"))
                for a, b in self.pairs:
                    terms.append((row[a], f"{src}_a{a}"))
            elif par == "odd":
                for a, b in self.pairs:
                    terms.append((row[a], f"{src}_b{a}"))
            else:
                for k in range(sc.nv):
                    terms.append((row[k], f"{src}[{k}]"))
            lines.append(f"{indent}{dst}[{i}] = {_emit_combo(terms)};")
        return lines

    def _populations_code(self, src, dst, indent="  "):
        """dst = M^-1 src, via even/odd halves for opposite velocities."""
        sc = self.scheme
        inv = sc.invM_frac
        even = [j for j in range(sc.nv) if self.parity[j] == "even"]
        odd = [j for j in range(sc.nv) if self.parity[j] == "odd"]
        pure = len(even) + len(odd) == sc.nv
        if pure:
            for a, b in self.pairs:
                pure = pure and all(inv[b][j] == inv[a][j] for j in even) and all(inv[b][j] == -inv[a][j] for j in odd)
            for k in self.selfs:
                pure = pure and all(inv[k][j] == 0 for j in odd)
        lines = []
        if pure:
            for k in self.selfs:
                lines.append(f"{indent}{dst}[{k}] = {_emit_combo([(inv[k][j], f'{src}[{j}]') for j in even])};")
            for a, b in self.pairs:
                e = _emit_combo([(inv[a][j], f"{src}[{j}]") for j in even])
                o = _emit_combo([(inv[a][j], f"{src}[{j}]") for j in odd])
                lines.append(f"{indent}{{ const R e_ = {e}; const R o_ = {o};")
                lines.append(f"{indent}  {dst}[{a}] = e_ + o_; {dst}[{b}] = e_ - o_; }}")
        else:
            for k in range(sc.nv):
                lines.append(f"{indent}{dst}[{k}] = {_emit_combo([(inv[k][j], f'{src}[{j}]') for j in range(sc.nv)])};")
        return lines

    def _relax_code(self, m, indent="  ", deviation=True):
        """Relax the non-conserved moments of m (deviation or absolute form)."""
        sc = self.scheme
        nc = sc.nconsm
        cons = list(sc.consm.keys())
        dsym = [sp.Symbol(f"__d{c}") for c in range(nc)]
        names = {}
        for c in range(nc):
            names[dsym[c]] = f"{m}[{c}]"
        for i, s in enumerate(self.params):
            names[s] = f"prm[{i}]"
        exprs = []
        for k in range(nc, sc.nv):
            e = sc.EQ[k]
            if deviation and self.shifted:
                c0s = [sp.Rational(c.numerator, c.denominator) for c in self.c0]
                full = e.subs({cons[c]: c0s[c] + dsym[c] for c in range(nc)})
                d = sp.expand(full - self.meq_ref[k])
                d = sp.together(d) if d.has(sp.Pow) and any(p.exp.is_negative for p in d.atoms(sp.Pow)) else d
            else:
                d = sp.expand(e.subs({cons[c]: dsym[c] for c in range(nc)}))
            exprs.append(d)
        lines = []
        pr = ExprPrinter(names)
        repl, red = _cse(exprs, "t_", pr)
        for sym, val in repl:
            lines.append(f"{indent}const R {sym} = {pr(val)};")
            names[sym] = str(sym)
        for idx, k in enumerate(range(nc, sc.nv)):
            s = sc.s[k]
            if isinstance(s, sp.Expr):
                sstr = ExprPrinter(names)(s)
            else:
                if s == 0.0:
                    continue
                sstr = _lit(s)
            eqs = pr(red[idx])
            if not isinstance(s, sp.Expr) and s == 1.0:
                lines.append(f"{indent}{m}[{k}] = {eqs};")
            elif red[idx] == 0:  # m + s (0 - m) = fma(-s, m, m), the same rounding
                lines.append(f"{indent}{m}[{k}] = lbm_fma<R>(-({sstr}), {m}[{k}], {m}[{k}]);")
            else:
                # eq - m printed as one sum, so a product in eq becomes fma(., ., -m)
                mk = sp.Symbol(f"__m{k}")
                names[mk] = f"{m}[{k}]"
                lines.append(f"{indent}{m}[{k}] = lbm_fma<R>({sstr}, {pr(red[idx] - mk)}, {m}[{k}]);")
        return lines

    def _eq_abs_code(self, m, indent="  "):
        """Set every non-conserved moment of absolute m to its equilibrium."""
        sc = self.scheme
        nc = sc.nconsm
        cons = list(sc.consm.keys())
        names = {cons[c]: f"{m}[{c}]" for c in range(nc)}
        for i, s in enumerate(self.params):
            names[s] = f"prm[{i}]"
        exprs = [sc.EQ[k] for k in range(nc, sc.nv)]
        pr = ExprPrinter(names)
        repl, red = _cse(exprs, "u_", pr)
        lines = []
        for sym, val in repl:
            lines.append(f"{indent}const R {sym} = {pr(val)};")
            names[sym] = str(sym)
        for idx, k in enumerate(range(nc, sc.nv)):
            lines.append(f"{indent}{m}[{k}] = {pr(red[idx])};")
        return lines

    def _relax_abs_code(self, m, indent="  "):
        return self._relax_code(m, indent, deviation=False)

    def _eq_dev_code(self, m, indent="  "):
        """Shifted storage: the non-conserved moments of a deviation vector set
        to meq_k(c0 + dc) - meq_k(c0) from its conserved deviations dc (the
        expansions the relaxation uses); unshifted: the absolute equilibrium."""
        if not self.shifted:
            return self._eq_abs_code(m, indent)
        sc = self.scheme
        nc = sc.nconsm
        cons = list(sc.consm.keys())
        dsym = [sp.Symbol(f"__d{c}") for c in range(nc)]
        names = {dsym[c]: f"{m}[{c}]" for c in range(nc)}
        for i, s in enumerate(self.params):
            names[s] = f"prm[{i}]"
        c0s = [sp.Rational(c.numerator, c.denominator) for c in self.c0]
        exprs = []
        for k in range(nc, sc.nv):
            full = sc.EQ[k].subs({cons[c]: c0s[c] + dsym[c] for c in range(nc)})
            d = sp.expand(full - self.meq_ref[k])
            d = sp.together(d) if d.has(sp.Pow) and any(p.exp.is_negative for p in d.atoms(sp.Pow)) else d
            exprs.append(d)
        pr = ExprPrinter(names)
        repl, red = _cse(exprs, "e_", pr)
        lines = []
        for sym, val in repl:
            lines.append(f"{indent}const R {sym} = {pr(val)};")
            names[sym] = str(sym)
        for idx, k in enumerate(range(nc, sc.nv)):
            lines.append(f"{indent}{m}[{k}] = {pr(red[idx])};")
        return lines

    # --------------------------------------------------------------- frame-relative / source-term collide
    @property
    def absolute_collide(self):
        """Schemes with a relative velocity or source terms collide in absolute form."""
        return self.scheme.Tu is not None or bool(self.scheme.source_terms)

    def _names(self, m="m"):
        sc = self.scheme
        names = {c: f"{m}[{i}]" for i, c in enumerate(sc.consm.keys())}
        for i, s in enumerate(self.params):
            names[s] = f"prm[{i}]"
        for d, u in enumerate(sc.rel_vel_symbols):
            names[u] = f"u_{d}"
        return names

    def _assign_block(self, targets, exprs, names, prefix, indent):
        """targets[i] = exprs[i] evaluated together (all right-hand sides first)."""
        pr = ExprPrinter(dict(names))
        repl, red = _cse(exprs, f"{prefix}c_", pr)
        lines = [f"{indent}{{"]
        for sym, val in repl:
            lines.append(f"{indent}  const R {sym} = {pr(val)};")
            pr.names[sym] = str(sym)
        for i, e in enumerate(red):
            lines.append(f"{indent}  const R {prefix}{i} = {pr(e)};")
        for i, t in enumerate(targets):
            lines.append(f"{indent}  {t} = {prefix}{i};")
        lines.append(f"{indent}}}")
        return lines

    def _source_code(self, names, indent):
        """m_c += dt/2 S_c(m) for every source term (pylbm/algorithm/base.py:439-495, ode.py:11-16)."""
        sc = self.scheme
        if not sc.source_terms:
            return []
        cons = list(sc.consm.keys())
        from .scheme import DT
        targets, exprs = [], []
        for k, rhs in sc.source_terms:
            targets.append(f"m[{k}]")
            exprs.append(cons[k] + DT / 2 * rhs)
        return self._assign_block(targets, exprs, names, "src_", indent)

    def _absolute_collide_code(self, indent="  "):
        """One node: pull values g (stored form) -> post-collision g.

        Order of pylbm's PullAlgorithm.one_time_step_local
        (pylbm/algorithm/pull.py:11-59): moments (conserved ones absolute; the
        others, with a relative velocity u(m_cons), seen from the frame moving
        at u: T(u) M f), source terms over dt/2, relaxation towards
        T(u) m_eq, the conserved moments replaced by their moving-frame values
        (T(u) M f)_c, source terms over dt/2, and f = M^-1 T(-u) m.
        """
        sc = self.scheme
        nv, nc = sc.nv, sc.nconsm
        msym = [sp.Symbol(f"__m{l}") for l in range(nv)]
        names = self._names()
        lines = [f"{indent}R m[LBM_Q];"]
        if self.shifted:
            for k in range(nv):
                if self.shift[k] != 0:
                    lines.append(f"{indent}g[{k}] = g[{k}] + {_lit(self.shift[k])};")
        lines.append(f"{indent}lbm_moments<R>(g, m);")
        rel = sc.Tu is not None
        if rel:
            pr = ExprPrinter(names)
            for d, e in enumerate(sc.rel_vel):
                lines.append(f"{indent}const R u_{d} = {pr(e)};")
            mnames = dict(names)
            mnames.update({msym[l]: f"m[{l}]" for l in range(nv)})
            # every moment in the moving frame; the conserved ones are kept
            # aside until after the relaxation (PullAlgorithm, pull.py:48-49)
            lines.append(f"{indent}R mc_rel[LBM_NCONS];")
            targets = [f"mc_rel[{k}]" for k in range(nc)] + [f"m[{k}]" for k in range(nc, nv)]
            exprs = [sp.expand(sum(sc.Tu[k, l] * msym[l] for l in range(nv))) for k in range(nv)]
            lines += self._assign_block(targets, exprs, mnames, "rel_", indent)
        lines += self._source_code(names, indent)
        # relaxation of every moment with a non-zero rate towards T(u) m_eq
        eqv = sp.Matrix(sc.EQ)
        eq_rel = (sc.Tu * eqv).applyfunc(sp.expand) if rel else eqv
        if rel and self.simplify_frame:
            sub = {REL_U[d]: e for d, e in enumerate(sc.rel_vel)}
            eq_rel = sp.Matrix([_cheaper(e, sp.factor(sp.cancel(e.subs(sub)))) for e in eq_rel])
        targets, exprs = [], []
        for k in range(nv):
            rate = sc.s[k]
            if not isinstance(rate, sp.Expr) and rate == 0.0:
                continue
            rate = rate if isinstance(rate, sp.Expr) else sp.Float(rate)
            targets.append(f"m[{k}]")
            exprs.append(msym[k] + rate * (eq_rel[k] - msym[k]))
        rnames = dict(names)
        rnames.update({msym[l]: f"m[{l}]" for l in range(nv)})
        if targets:
            lines += self._assign_block(targets, exprs, rnames, "rlx_", indent)
        if rel:  # restore_conserved_moments (pylbm/algorithm/base.py:255-263)
            for k in range(nc):
                lines.append(f"{indent}m[{k}] = mc_rel[{k}];")
        lines += self._source_code(names, indent)
        if rel:
            targets = [f"m[{k}]" for k in range(nv)]
            exprs = [sp.expand(sum(sc.Tmu[k, l] * msym[l] for l in range(nv))) for k in range(nv)]
            lines += self._assign_block(targets, exprs, rnames, "back_", indent)
        lines.append(f"{indent}lbm_populations<R>(m, g);")
        if self.shifted:
            for k in range(nv):
                if self.shift[k] != 0:
                    lines.append(f"{indent}g[{k}] = g[{k}] - {_lit(self.shift[k])};")
        lines.append(f"{indent}(void)prm;")
        return lines

    # ---------------------------------------------------------------
    def header(self):
        sc = self.scheme
        nv = sc.nv
        v = np.zeros((nv, 3), dtype=np.int64)
        v[:, :sc.dim] = sc.stencil.get_all_velocities()
        out = []
        out.append("// generated by pylbm_gb300.codegen -- scheme constants and per-node algebra")
        out.append(f"#define LBM_DIM {sc.dim}")
        out.append(f"#define LBM_Q {nv}")
        out.append(f"#define LBM_NCONS {sc.nconsm}")
        out.append(f"#define LBM_NPRM {len(self.params)}")
        out.append(f"#define LBM_SHIFTED {int(self.shifted)}")
        out.append("#define LBM_R(x) static_cast<R>(x)")
        vmax = int(np.abs(v).max()) if v.size else 0
        out.append(f"#define LBM_VMAX {max(vmax, 1)}")
        out.append("#define LBM_FOR_EACH_V(X) " + " ".join(
            f"X({k}, {int(v[k, 0])}, {int(v[k, 1])}, {int(v[k, 2])})" for k in range(nv)))
        out.append("__device__ __constant__ double lbm_dev_shift[LBM_Q] = {" +
                   ", ".join(repr(float(x)) for x in self.shift) + "};")
        out.append("__device__ __constant__ double lbm_dev_mref[LBM_Q] = {" +
                   ", ".join(repr(float(x)) for x in self.mref) + "};")
        out.append("static const double lbm_host_shift[LBM_Q] = {" +
                   ", ".join(repr(float(x)) for x in self.shift) + "};")
        out.append("static const double lbm_host_mref[LBM_Q] = {" +
                   ", ".join(repr(float(x)) for x in self.mref) + "};")
        out.append("")
        if self.style == "reference":
            out += self._reference_functions()
            return "\n".join(out) + "\n"
        # moments of a deviation vector
        out.append("template <typename R>")
        out.append("__device__ __forceinline__ void lbm_moments(const R (&g)[LBM_Q], R (&m)[LBM_Q]) {")
        out += self._moments_code("g", "m")
        out.append("}")
        out.append("template <typename R>")
        out.append("__device__ __forceinline__ void lbm_populations(const R (&m)[LBM_Q], R (&g)[LBM_Q]) {")
        out += self._populations_code("m", "g")
        out.append("}")
        out.append("// relaxation of the moments of a stored (deviation) state")
        out.append("template <typename R>")
        out.append("__device__ __forceinline__ void lbm_relax(R (&m)[LBM_Q], const R* __restrict__ prm) {")
        out += self._relax_code("m")
        out.append("  (void)prm;")
        out.append("}")
        out.append("// equilibrium of absolute moments (non-conserved set from conserved)")
        out.append("template <typename R>")
        out.append("__device__ __forceinline__ void lbm_equilibrium_abs(R (&m)[LBM_Q], const R* __restrict__ prm) {")
        out += self._eq_abs_code("m")
        out.append("  (void)prm;")
        out.append("}")
        out.append("// equilibrium of a stored (deviation) state from its conserved moments")
        out.append("template <typename R>")
        out.append("__device__ __forceinline__ void lbm_equilibrium_dev(R (&m)[LBM_Q], const R* __restrict__ prm) {")
        out += self._eq_dev_code("m")
        out.append("  (void)prm;")
        out.append("}")
        out.append("// relaxation of absolute moments")
        out.append("template <typename R>")
        out.append("__device__ __forceinline__ void lbm_relax_abs(R (&m)[LBM_Q], const R* __restrict__ prm) {")
        out += self._relax_abs_code("m")
        out.append("  (void)prm;")
        out.append("}")
        out += self._source_half_function()
        out.append("template <typename R>")
        out.append("__device__ __forceinline__ void lbm_collide(R (&g)[LBM_Q], const R* __restrict__ prm) {")
        if self.absolute_collide:
            out += self._absolute_collide_code()
        else:
            out.append("  R m[LBM_Q];")
            out.append("  lbm_moments<R>(g, m);")
            out.append("  lbm_relax<R>(m, prm);")
            out.append("  lbm_populations<R>(m, g);")
        out.append("}")
        return "\n".join(out) + "\n"

    def reference_forms(self):
        from .refforms import ReferenceForms

        if self._ref is None:
            self._ref = ReferenceForms(self.scheme.dico, self.params)
        return self._ref

    def _reference_functions(self):
        """Per-node functions printed as the reference generator prints them."""
        ref = self.reference_forms()
        ind = "  "

        def fn(sig, body):
            return ["template <typename R>", f"__device__ __forceinline__ void {sig} {{"] + \
                   [ind + line for line in body] + [ind + "(void)prm;" if "prm" in sig else "", "}"]

        out = []
        out += fn("lbm_moments(const R (&g)[LBM_Q], R (&m)[LBM_Q])", ref.moments_full("g", "m"))
        out += fn("lbm_populations(const R (&m)[LBM_Q], R (&g)[LBM_Q])", ref.populations_routine("m", "g"))
        out += fn("lbm_relax_abs(R (&m)[LBM_Q], const R* __restrict__ prm)", ref.relaxation_routine("m"))
        out += fn("lbm_relax(R (&m)[LBM_Q], const R* __restrict__ prm)", ref.relaxation("m"))
        out += fn("lbm_equilibrium_abs(R (&m)[LBM_Q], const R* __restrict__ prm)", ref.equilibrium("m"))
        out += fn("lbm_equilibrium_dev(R (&m)[LBM_Q], const R* __restrict__ prm)", ref.equilibrium("m"))
        out += fn("lbm_collide(R (&g)[LBM_Q], const R* __restrict__ prm)",
                  ["R m[LBM_Q];"] + ref.moments_pull("g", "m") + ref.relaxation("m") + ref.populations("m", "g"))
        out += self._source_half_function()
        return out

    def _source_half_function(self):
        """pylbm's standalone source_term on absolute moments: m_c += dt/2 S_c(m)
        (pylbm/algorithm/base.py:439-504 with ode.py:11-16); empty without
        source terms."""
        body = self._source_code(self._names(), "  ")
        return ["// source terms over half a time step (absolute moments)",
                f"#define LBM_HAS_SOURCE {1 if self.scheme.source_terms else 0}",
                "template <typename R>",
                "__device__ __forceinline__ void lbm_source_half(R (&m)[LBM_Q], const R* __restrict__ prm) {"] + \
            body + ["  (void)m;", "  (void)prm;", "}"]

    def module_source(self, storage, compute):
        """Full translation unit of the module for one storage/compute type (memoised:
        sympy is not thread-safe, so callers that compile in parallel generate first)."""
        key = (storage, compute)
        cache = self.__dict__.setdefault("_sources", {})
        if key not in cache:
            cache[key] = self._module_source(storage, compute)
        return cache[key]

    def _module_source(self, storage, compute):
        ctypes_ = {"float64": "double", "float32": "float", "float16": "__half", "bfloat16": "__nv_bfloat16"}
        pairs = (self.node_pairs and self.style == "fast" and storage in ("float16", "bfloat16")
                 and compute == "float32")
        return (f"#define LBM_STORAGE {ctypes_[storage]}\n"
                f"#define LBM_COMPUTE {ctypes_[compute]}\n"
                + ("#define LBM_PAIRS 1\n" if pairs else "") +
                "#include \"lbm_common.cuh\"\n"
                "using lbm::lbm_fma;\n"
                "template <typename R> __device__ __forceinline__ R lbm_sqrt(R x) { return sqrt(x); }\n"
                "template <typename R> __device__ __forceinline__ R lbm_pow(R x, R e) { return pow(x, e); }\n"
                + self.header() +
                "#include \"scheme_kernels.cuh\"\n")
