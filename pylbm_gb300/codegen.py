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

from .scheme import SchemeError, to_fraction


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
            terms = [self.p(a) for a in e.args]
            return "(" + " + ".join(terms) + ")"
        if e.is_Mul:
            num, den = [], []
            for a in e.args:
                if a.is_Pow and a.exp.is_Integer and a.exp < 0:
                    den.append(self.p(a.base) if a.exp == -1 else self.p(sp.Pow(a.base, -a.exp)))
                elif a.is_Rational and not a.is_Integer and a.p == 1:
                    den.append(_lit(a.q))
                else:
                    num.append(self.p(a))
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
            raise SchemeError(f"unsupported power {e}")
        raise SchemeError(f"unsupported expression {e} ({type(e).__name__})")


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
    """sum of coef*var, grouped by |coef|: 'c1*(x + y - z) + c2*(...)'."""
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
    parts = []
    for key in order:
        items = groups[key]
        inner = ""
        for i, (sg, v) in enumerate(items):
            if i == 0:
                inner = v if sg == "+" else f"-{v}"
            else:
                inner += f" {sg} {v}"
        if key == 1:
            parts.append(f"({inner})")
        else:
            parts.append(f"{_lit(key)}*({inner})")
    return " + ".join(parts)


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
    """

    def __init__(self, scheme, shifted, c0=None, style="fast"):
        self.scheme = scheme
        self.shifted = bool(shifted)
        if style not in ("fast", "reference"):
            raise SchemeError(f"unknown style {style!r}")
        if style == "reference" and self.shifted:
            raise SchemeError("the reference style is the unshifted float64 form")
        self.style = style
        self.nvcc_flags = ["-fmad=false"] if style == "reference" else []
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
            v = e.subs(ref)
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
        repl, red = sp.cse(exprs, symbols=sp.numbered_symbols("t_"), optimizations="basic")
        lines = []
        pr = ExprPrinter(names)
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
            else:
                lines.append(f"{indent}{m}[{k}] = {m}[{k}] + {sstr}*({eqs} - {m}[{k}]);")
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
        repl, red = sp.cse(exprs, symbols=sp.numbered_symbols("u_"), optimizations="basic")
        pr = ExprPrinter(names)
        lines = []
        for sym, val in repl:
            lines.append(f"{indent}const R {sym} = {pr(val)};")
            names[sym] = str(sym)
        for idx, k in enumerate(range(nc, sc.nv)):
            lines.append(f"{indent}{m}[{k}] = {pr(red[idx])};")
        return lines

    def _relax_abs_code(self, m, indent="  "):
        return self._relax_code(m, indent, deviation=False)

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
        out.append("// relaxation of absolute moments")
        out.append("template <typename R>")
        out.append("__device__ __forceinline__ void lbm_relax_abs(R (&m)[LBM_Q], const R* __restrict__ prm) {")
        out += self._relax_abs_code("m")
        out.append("  (void)prm;")
        out.append("}")
        out.append("template <typename R>")
        out.append("__device__ __forceinline__ void lbm_collide(R (&g)[LBM_Q], const R* __restrict__ prm) {")
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
        out += fn("lbm_collide(R (&g)[LBM_Q], const R* __restrict__ prm)",
                  ["R m[LBM_Q];"] + ref.moments_pull("g", "m") + ref.relaxation("m") + ref.populations("m", "g"))
        return out

    def module_source(self, storage, compute):
        """Full translation unit of the module for one storage/compute type."""
        ctypes_ = {"float64": "double", "float32": "float", "float16": "__half", "bfloat16": "__nv_bfloat16"}
        return (f"#define LBM_STORAGE {ctypes_[storage]}\n"
                f"#define LBM_COMPUTE {ctypes_[compute]}\n"
                "#include \"lbm_common.cuh\"\n"
                "template <typename R> __device__ __forceinline__ R lbm_sqrt(R x) { return sqrt(x); }\n"
                + self.header() +
                "#include \"scheme_kernels.cuh\"\n")
