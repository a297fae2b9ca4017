"""Host-side logic against the reference (golden fixtures), and the C ABI build.

No GPU needed: velocity numbering, moment matrices, domain flags and boundary
lists must equal pylbm's exactly; the libraries must build for sm_103a and
export every entry point of include/lbm_gb300.h.
"""
import ctypes
import os
import re

import numpy as np
import sympy as sp
import pytest

from conftest import ROOT, golden
from pylbm_gb300 import runtime
from pylbm_gb300 import workloads as W
from pylbm_gb300.boundary import Boundary
from pylbm_gb300.codegen import SchemeSource
from pylbm_gb300.domain import Domain
from pylbm_gb300.scheme import Scheme, SchemeError
from pylbm_gb300.stencil import velocity, velocity_number


def test_velocity_numbering_matches_reference():
    g = golden("velocities.npz")
    for dim in (1, 2, 3):
        ref = g[f"v{dim}"]
        ours = np.array([velocity(dim, i) for i in range(ref.shape[0])])
        assert np.array_equal(ours, ref.reshape(ours.shape))
        for i in range(ref.shape[0]):
            assert velocity_number(ours[i]) == i


@pytest.mark.parametrize("fixture,dico", [
    ("cavity_n32.npz", lambda: W.cavity(n=32)),
    ("tgv3d_n16.npz", lambda: W.tgv3d(n=16)),
])
def test_moment_matrices_match_reference(fixture, dico):
    g = golden(fixture)
    sc = Scheme(dico())
    assert np.array_equal(sc.M, g["M"])
    assert np.abs(sc.invM - g["invM"]).max() < 1e-15
    assert [str(c) for c in sc.consm] == list(g["consm"])
    assert np.allclose(sc.rates_numpy(), g["s"], rtol=0, atol=1e-14)


def _bc_equal(methods, g):
    assert len(methods) == int(g["bc_count"])
    for i, meth in enumerate(methods):
        assert type(meth).__name__ == str(g[f"bc{i}_name"])
        assert np.array_equal(meth.istore, g[f"bc{i}_istore"])
        assert np.array_equal(meth.iload[0], g[f"bc{i}_iload0"])


class _HostSim:
    """Just enough of a simulation for prepare_rhs on the host."""

    def __init__(self, dico):
        self.scheme = Scheme(dico)
        self.domain = Domain(dico, self.scheme.stencil)
        self.extra_parameters = {}

    def extra_parameters_str(self):
        return {}


@pytest.mark.parametrize("fixture,dico", [
    ("cavity_n32.npz", lambda: W.cavity(n=32)),
    ("cylinder_small.npz", lambda: W.cylinder(nx=96, ny=32, radius=5, center=(24, 17), re=40.0)),
])
def test_boundary_lists_match_reference(fixture, dico):
    g = golden(fixture)
    d = dico()
    sim = _HostSim(d)
    bc = Boundary(sim.domain, d)
    for meth in bc.methods:
        meth.set_iload()
        meth.prepare_rhs(sim)
        meth.fix_iload()
        meth.set_rhs()
    _bc_equal(bc.methods, g)
    for i, meth in enumerate(bc.methods):
        assert np.abs(meth.rhs - g[f"bc{i}_rhs"]).max() < 1e-15


def test_domain_flags_match_reference():
    g = golden("cylinder_small.npz")
    d = W.cylinder(nx=96, ny=32, radius=5, center=(24, 17), re=40.0)
    dom = Domain(d)
    assert np.array_equal(dom.flag, g["flag"])
    assert np.array_equal(dom.in_or_out, g["in_or_out"])
    assert np.abs(dom.distance - g["distance"]).max() < 1e-14


def test_unsupported_scheme_is_rejected():
    d = W.cavity(n=8)
    d["schemes"][0]["source_terms"] = {W.QX: W.RHO * sp.Symbol("X")}  # space-dependent source
    with pytest.raises(SchemeError):
        Scheme(d)
    d = W.cavity(n=8)
    d["relative_velocity"] = [W.QX / W.RHO]  # one component for two dimensions
    with pytest.raises(SchemeError):
        Scheme(d)


def test_relative_velocity_translation_matrix():
    """T(0) = I and T(u) T(-u) = I (pylbm/scheme.py:534-543); conserved rows first."""
    d = W.cavity(n=8)
    d["relative_velocity"] = [W.QX / W.RHO, W.QY / W.RHO]
    sc = Scheme(d)
    u = sc.rel_vel_symbols
    assert sc.Tu.subs({u[0]: 0, u[1]: 0}) == sp.eye(9)
    assert (sc.Tu * sc.Tmu).applyfunc(sp.expand) == sp.eye(9)
    assert sc.Tu[1, 0] == -u[0] and sc.Tu[2, 0] == -u[1]  # qx - ux rho, qy - uy rho
    src = SchemeSource(sc, shifted=False)
    assert src.absolute_collide and "mc_rel" in src.header()
    with pytest.raises(SchemeError):
        SchemeSource(sc, shifted=False, style="reference")


def test_source_terms_add_the_time_step_parameter():
    d = W.cavity(n=8)
    d["schemes"][0]["source_terms"] = {W.QY: -W.RHO * 0.01}
    sc = Scheme(d)
    assert [str(s) for s in sc.free_symbols] == ["dt"]
    (k, rhs), = sc.source_terms
    assert k == 2 and rhs == -0.01 * W.RHO


def test_shifted_source_cancels_reference_state():
    """The generated deviation equilibrium has no constant term."""
    sc = Scheme(W.cavity(n=8))
    src = SchemeSource(sc, shifted=True, c0=[1, 0, 0])
    assert np.allclose(src.shift_float, [4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
    text = src.header()
    assert "lbm_relax" in text and "LBM_FOR_EACH_V" in text


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "lbm_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\**(lbm_\w+)\s*\(", text, flags=re.M)


def test_core_library_builds_and_exports_header():
    path = runtime.build_core()
    lib = ctypes.CDLL(path)
    names = _declared_symbols()
    core_names = [n for n in names if not n.startswith("lbm_scheme") and n not in runtime_scheme_symbols()]
    assert core_names
    for n in core_names:
        assert hasattr(lib, n), n


def runtime_scheme_symbols():
    return {"lbm_one_time_step", "lbm_one_time_step_periodic", "lbm_transport", "lbm_f2m", "lbm_m2f",
            "lbm_equilibrium", "lbm_relaxation", "lbm_scheme_last_error", "lbm_scheme_describe",
            "lbm_ensemble_step", "lbm_ensemble_step_pairs", "lbm_one_time_step_periodic_closure",
            "lbm_f2m_conserved", "lbm_source_term", "lbm_scheme_set_step_variant", "lbm_scheme_wait_timeouts",
            "lbm_init_conserved", "lbm_f2m_conserved_dense",
            "lbm_one_time_step_walls", "lbm_one_time_step_periodic_closure_tc",
            "lbm_scheme_set_closure_tc_occupancy", "lbm_scheme_closure_tc_occupancy"}


def test_scheme_module_builds_and_exports_header():
    sc = Scheme(W.cavity(n=8))
    mod = runtime.SchemeModule(SchemeSource(sc, shifted=False), "float64", "float64")
    declared = set(_declared_symbols())
    for n in runtime_scheme_symbols():
        assert n in declared
        assert hasattr(mod.lib, n), n
    assert mod.nv == 9 and mod.dim == 2


def test_lattice_layout():
    lat = runtime.lattice(2, 9, "float32", [256, 256], [1, 1])
    assert lat.stride[1] == 1
    assert lat.stride[0] % 8 == 0                    # 32-byte rows
    assert (lat.origin + 1) * 4 % 32 == 0            # interior rows start aligned
    assert lat.vstride * 4 % 128 == 0
    assert lat.elements == 9 * lat.vstride
    lat3 = runtime.lattice(3, 19, "float16", [16, 8, 4], [1, 1, 1])
    assert lat3.stride[2] == 1 and lat3.stride[1] % 16 == 0
    assert lat3.stride[0] == lat3.stride[1] * (8 + 2)


def test_c_abi_rejects_bad_arguments_without_gpu():
    lib = runtime.core()
    lat = runtime.Lattice()
    rc = lib.lbm_lattice_init(ctypes.byref(lat), 4, 9, 0, None, None)
    assert rc == 1
    assert b"NULL" in lib.lbm_last_error() or b"dim" in lib.lbm_last_error()
    n3 = (ctypes.c_int32 * 3)(8, 8, 1)
    h3 = (ctypes.c_int32 * 3)(1, 1, 0)
    assert lib.lbm_lattice_init(ctypes.byref(lat), 2, 9, 7, ctypes.cast(n3, ctypes.c_void_p),
                                ctypes.cast(h3, ctypes.c_void_p)) == 1
    good = runtime.lattice(2, 9, "float64", [8, 8], [1, 1])
    good.n[0] = 0
    assert lib.lbm_update_halo(None, ctypes.byref(good), None) == 1


def test_reference_forms_reproduce_generated_boundary_rhs():
    """Boundary right-hand sides from the printed reference forms equal pylbm's bit for bit."""
    from pylbm_gb300.refforms import ReferenceForms
    for fixture, d in (("cavity_n32.npz", W.cavity(n=32)),
                       ("cylinder_small.npz", W.cylinder(nx=96, ny=32, radius=5, center=(24, 17), re=40.0))):
        g = golden(fixture)
        sim = _HostSim(d)
        rf = ReferenceForms(d)
        sim.feq_host = lambda cons, rf=rf: rf.feq_host(cons)
        bc = Boundary(sim.domain, d)
        for i, meth in enumerate(bc.methods):
            meth.set_iload()
            meth.prepare_rhs(sim)
            meth.fix_iload()
            meth.set_rhs()
            assert np.array_equal(meth.rhs, g[f"bc{i}_rhs"])


def test_reference_forms_print_like_the_generator():
    """Spot checks of the printed constants and term order of the reference generator."""
    from pylbm_gb300.refforms import ReferenceForms
    rf = ReferenceForms(W.cavity(n=32))
    relax = rf.relaxation()
    assert relax[0] == ("m[3] = -4.5*(0.666666666666667*m[0] - 1.0*(m[1]*m[1]) - 1.0*(m[2]*m[2]) "
                        "+ 0.111111111111111*m[3]);")
    assert rf.populations()[0] == ("g[0] = (0.1111111111111111)*m[0] - 0.111111111111111*m[3] "
                                   "+ 0.111111111111111*m[4];")
    assert rf.moments_pull()[0].startswith("m[0] = g[7] + g[6] + g[3] + g[8]")
    # the standalone m2f routine orders indexed moments by their printed index
    r3 = ReferenceForms(W.tgv3d(n=8))
    line = r3.populations_routine()[1]
    assert line.index("m[10]") < line.index("m[3]")


def test_fast_and_reference_styles_share_constants():
    sc = Scheme(W.cavity(n=8))
    fast = SchemeSource(sc, shifted=False)
    ref = SchemeSource(sc, shifted=False, style="reference")
    # both styles forbid implicit contraction; the fast one fuses explicitly
    assert ref.nvcc_flags == ["-fmad=false"] and fast.nvcc_flags == ["-fmad=false"]
    assert "lbm_fma<R>" in fast.header() and "lbm_fma" not in ref.header()
    assert "0.666666666666667" in ref.header()
    with pytest.raises(SchemeError):
        SchemeSource(sc, shifted=True, c0=[1, 0, 0], style="reference")


def test_periodic_domain_without_flags():
    d = W.tgv3d(n=8)
    dom = Domain(d, with_flags=False)
    assert dom.flag is None and dom.shape_in == [8, 8, 8]
    full = Domain(d)
    assert [c.tolist() for c in dom.coords_halo] == [c.tolist() for c in full.coords_halo]
    with pytest.raises(ValueError):
        Domain(W.cavity(n=8), with_flags=False)


def test_domain_coordinate_accessors():
    """pylbm's Domain.x / y / z, *_halo and get_bounds (pylbm/domain.py:318-361, 444-461)."""
    from pylbm_gb300.domain import Domain
    d = W.cavity(n=8)
    sc = Scheme(d)
    dom = Domain(d, sc.stencil)
    assert np.array_equal(dom.x, dom.coords[0]) and np.array_equal(dom.y_halo, dom.coords_halo[1])
    assert dom.x.size == 8 and dom.x_halo.size == 10
    lo, hi = dom.get_bounds()
    assert np.allclose(lo, [1 / 16, 1 / 16]) and np.allclose(hi, [15 / 16, 15 / 16])
    lo, hi = dom.get_bounds_halo()
    assert np.allclose(lo, [-1 / 16, -1 / 16]) and np.allclose(hi, [17 / 16, 17 / 16])


def test_float_form_constants_reproduce_the_physical_formula():
    """LBM_BC_FLOAT_FORM: +/- g0 + c (Bouzidi: (1-d) g1 +/- d g0 + c) on stored
    deviations equals the float64 formula on physical values minus the store shift."""
    from pylbm_gb300.simulation import float_form_constants
    rng = np.random.default_rng(7)
    n, nv = 200, 9
    shift = rng.uniform(0.02, 0.45, nv)
    rows = lambda: np.column_stack([rng.integers(0, nv, n), rng.integers(0, 40, (n, 2))])  # noqa: E731
    il0, il1, st = rows(), rows(), rows()
    rhs, dist = rng.uniform(-0.1, 0.1, n), rng.uniform(0.0, 1.0, n)
    g0, g1 = rng.uniform(-1e-3, 1e-3, n), rng.uniform(-1e-3, 1e-3, n)
    f0, f1 = g0 + shift[il0[:, 0]], g1 + shift[il1[:, 0]]
    for kind, sign in (("bounce_back", 1), ("anti_bounce_back", -1), ("neumann", 1)):
        c = float_form_constants(kind, [il0], st, rhs, None, shift).astype(np.float64)
        want = sign * f0 + (0.0 if kind == "neumann" else rhs) - shift[st[:, 0]]
        assert np.abs(sign * g0 + c - want).max() < 1e-7
    for kind, sign in (("bouzidi_bounce_back", 1), ("bouzidi_anti_bounce_back", -1)):
        c = float_form_constants(kind, [il0, il1], st, rhs, dist, shift).astype(np.float64)
        want = (1 - dist) * f1 + sign * dist * f0 + rhs - shift[st[:, 0]]
        assert np.abs((1 - dist) * g1 + sign * dist * g0 + c - want).max() < 1e-7


def test_flat_slots_match_the_lattice_layout():
    from pylbm_gb300.simulation import flat_slots
    lat = runtime.Lattice()
    lat.vstride, lat.origin = 5000, 13
    lat.stride[0], lat.stride[1], lat.stride[2] = 70, 1, 0
    rows = np.array([[0, 0, 0], [2, 3, 4], [8, 41, 69]])
    assert flat_slots(rows, lat, 2).tolist() == [13, 2 * 5000 + 13 + 3 * 70 + 4, 8 * 5000 + 13 + 41 * 70 + 69]


@pytest.mark.parametrize("case,storage", [("d2q13_advection", "float16"), ("d1q5_advection", "bfloat16"),
                                          ("karman_3d", "float16"), ("riemann_p_system", "float32")])
def test_rare_template_paths_compile(case, storage):
    """Modules whose kernels take the less common template paths build for
    sm_103a and load: reach 2 (no two-node path), 1D, 3D relative-velocity
    free D3Q15 with Bouzidi links in FP16, real powers (p-system)."""
    import demo_cases
    sc = Scheme(demo_cases.CASES[case][0]())
    c0 = [1.0] + [0.0] * (sc.nconsm - 1)
    mod = runtime.SchemeModule(SchemeSource(sc, shifted=True, c0=c0, simplify_frame=True), storage, "float32")
    for n in runtime_scheme_symbols():
        assert hasattr(mod.lib, n), n
    assert mod.nv == sc.nv and mod.dim == sc.dim
