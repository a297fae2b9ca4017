"""GPU parity: the CUDA path against the oracle and the reference fixtures.

Every test drives the kernels through the C ABI (pylbm_gb300.runtime ->
liblbm_gb300.so / lbm_scheme_<id>.so).  Integer work (boundary index lists,
halo copies) must be bit-exact; FP64 arithmetic is held to the reference's
own tolerance (max relative error per moment, ``rel_err``).
"""
import ctypes

import numpy as np
import pytest

from conftest import golden, rel_err
from oracle import OracleSimulation, lib as oracle_lib
from pylbm_gb300 import Simulation, runtime
from pylbm_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _gpu_moments(sim):
    return np.array([sim.m[k] for k in range(sim.scheme.nv)])


def test_cavity_fp64_matches_reference_and_oracle():
    """Parity form: bit-identical to pylbm's Cython output (bound asked for: 1e-12)."""
    g = golden("cavity_n32.npz")
    sim = Simulation(W.cavity(n=32))
    assert np.array_equal(_gpu_moments(sim), g["m0"])
    o = OracleSimulation(W.cavity(n=32))
    o.initialize()
    sim.run(50)
    o.run(50)
    assert np.array_equal(_gpu_moments(sim), g["m50"])
    assert rel_err(_gpu_moments(sim), o.moments()).max() < 1e-12
    sim.run(250)
    o.run(250)
    assert np.array_equal(_gpu_moments(sim), g["m300"])
    assert rel_err(_gpu_moments(sim), o.moments()).max() < 2e-12


def test_cavity_fast_form_within_tolerance():
    """The exact-constant FP64 form (parity=False) stays within 2e-12 after 300 steps."""
    g = golden("cavity_n32.npz")
    sim = Simulation(W.cavity(n=32), parity=False)
    sim.run(300)
    assert rel_err(_gpu_moments(sim), g["m300"]).max() < 2e-12


def test_cylinder_fp64_boundaries_match_reference():
    """Anti-bounce-back inflow, Neumann-x outflow, bounce-back disc, periodic y."""
    d = W.cylinder(nx=96, ny=32, radius=5, center=(24, 17), re=40.0)
    g = golden("cylinder_small.npz")
    sim = Simulation(d)
    sim.run(100)
    assert np.array_equal(_gpu_moments(sim), g["m100"])


def test_tgv3d_fp64_matches_reference():
    g = golden("tgv3d_n16.npz")
    sim = Simulation(W.tgv3d(n=16))
    assert sim.periodic
    assert rel_err(_gpu_moments(sim), g["m0"]).max() < 1e-14
    sim.run(20)
    assert rel_err(_gpu_moments(sim), g["m20"]).max() < 1e-14


def test_shear_layer_fp64_matches_reference():
    g = golden("shear_n64.npz")
    sim = Simulation(W.shear_layer(n=64))
    sim.run(200)
    # bit-identical on the GB300 host; the bound leaves room for the last bit
    # of the host libm's tanh/sin in the initial data
    assert rel_err(_gpu_moments(sim), g["m200"]).max() < 1e-14


def test_periodic_kernel_equals_ghost_kernel():
    """Wrapped pull == halo refresh + ghost pull, bit for bit."""
    a = Simulation(W.shear_layer(n=48))
    b = Simulation(W.shear_layer(n=48))
    b.periodic = False  # force halo refresh + lbm_one_time_step
    a.run(30)
    b.run(30)
    ma, mb = _gpu_moments(a), _gpu_moments(b)
    assert np.array_equal(ma, mb)


def test_halo_kernel_bit_exact_against_oracle():
    rng = np.random.default_rng(1)
    for dim, n, h in ((2, [13, 7], [1, 1]), (3, [5, 6, 4], [1, 1, 1]), (2, [9, 8], [2, 2])):
        nv = 5
        lat = runtime.lattice(dim, nv, "float64", n, h)
        shape = [nv] + [x + 2 * y for x, y in zip(n, h)]
        host = rng.standard_normal(shape)
        buf = runtime.DeviceBuffer(lat.elements * 8)
        flat = np.zeros(lat.elements)
        view = np.lib.stride_tricks.as_strided(flat[lat.origin:], shape=shape,
                                               strides=[lat.vstride * 8] + [lat.stride[d] * 8 for d in range(dim)])
        view[...] = host
        buf.upload(flat)
        runtime.check(runtime.core().lbm_update_halo(buf.handle, ctypes.byref(lat), None))
        buf.download(flat)
        ref = np.ascontiguousarray(host)
        n32 = np.array(n, dtype=np.int32)
        h32 = np.array(h, dtype=np.int32)
        oracle_lib().oracle_update_halo(ref.ctypes.data_as(ctypes.c_void_p), dim, nv,
                                        n32.ctypes.data_as(ctypes.c_void_p), h32.ctypes.data_as(ctypes.c_void_p))
        assert np.array_equal(np.array(view), ref)


@pytest.mark.parametrize("kind", ["bounce_back", "anti_bounce_back", "neumann"])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_boundary_kernels_against_oracle(kind, dtype):
    d = W.cylinder(nx=40, ny=16, radius=3, center=(12, 8), re=20.0)
    sim = Simulation(d, dtype=dtype)
    meth = sim.bc.methods[0]
    rng = np.random.default_rng(2)
    rhs = rng.standard_normal(meth.ncond)
    nv = sim.scheme.nv
    shape = [nv] + sim.domain.shape_halo
    host = rng.uniform(0.0, 0.2, shape)
    for k in range(nv):
        sim.F_halo[k] = host[k]
    ref = np.array([sim.F_halo[k] for k in range(nv)])
    il = runtime.DeviceBuffer(meth.iload[0].nbytes)
    il.upload(meth.iload[0])
    st = runtime.DeviceBuffer(meth.istore.nbytes)
    st.upload(meth.istore)
    rb = runtime.DeviceBuffer(rhs.nbytes)
    rb.upload(rhs)
    core = runtime.core()
    lat = ctypes.byref(sim._lat)
    if kind == "bounce_back":
        rc = core.lbm_bounce_back(sim._F.handle, il.handle, st.handle, meth.ncond, rb.handle, lat, 0, None)
        sign, r = 1.0, rhs
    elif kind == "anti_bounce_back":
        rc = core.lbm_anti_bounce_back(sim._F.handle, il.handle, st.handle, meth.ncond, rb.handle, lat, 0, None)
        sign, r = -1.0, rhs
    else:
        rc = core.lbm_neumann(sim._F.handle, il.handle, st.handle, meth.ncond, lat, 0, None)
        sign, r = 1.0, None
    runtime.check(rc)
    got = np.array([sim.F_halo[k] for k in range(nv)])
    n32 = np.array(sim.domain.shape_in, dtype=np.int32)
    h32 = np.array(sim.domain.halo, dtype=np.int32)
    ref = np.ascontiguousarray(ref)
    oracle_lib().oracle_boundary(ref.ctypes.data_as(ctypes.c_void_p), 2, nv, n32.ctypes.data_as(ctypes.c_void_p),
                                 h32.ctypes.data_as(ctypes.c_void_p), meth.iload[0].ctypes.data_as(ctypes.c_void_p),
                                 meth.istore.ctypes.data_as(ctypes.c_void_p), meth.ncond,
                                 r.ctypes.data_as(ctypes.c_void_p) if r is not None else None, sign)
    tol = 0.0 if dtype == "float64" else 1e-6
    assert np.abs(got - ref).max() <= tol


def test_population_sums_and_conservation():
    sim = Simulation(W.shear_layer(n=64))
    c0 = sim.conserved_sums()
    sim.run(100)
    c1 = sim.conserved_sums()
    assert abs(c1[0] - c0[0]) <= 1e-12 * abs(c0[0])
    assert np.all(np.abs(c1[1:] - c0[1:]) <= 1e-12 * abs(c0[0]))
    sums, bad = sim.population_sums()
    ref = np.array([sim.F[k].sum() for k in range(sim.scheme.nv)])
    assert bad == 0
    assert np.allclose(sums, ref, rtol=1e-13, atol=1e-12)


@pytest.mark.parametrize("dtype,tol", [("float32", 2e-5), ("float16", 2e-2), ("bfloat16", 1e-1)])
def test_reduced_precision_tgv_error_bound(dtype, tol):
    """Shifted low-precision storage, FP32 arithmetic, against the FP64 oracle."""
    o = OracleSimulation(W.tgv3d(n=24), nthreads=4)
    o.run(40)
    ref = o.moments()
    sim = Simulation(W.tgv3d(n=24), dtype=dtype)
    sim.run(40)
    got = _gpu_moments(sim)
    err = rel_err(got[:4], ref[:4])
    assert err.max() < tol, (dtype, err)


def test_cavity_full_size_fp64_against_reference():
    """The 256^2 cavity after 1000 steps against the reference (sampled fixture)."""
    g = golden("cavity_n256_sampled.npz")
    sim = Simulation(W.cavity(n=256))
    sim.run(int(g["steps"]))
    m = _gpu_moments(sim)
    e = max(rel_err(m[:, ::4, ::4], g["sub"]).max(), rel_err(m[:, :2], g["lo_x"]).max(),
            rel_err(m[:, :, -2:], g["hi_y"]).max())
    assert e <= 1e-12, e
    assert np.array_equal(m[:, ::4, ::4], g["sub"])


@pytest.mark.parametrize("make", [lambda: Simulation(W.cavity(n=48)),
                                  lambda: Simulation(W.shear_layer(n=48), dtype="float32"),
                                  lambda: Simulation(W.cylinder(nx=64, ny=24, radius=4, center=(16, 12), re=30.0),
                                                     dtype="float16")])
def test_graph_replay_equals_step_loop(make):
    """run(n) replays a captured graph of two steps; it must equal n one_time_step calls bit for bit."""
    a, b = make(), make()
    a.run(37)
    for _ in range(37):
        b.one_time_step()
    assert a.nt == b.nt == 37 and a.t == b.t
    assert np.array_equal(_gpu_moments(a), _gpu_moments(b))


@pytest.mark.parametrize("case,steps,tol", [("karman", 100, 5e-5), ("kelvin_helmholtz", 60, 2e-4)])
def test_relative_velocity_fp32_against_oracle(case, steps, tol, monkeypatch):
    """Geier relative-velocity schemes in FP32 against the FP64 oracle.

    The FP32 module writes the moving-frame equilibrium T(u) m_eq simplified
    with u = q / rho (constants times rho); the FP64 oracle evaluates T(u)
    times m_eq as pylbm does.  The simplified form is as close to the oracle
    as the FP32 module that evaluates T(u) m_eq term by term."""
    import demo_cases
    from pylbm_gb300 import simulation as simulation_module
    if case == "karman":
        make = lambda: W.karman(dx=1.0 / 32)  # noqa: E731
    else:
        make = lambda: demo_cases.kelvin_helmholtz(dx=1.0 / 32)  # noqa: E731
    o = OracleSimulation(make())
    o.run(steps)
    ref = o.moments()
    errs = []
    for simplify in (True, False):
        if not simplify:
            base = simulation_module.SchemeSource

            class TermByTerm(base):
                def __init__(self, *a, **k):
                    k["simplify_frame"] = False
                    super().__init__(*a, **k)
            monkeypatch.setattr(simulation_module, "SchemeSource", TermByTerm)
        sim = Simulation(make(), dtype="float32")
        assert sim.module.src.simplify_frame == simplify
        sim.run(steps)
        got = _gpu_moments(sim)
        dom = sim.domain
        fluid = np.ones(dom.shape_in, dtype=bool)
        if dom.in_or_out is not None:
            inner = tuple(slice(int(h), -int(h)) for h in dom.halo)
            fluid = dom.in_or_out[inner] == dom.valin
        assert np.isfinite(got).all()
        errs.append(rel_err(got[:3, fluid], ref[:3, fluid]).max())
        sim.free()
    assert errs[0] < tol, errs
    assert errs[0] <= 1.5 * errs[1], errs


@pytest.mark.parametrize("dtype,tol", [("float64", 1e-12), ("float32", 2e-5)])
def test_lid_driven_cube_against_oracle(dtype, tol):
    """D3Q19 cube with bounce-back on all six walls and a moving lid (the
    bounded 3D bench workload at 16^3) against the FP64 oracle."""
    o = OracleSimulation(W.cavity3d(n=16))
    o.run(30)
    ref = o.moments()
    sim = Simulation(W.cavity3d(n=16), dtype=dtype)
    sim.run(30)
    got = _gpu_moments(sim)
    assert np.isfinite(got).all()
    err = rel_err(got[:4], ref[:4])
    assert err.max() < tol, err
