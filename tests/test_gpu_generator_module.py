"""pylbm's call sequence through ``CudaModule`` on the GPU.

Each step is driven the way pylbm drives its generated module: the ghost
refresh one axis at a time (``Array.update``, pylbm/storage.py:307-367), every
boundary routine, then ``one_time_step`` (pylbm/simulation.py:374-420), all
called through a by-name binder equal to ``call_genfunction``
(pylbm/symbolic.py:288-299)."""
import inspect

import numpy as np
import pytest

import demo_cases
from conftest import golden
from pylbm_gb300 import Simulation
from pylbm_gb300.generator import CudaModule, LinkArray, to_device

pytestmark = pytest.mark.gpu


def call(fn, namespace):
    fn(**{k: namespace[k] for k in inspect.getfullargspec(fn).args})


def space(a):
    return dict(zip(("nx", "ny", "nz"), a.nspace))


def run(mod, f, fnew, methods, steps, params=None):
    for _ in range(steps):
        ns = dict(f=f, nv=f.nv, **space(f))
        for axis in "xyz"[:f.dim]:
            call(getattr(mod, "update_" + axis), ns)
        for name, lists in methods:
            call(getattr(mod, name), dict(f=f, fcopy=None, **space(f), **lists))
        call(mod.one_time_step, dict(f=f, fnew=fnew, **space(f), **(params or {})))
        f, fnew = fnew, f
    return f, fnew


def test_cavity_from_reference_lists_matches_reference_moments():
    """The reference's own boundary lists and initial moments (fixture), 300
    steps through the module, pylbm's moments bit for bit."""
    from pylbm_gb300 import workloads as W
    g = golden("cavity_n32.npz")
    mod = CudaModule(W.cavity(n=32))
    nspace = [34, 34]
    f, fnew, m = mod.populations(nspace), mod.populations(nspace), mod.moments(nspace)
    # pylbm's initialisation: conserved moments rho = 1, q = 0 on the whole
    # box, equilibrium of the others, then m2f (pylbm/simulation.py:258-313)
    m0 = np.zeros((9, 34, 34))
    m0[0] = 1.0
    m.set(m0)
    call(mod.equilibrium, dict(m=m, **space(m)))
    call(mod.m2f, dict(f=f, m=m, **space(f)))
    call(mod.f2m, dict(f=f, m=m, **space(f)))
    assert np.array_equal(m.get()[:, 1:-1, 1:-1], g["m0"])
    lists = {"iload0": to_device(g["bc0_iload0"]), "istore": to_device(g["bc0_istore"]),
             "rhs": to_device(g["bc0_rhs"]), "ncond": int(g["bc0_istore"].shape[0])}
    f, fnew = run(mod, f, fnew, [("bounce_back", lists)], 300)
    call(mod.f2m, dict(f=f, m=m, **space(f)))
    assert np.array_equal(m.get()[:, 1:-1, 1:-1], g["m300"])


@pytest.mark.parametrize("name,dtype", [("karman_vortex_street", "float64"), ("poiseuille_3d", "float64"),
                                        ("euler_1d", "float64"), ("poiseuille_vec", "float32")])
def test_module_equals_simulation(name, dtype):
    """Bouzidi, Neumann and 1D/3D routines through the module equal
    ``Simulation`` (full ghost refresh) bit for bit."""
    build = demo_cases.CASES[name][0]
    sim = Simulation(build(), dtype=dtype, halo="full")
    sim.batch_boundary = False  # the per-method kernels, as pylbm calls them
    c0 = [float(c) for c in sim.module.src.c0] if dtype != "float64" else None
    mod = CudaModule(build(), storage=dtype, c0=c0)
    assert np.array_equal(mod.module.shift, sim.module.shift)
    nspace = sim.domain.shape_halo
    f, fnew = mod.populations(nspace), mod.populations(nspace)
    f.set(np.array([sim.F_halo[k] for k in range(sim.scheme.nv)]))
    methods = []
    for meth in sim.bc.methods:
        lists = {"istore": LinkArray(meth.istore), "rhs": LinkArray(meth.rhs), "ncond": meth.ncond}
        for i, il in enumerate(meth.iload):
            lists[f"iload{i}"] = LinkArray(il)
        if hasattr(meth, "s"):
            lists["dist"] = LinkArray(np.asarray(meth.s, dtype=np.float64))
        methods.append((meth.name, lists))
    params = {("lambda_" if k == "lambda" else k): v for k, v in sim.extra_parameters_str().items()}
    params.setdefault("dt", sim.dt)
    steps = 12
    f, fnew = run(mod, f, fnew, methods, steps, params)
    sim.run(steps)
    ref = np.array([sim.F[k] for k in range(sim.scheme.nv)])
    inner = (slice(None),) + tuple(slice(int(h), -int(h)) for h in sim.domain.halo)
    assert np.array_equal(f.get()[inner], ref)


def test_update_axis_is_one_periodic_pass():
    """update_x alone wraps along x only (ghost rows in y keep their values)."""
    from pylbm_gb300 import workloads as W
    mod = CudaModule(W.cavity(n=8))
    f = mod.populations([10, 12])
    rng = np.random.default_rng(5)
    host = rng.standard_normal((9, 10, 12))
    f.set(host)
    call(mod.update_x, dict(f=f, nx=10, ny=12, nv=9))
    want = host.copy()
    want[:, 0, :] = host[:, 8, :]
    want[:, 9, :] = host[:, 1, :]
    assert np.array_equal(f.get(), want)
    call(mod.update_y, dict(f=f, nx=10, ny=12, nv=9))
    want2 = want.copy()
    want2[:, :, 0] = want[:, :, 10]
    want2[:, :, 11] = want[:, :, 1]
    assert np.array_equal(f.get(), want2)


def test_run_time_parameter_by_name():
    """A periodic shear layer whose rate omega is a run-time parameter: pylbm
    passes it to one_time_step by name; ghost refresh axis by axis, then the
    step, equals Simulation (which wraps inside the periodic kernel) bit for bit."""
    import sympy as sp
    from pylbm_gb300 import workloads as W
    omega = sp.Symbol("omega")
    w = W.omega_from_nu(2e-3)
    sim = Simulation(W.shear_layer(n=32, omega=omega))
    sim.extra_parameters = {omega: w}
    mod = CudaModule(W.shear_layer(n=32, omega=omega))
    assert "omega" in inspect.getfullargspec(mod.one_time_step).args
    nspace = sim.domain.shape_halo
    f, fnew = mod.populations(nspace), mod.populations(nspace)
    f.set(np.array([sim.F_halo[k] for k in range(9)]))
    f, fnew = run(mod, f, fnew, [], 10, {"omega": w})
    sim.run(10)
    ref = np.array([sim.F[k] for k in range(9)])
    assert np.array_equal(f.get()[:, 1:-1, 1:-1], ref)
