"""Domain construction on the device (lbm_domain_* and lbm_links_* kernels).

The GPU builds the fluid/solid map, the per-link wall distances and labels
and the boundary link lists; everything must equal the host construction
(which the reference fixtures pin) bit for bit, lists in the same order.
"""
import numpy as np
import pytest

import demo_cases
import element_cases
from conftest import golden
from pylbm_gb300 import geometry
from pylbm_gb300 import workloads as W
from pylbm_gb300.boundary import Boundary
from pylbm_gb300.domain import Domain
from pylbm_gb300.scheme import Scheme
from test_elements import assert_domain_equals_fixture

pytestmark = pytest.mark.gpu

CASES = {
    "cylinder": lambda: W.cylinder(nx=256, ny=96, radius=11, center=(60, 47), re=100.0),
    "karman": lambda: demo_cases.karman_vortex_street(),
    "air_conditioning": lambda: demo_cases.air_conditioning(),
    "bend": lambda: demo_cases.bend(),
    "cavity": lambda: W.cavity(n=48),
    "poiseuille_3d": lambda: demo_cases.poiseuille_3d(),
    "euler_1d": lambda: demo_cases.euler_1d(),
    "rayleigh_benard": lambda: demo_cases.rayleigh_benard(),
    # 3D: pylbm's flow past a sphere (D3Q15, Bouzidi on the sphere) and a
    # sphere in the lid-driven cube (D3Q19, off-grid centre)
    "karman_3d": lambda: demo_cases.karman_3d(),
    "sphere_cube": lambda: _sphere_cube(),
}


def _sphere_cube():
    from pylbm_gb300.geometry import Sphere
    d = W.cavity3d(n=40)
    d["elements"] = [Sphere((0.43, 0.51, 0.37), 0.17, label=2)]
    d["boundary_conditions"][2] = {"method": {0: d["boundary_conditions"][0]["method"][0]}}
    return d


@pytest.mark.parametrize("name", list(CASES))
def test_device_domain_equals_host(name):
    d = CASES[name]()
    sc = Scheme(d)
    host = Domain(d, sc.stencil)
    dev = Domain(d, sc.stencil, device=True)
    ioo, dist, flag = dev.download_arrays()
    assert np.array_equal(ioo, host.in_or_out)
    assert np.array_equal(flag, host.flag)
    assert np.array_equal(dist.view(np.int64), host.distance.view(np.int64))  # bit for bit
    bh, bd = Boundary(host, d), Boundary(dev, d)
    assert [type(m) for m in bh.methods] == [type(m) for m in bd.methods]
    for mh, md in zip(bh.methods, bd.methods):
        assert np.array_equal(mh.istore, md.istore)
        assert np.array_equal(mh.ilabel, md.ilabel)
        assert np.array_equal(mh.distance.view(np.int64), md.distance.view(np.int64))


@pytest.mark.parametrize("name", list(element_cases.cases(geometry)))
def test_device_elements_equal_host_and_reference(name):
    """Ellipse, triangle, ellipsoid and the four cylinders built on the device:
    the same arrays as the host build, bit for bit, and as the reference's
    own Domain (tests/golden/elements.npz; distances to 1e-13 relative, the
    fixture's host libraries may round a tilted frame differently)."""
    d = element_cases.cases(geometry)[name]
    host = Domain(d)
    dev = Domain(d, device=True)
    ioo, dist, flag = dev.download_arrays()
    assert np.array_equal(ioo, host.in_or_out)
    assert np.array_equal(flag, host.flag)
    assert np.array_equal(dist.view(np.int64), host.distance.view(np.int64))
    host.in_or_out, host.distance, host.flag = ioo, dist, flag
    assert_domain_equals_fixture(host, name, golden("elements.npz"), rtol=1e-13)


def test_large_disc_domain_on_device():
    """A 4096 x 1024 channel with a disc: built and listed on the device, same lists."""
    d = W.cylinder(nx=4096, ny=1024, radius=64, center=(800, 513), re=200.0)
    sc = Scheme(d)
    dev = Domain(d, sc.stencil, device=True)
    host = Domain(d, sc.stencil)
    bh, bd = Boundary(host, d), Boundary(dev, d)
    for mh, md in zip(bh.methods, bd.methods):
        assert np.array_equal(mh.istore, md.istore)


def test_simulation_with_device_domain_is_identical():
    d = demo_cases.karman_vortex_street()
    runs = []
    for dev in (False, True):
        from pylbm_gb300 import Simulation
        sim = Simulation(d, device_domain=dev)
        sim.run(20)
        runs.append(np.array([sim.m[k] for k in range(sim.scheme.nv)]))
        sim.free()
    assert np.array_equal(runs[0], runs[1])
