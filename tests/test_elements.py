"""Every analytic element of pylbm on the host (pylbm_gb300.geometry).

The domains of tests/element_cases.py are built with this package's element
classes and compared bit for bit with the reference's own Domain arrays
(tests/golden/elements.npz, made by tests/golden/make_element_golden.py):
fluid/solid map, and for every link the wall distance and label.  Where the
reference sources are present, each element's point_inside and distance are
also compared with the reference's element on random points and rays.
"""
import os
import sys

import numpy as np
import pytest

import element_cases
from conftest import ROOT, golden
from pylbm_gb300 import geometry
from pylbm_gb300.domain import Domain


def sparse_links(dom):
    """(u, node, distance, flag) of the links whose flag is not 999, velocities
    as vectors, in the fixture's order (velocity index, then node)."""
    links = np.nonzero(dom.flag != 999)
    node = np.ravel_multi_index(links[1:], dom.flag.shape[1:])
    return links[0], node, dom.distance[links], dom.flag[links]


def assert_domain_equals_fixture(dom, name, g, rtol=0.0):
    """rtol = 0: distances bit for bit.  A tilted cylinder's frame comes from
    LAPACK's inverse and a BLAS product, whose last bits depend on the host's
    library build: on another machine than the fixture's, distances agree to
    rtol and everything else exactly."""
    fluid = dom.in_or_out == 999
    assert np.array_equal(fluid, g[name + "/fluid"])
    ref_v = g[name + "/velocities"]
    mine = {tuple(v): k for k, v in enumerate(dom.stencil.unique_v)}
    assert len(mine) == len(ref_v)
    # the reference's velocity index -> this domain's
    perm = np.array([mine[tuple(v)] for v in ref_v])
    u, node, dist, flag = sparse_links(dom)
    ru = perm[g[name + "/u"].astype(np.int64)]
    order = np.lexsort((g[name + "/node"], ru))
    mo = np.lexsort((node, u))
    assert np.array_equal(u[mo], ru[order])
    assert np.array_equal(node[mo], g[name + "/node"][order])
    assert np.array_equal(flag[mo], g[name + "/flag"][order].astype(np.int64))
    if rtol == 0.0:
        assert np.array_equal(dist[mo].view(np.int64), g[name + "/distance"][order].view(np.int64))
    else:
        assert np.allclose(dist[mo], g[name + "/distance"][order], rtol=rtol, atol=0.0)


@pytest.mark.parametrize("name", list(element_cases.cases(geometry)))
def test_domain_with_elements_equals_reference(name):
    g = golden("elements.npz")
    dico = element_cases.cases(geometry)[name]
    dom = Domain(dico)
    assert_domain_equals_fixture(dom, name, g)


def test_element_checks():
    with pytest.raises(ValueError):
        geometry.Ellipse([0, 0], [1, 0], [0.5, 1])
    with pytest.raises(ValueError):
        geometry.Ellipsoid([0, 0, 0], [1, 0, 0], [0.5, 1, 0], [0, 0, 1])
    with pytest.raises(ValueError):
        geometry.CylinderCircle([0, 0, 0], [1, 0, 0], [0, 2, 0], [0, 0, 1])
    p = geometry.Parallelepiped([0.1, 0.2, 0.3], [1, 0, 0], [0, 1, 0], [0, 0, 2])
    assert p.label == [0] * 6 and np.allclose(p.center, [0.1, 0.2, 1.3])
    t = geometry.CylinderTriangle([0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], label=[1, 2, 3, 4, 5])
    # the frame: (v1, v2, w) -> unit section, z in [-1, 1]
    inside = t.point_inside(np.meshgrid([0.2, 0.8], [0.2, 0.8], [-0.9, 1.1], sparse=True, indexing="ij"))
    assert inside[0, 0].tolist() == [True, False] and not inside[1, 1].any()


def reference_elements():
    ref = os.environ.get("PYLBM_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
    if not os.path.isfile(os.path.join(ref, "pylbm", "elements", "__init__.py")):
        pytest.skip("the reference pylbm sources are not present on this machine")
    sys.dont_write_bytecode = True
    for p in (ref, os.path.join(ROOT, "oracle", "shims")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import pylbm
    return pylbm


@pytest.mark.parametrize("name", list(element_cases.cases(geometry)))
def test_elements_match_reference_on_random_rays(name):
    ref = reference_elements()
    rng = np.random.default_rng(7)
    mine = element_cases.cases(geometry)[name]
    theirs = element_cases.cases(ref)[name]
    dim = 3 if "z" in mine["box"] else 2
    axes = [np.sort(rng.uniform(-0.05, 1.05, 9 + k)) for k in range(dim)]
    grid = np.meshgrid(*axes, sparse=True, indexing="ij")
    for em, er in zip(mine["elements"], theirs["elements"]):
        assert np.array_equal(em.point_inside(grid), er.point_inside(grid))
        lo_m, hi_m = em.get_bounds()
        lo_r, hi_r = er.get_bounds()
        assert np.array_equal(lo_m, lo_r) and np.array_equal(hi_m, hi_r)
        for _ in range(12):
            v = rng.integers(-2, 3, dim) * 0.05
            if not v.any():
                continue
            am, bm = em.distance(grid, v, 1.0)
            ar, br = er.distance(grid, v, 1.0)[:2]
            hit = ar > 0
            assert np.array_equal(am > 0, hit)
            assert np.array_equal(am[hit].view(np.int64), ar[hit].view(np.int64))
            assert np.array_equal(bm[hit], br[hit])
