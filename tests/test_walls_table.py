"""Bounce-back box walls folded into the pull (boundary.box_wall_table), on the CPU.

The oracle applies pylbm's bounce-back links to the ghost slots of a random
population state (pylbm/boundary.py:400-469); the pull from those ghosts
must equal the folded value f_k'(x) + c[k][signature] at every wall node.
Domains with other boundary methods get no table.
"""
import numpy as np
import pytest

from oracle import OracleSimulation, _p, lib
from pylbm_gb300 import workloads as W
from pylbm_gb300.boundary import box_wall_table, wall_signature


def _table(o):
    o.initialize()
    return box_wall_table(o.bc.methods, o.domain.shape_in, o.domain.halo,
                          o.scheme.stencil.get_all_velocities(), [m.rhs for m in o.bc.methods])


@pytest.mark.parametrize("case", ["cavity", "cube"])
def test_folded_pull_equals_bounce_back_links(case):
    d = W.cavity(n=24) if case == "cavity" else W.cavity3d(n=12)
    o = OracleSimulation(d)
    table = _table(o)
    assert table is not None
    sc = o.scheme
    rng = np.random.default_rng(1)
    f = np.ascontiguousarray(rng.random(o.f.shape))
    ghosts = f.copy()
    for meth in o.bc.methods:
        lib().oracle_boundary(_p(ghosts), o.dim, sc.nv, _p(o.n), _p(o.h), _p(meth.iload[0]), _p(meth.istore),
                              meth.ncond, _p(meth.rhs), 1.0)
    v = sc.stencil.get_all_velocities()
    sym = sc.stencil.get_symmetric()
    n, h = o.domain.shape_in, o.domain.halo
    inner = tuple(slice(int(hh), int(hh) + int(nn)) for hh, nn in zip(h, n))
    coords = np.meshgrid(*[np.arange(int(hh), int(hh) + int(nn)) for hh, nn in zip(h, n)], indexing="ij")
    walls = 0
    for k in range(sc.nv):
        src = [c - int(v[k, dd]) for dd, c in enumerate(coords)]
        pulled = ghosts[(k,) + tuple(src)]
        sig = wall_signature(np.array([s.ravel() for s in src]), n, h).reshape(pulled.shape)
        folded = np.where(sig == 13, pulled, f[(int(sym[k]),) + inner] + table[k][sig])
        walls += int(np.count_nonzero(sig != 13))
        assert np.array_equal(folded, pulled), k
    assert walls > 0


def test_no_table_for_other_boundary_methods():
    o = OracleSimulation(W.cylinder(nx=96, ny=32, radius=5, center=(24, 17), re=40.0))
    assert _table(o) is None  # anti-bounce-back inflow, Neumann outflow, periodic axis
