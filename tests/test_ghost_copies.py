"""Observed ghost copies (the pruned periodic refresh) against the oracle.

pylbm refreshes every ghost population before the boundary methods
(pylbm/storage.py:307-367, periodic along all axes: pylbm/domain.py:373-383).
``observed_ghost_copies`` keeps only the copies a later read observes.  The
check: the oracle runs each bounded demo case with every other ghost
population set to NaN right after its full refresh, and must reproduce the
unpoisoned run bit for bit on the interior (NaN anywhere it reads would
propagate)."""
import numpy as np
import pytest

import demo_cases
from oracle import OracleSimulation
from pylbm_gb300.boundary import batch_entries, observed_ghost_copies

BOUNDED = ["poiseuille", "poiseuille_vec", "lid_driven_cavity", "karman_vortex_street", "air_conditioning",
           "rayleigh_benard", "burgers_1d", "euler_1d", "poiseuille_3d", "riemann_p_system", "bend",
           "d1q5_advection", "karman_3d", "lid_cavity_3d"]


def copies_of(o):
    return observed_ghost_copies(o.domain.shape_in, o.domain.halo, o.scheme.stencil.get_all_velocities(),
                                 o.bc.methods)


@pytest.mark.parametrize("name", BOUNDED)
def test_unobserved_ghosts_are_never_read(name):
    build = demo_cases.CASES[name][0]
    steps = 4
    ref = OracleSimulation(build())
    ref.run(steps)
    o = OracleSimulation(build())
    o.initialize()
    copies = copies_of(o)
    assert copies is not None
    istore, iload = copies
    dim = o.dim
    h = o.domain.halo
    inner = tuple(slice(int(a), int(a) + int(n)) for a, n in zip(h, o.domain.shape_in))
    poison = np.ones(o.f.shape, dtype=bool)
    poison[(slice(None),) + inner] = False
    poison[tuple(istore.T.astype(np.int64))] = False
    # every copy reads an interior slot and stores a ghost slot
    assert not poison[tuple(iload.T.astype(np.int64))].any()
    for lst in (istore, iload):
        assert lst.shape[1] == dim + 1
    src_inner = np.all((iload[:, 1:] >= np.array(h)) & (iload[:, 1:] < np.array(h) + o.domain.shape_in), axis=1)
    assert src_inner.all()

    def after_halo(f):
        f[poison] = np.nan

    o.after_halo = after_halo
    o.run(steps)
    got = o.f[(slice(None),) + inner]
    want = ref.f[(slice(None),) + inner]
    assert np.array_equal(got, want)


def test_copies_are_periodic_images():
    o = OracleSimulation(demo_cases.CASES["rayleigh_benard"][0]())
    o.initialize()
    istore, iload = copies_of(o)
    assert len(istore) > 0
    n = np.array(o.domain.shape_in)
    h = np.array(o.domain.halo)
    assert np.array_equal(istore[:, 0], iload[:, 0])
    for d in range(o.dim):
        c, s = istore[:, 1 + d], iload[:, 1 + d]
        want = np.where(c < h[d], c + n[d], np.where(c >= n[d] + h[d], c - n[d], c))
        assert np.array_equal(s, want)


def test_fully_walled_domain_needs_no_copy():
    for name in ("lid_driven_cavity", "karman_vortex_street", "lid_cavity_3d"):
        o = OracleSimulation(demo_cases.CASES[name][0]())
        o.initialize()
        assert len(copies_of(o)[0]) == 0


def test_short_axis_keeps_the_full_refresh():
    class M:
        istore = np.zeros((0, 3), np.int32)
        iload = []
    assert observed_ghost_copies([1, 8], [2, 2], [[0, 0], [1, 0]], [M()]) is None


def _batch_phase(o, copies, entries, joined):
    """The boundary phase as one batched launch computes it: every link reads
    the populations as they are before the launch, then all links store."""
    def load(f, rows):
        return f[tuple(np.asarray(rows, dtype=np.int64).T)]

    def phase(f):
        for m in o.bc.methods:
            if m.update_feq(o):
                m.set_rhs()
        if len(copies[0]) and not joined:  # copies that cannot join run first
            f[tuple(copies[0].T.astype(np.int64))] = load(f, copies[1])
        f0 = f.copy()
        out = []
        if joined:
            out.append((copies[0], load(f0, copies[1])))
        for e in entries:
            m = o.bc.methods[e["method"]]
            sel = slice(None) if e["links"] is None else e["links"]
            rhs = np.asarray(m.rhs)[sel]
            kind = e["kind"]
            if kind == "bounce_back":
                v = load(f0, e["iload"][0]) + rhs
            elif kind == "anti_bounce_back":
                v = -load(f0, e["iload"][0]) + rhs
            elif kind == "neumann":
                v = load(f0, e["iload"][0])
            else:
                d = np.asarray(m.s, dtype=np.float64)[sel]
                t1 = (1.0 - d) * load(f0, e["iload"][1])
                t0 = d * load(f0, e["iload"][0])
                v = (t1 - t0 if kind == "bouzidi_anti_bounce_back" else t1 + t0) + rhs
            out.append((e["istore"], v))
        for st, v in out:
            f[tuple(np.asarray(st, dtype=np.int64).T)] = v
    return phase


@pytest.mark.parametrize("name", BOUNDED)
def test_one_batched_boundary_launch_equals_the_sequential_phase(name):
    """batch_entries (one launch: ghost copies joined, loads of copied ghosts
    forwarded, Neumann loads of stored slots given the storing formula) gives
    the same interior as pylbm's refresh + methods one after the other."""
    build = demo_cases.CASES[name][0]
    steps = 4
    ref = OracleSimulation(build())
    ref.run(steps)
    o = OracleSimulation(build())
    o.initialize()
    copies = copies_of(o)
    ext = [o.scheme.nv] + list(o.domain.shape_halo)
    plan = batch_entries(o.bc.methods, ext, copies if len(copies[0]) else None)
    if plan is None:
        pytest.skip("the methods of this case stay sequential")
    entries, joined = plan
    o.boundary_phase = _batch_phase(o, copies, entries, joined)
    o.run(steps)
    inner = (slice(None),) + tuple(slice(int(a), int(a) + int(n)) for a, n in zip(o.domain.halo, o.domain.shape_in))
    assert np.array_equal(o.f[inner], ref.f[inner])


def test_outflow_corners_take_the_wall_formula():
    """The Kármán channel: the NeumannX corner links load wall ghosts that the
    Bouzidi method stores; the batch turns them into Bouzidi links."""
    o = OracleSimulation(demo_cases.CASES["karman_vortex_street"][0]())
    o.initialize()
    ext = [o.scheme.nv] + list(o.domain.shape_halo)
    entries, joined = batch_entries(o.bc.methods, ext, None)
    kinds = [e["kind"] for e in entries]
    assert kinds.count("bouzidi_bounce_back") >= 2 and "neumann" in kinds
    derived = [e for e in entries if e["kind"] != "neumann" and e["links"] is not None]
    assert derived and all(o.bc.methods[e["method"]].kind == "bouzidi_bounce_back" for e in derived)
