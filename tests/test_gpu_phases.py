"""pylbm's phase-by-phase routines (transport, f2m, relaxation, m2f,
equilibrium, m_halo assignment; pylbm/simulation.py:200-372) against host
arithmetic, and composed into a step against the fused one_time_step."""
import numpy as np
import pytest

from pylbm_gb300 import Simulation
from pylbm_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def planes(sim):
    return np.array([sim.m_halo[k] for k in range(sim.scheme.nv)])


def test_f2m_m2f_round_trip():
    sim = Simulation(W.cavity(n=32))
    sim.run(5)
    f0 = np.array([sim.F_halo[k] for k in range(9)])
    sim.f2m()
    sim.m2f()
    f1 = np.array([sim.F_halo[k] for k in range(9)])
    assert np.abs(f1 - f0).max() <= 1e-13 * np.abs(f0).max()
    sim.free()


def test_equilibrium_and_relaxation_against_host():
    sim = Simulation(W.cavity(n=16), parity=False)
    sc = sim.scheme
    rng = np.random.default_rng(3)
    shape = sim.domain.shape_halo
    cons = np.stack([1.0 + 0.01 * rng.standard_normal(shape), 0.02 * rng.standard_normal(shape),
                     0.02 * rng.standard_normal(shape)])
    for c in range(3):
        sim.m_halo[c] = cons[c]
    sim.equilibrium()
    got = planes(sim)
    want = sc.equilibrium_numpy(cons.reshape(3, -1)).reshape(got.shape)
    assert np.abs(got - want).max() <= 1e-14
    # perturb the non-conserved moments, then relax them
    m = want + np.concatenate([np.zeros((3,) + tuple(shape)), 1e-3 * rng.standard_normal((6,) + tuple(shape))])
    for k in range(9):
        sim.m_halo[k] = m[k]
    sim.relaxation()
    got = planes(sim)
    s = sc.rates_numpy()
    relaxed = m + s[:, None, None] * (want - m)
    assert np.array_equal(got[:3], m[:3])
    assert np.abs(got - relaxed).max() <= 1e-14
    sim.free()


@pytest.mark.parametrize("case", ["periodic", "walls"])
def test_phases_compose_to_a_step(case):
    """boundary_condition, transport, (swap), f2m, relaxation, m2f = one_time_step."""
    make = (lambda: W.tgv3d(n=16)) if case == "periodic" else (lambda: W.cavity(n=32))
    a = Simulation(make(), parity=False)
    b = Simulation(make(), parity=False)
    for sim in (a, b):
        sim.run(3)
    a.one_time_step()
    b.boundary_condition()
    b.transport()
    b._F, b._Fnew = b._Fnew, b._F  # the transported populations become F
    b.f2m()
    b.relaxation()
    b.m2f()
    fa = np.array([a.F[k] for k in range(a.scheme.nv)])
    fb = np.array([b.F[k] for k in range(b.scheme.nv)])
    assert np.abs(fa - fb).max() <= 1e-14 * np.abs(fa).max()
    a.free()
    b.free()


def test_source_term_against_oracle_half_step():
    """pylbm's standalone source_term (logistic reaction mu u (1 - u) of the
    advection-reaction demo): m_c + dt/2 S_c(m) on the interior, ghosts and
    other moments untouched, against the oracle's restatement."""
    import demo_cases
    from oracle import OracleSimulation

    d = demo_cases.advection_reaction_1d(dx=1.0 / 128)
    sim = Simulation(d)
    rng = np.random.default_rng(7)
    m = np.stack([0.5 + 0.3 * rng.standard_normal(sim.domain.shape_halo) for _ in range(sim.scheme.nv)])
    for k in range(sim.scheme.nv):
        sim.m_halo[k] = m[k]
    sim.source_term()
    got = planes(sim)
    want = OracleSimulation(d).source_term(m)
    assert not np.array_equal(want, m)
    assert np.abs(got - want).max() <= 1e-15 * np.abs(want).max()
    sim.free()
