"""The fused closure step (lbm_one_time_step_periodic_closure).

With a zero network it must equal the plain step bit for bit; with a random
network it must equal the plain relaxation plus the MLP correction computed
by the standalone inference kernel, and it must leave mass and momentum
exactly as the plain step does.
"""
import numpy as np
import pytest
import sympy as sp

from pylbm_gb300 import Simulation
from pylbm_gb300 import workloads as W
from pylbm_gb300.closure import ClosureModel, closure_pairs, init_params, _restrict
from pylbm_gb300.scheme import Scheme

pytestmark = pytest.mark.gpu


def _norm(scale_out=1.0):
    mu_in = np.zeros(16)
    mu_in[0] = 1.0
    isig = np.zeros(16)
    isig[:9] = [200.0, 20.0, 20.0, 50.0, 50.0, 50.0, 50.0, 200.0, 200.0]
    mu_out = np.zeros(8)
    sig_out = np.zeros(8)
    sig_out[:6] = scale_out
    return np.concatenate([mu_in, isig, mu_out, sig_out])


def _moments(sim):
    return np.array([sim.m[k] for k in range(sim.scheme.nv)])


@pytest.mark.parametrize("kernel", ["tc", "warp"])
def test_zero_network_equals_plain_step(kernel):
    d = W.shear_layer(n=64, nu=1e-3)
    a = Simulation(d, dtype="float32")
    b = Simulation(d, dtype="float32")
    p = np.zeros_like(init_params(0))
    b.set_closure(ClosureModel(p, _norm()))
    b.closure_kernel = kernel
    a.run(25)
    b.run(25)
    assert np.array_equal(_moments(a), _moments(b))


def test_tensor_memory_step_equals_warp_step():
    """The tcgen05 closure step (128 nodes per block, accumulators in tensor
    memory) against the warp-level one on a random network: the same run up
    to the FP32 accumulation order inside a layer (a hidden activation may
    round to the neighbouring BF16 value), and no wait gives up."""
    import ctypes
    d = W.shear_layer(n=96, nu=1e-3, seed=6)
    runs = []
    for kernel in ("tc", "warp"):
        sim = Simulation(d, dtype="float32")
        model = ClosureModel(init_params(4), _norm(scale_out=1e-4))
        model.guard[0] = 0.0  # guard off: a random network's corrections are not judged here
        sim.set_closure(model)
        sim.closure_kernel = kernel
        sim.run(20)
        runs.append(_moments(sim))
        count = ctypes.c_uint32()
        sim.module.call(sim.module.lib.lbm_scheme_wait_timeouts(ctypes.byref(count)))
        assert count.value == 0 and sim.closure_fallbacks() == 0
        sim.free()
    tc, warp = runs
    for k in range(tc.shape[0]):
        assert np.abs(tc[k] - warp[k]).max() <= 1e-5 * max(np.abs(warp[k]).max(), 1e-3), k


def test_tensor_core_step_does_not_depend_on_blocks_per_sm():
    """Tiles are independent: the tcgen05 closure step gives the same run bit
    for bit whatever the number of blocks per SM (one block looping over
    many tiles, or many blocks sharing an SM's tensor memory), and the
    resource bound it takes by default is at least one block."""
    import ctypes
    d = W.shear_layer(n=160, nu=1e-3, seed=8)
    runs = []
    for occ in (0, 1, 3, 8):
        sim = Simulation(d, dtype="float32")
        model = ClosureModel(init_params(5), _norm(scale_out=1e-4))
        model.guard[0] = 0.0
        sim.set_closure(model)
        sim.closure_kernel = "tc"
        lib = sim.module.lib
        sim.module.call(lib.lbm_scheme_set_closure_tc_occupancy(occ))
        try:
            sim.run(15)
            runs.append(_moments(sim))
            bound, used = ctypes.c_int32(), ctypes.c_int32()
            sim.module.call(lib.lbm_scheme_closure_tc_occupancy(ctypes.byref(bound), ctypes.byref(used)))
            assert 1 <= bound.value <= 8
            assert used.value == (occ if occ else bound.value)
        finally:
            sim.module.call(lib.lbm_scheme_set_closure_tc_occupancy(0))
            sim.free()
    for r in runs[1:]:
        assert np.array_equal(r, runs[0])


def test_auto_closure_kernel_follows_grid_size():
    """auto: the warp-level step below 2^20 nodes, the tcgen05 step from there on."""
    small = Simulation(W.shear_layer(n=768, nu=1e-3), dtype="float32")
    large = Simulation(W.shear_layer(n=1024, nu=1e-3), dtype="float32")
    model = ClosureModel(init_params(1), _norm(scale_out=1e-4))
    for sim in (small, large):
        sim.set_closure(model)
        assert sim.closure_kernel == "auto"
    assert not small._closure_on_tensor_cores() and large._closure_on_tensor_cores()
    small.closure_kernel = "bogus"
    with pytest.raises(ValueError):
        small.one_time_step()
    small.free()
    large.free()


def test_closure_step_equals_relaxation_plus_network():
    d = W.shear_layer(n=48, nu=1e-3, seed=4)
    sim = Simulation(d, dtype="float32")
    sim.run(10)
    before = _restrict(sim, 1)
    model = ClosureModel(init_params(3) * 0.5, _norm(scale_out=1e-4))
    sim.set_closure(model)
    sim.one_time_step()
    after = _restrict(sim, 1)
    sc = Scheme(d)
    rates = sc.rates_numpy()
    rng = np.random.default_rng(0)
    n = before.shape[1] * before.shape[2]
    x, corr_needed = closure_pairs(sc, before, after, rates, rng, nodes=n)
    # recompute the correction the kernel should have applied
    xn = np.zeros((n, 16))
    xn[:, :9] = (x - model.norm[:9]) * model.norm[16:25]
    y = model.mlp.forward(xn)
    expected = y[:, :6] * model.norm[40:46] + model.norm[32:38]
    # closure_pairs' target is exactly the correction that was applied
    assert np.abs(corr_needed - expected).max() < 2e-5 * max(1.0, np.abs(expected).max()) + 2e-6
    # conserved moments are those of the plain step (pulled mass and momentum)
    assert np.abs(corr_needed).max() > 1e-6  # the network did something


def test_closure_conserves_mass_and_momentum():
    d = W.shear_layer(n=64, nu=1e-3, seed=2)
    sim = Simulation(d, dtype="float32")
    sim.set_closure(ClosureModel(init_params(9), _norm(scale_out=1e-3)))
    c0 = sim.conserved_sums()
    sim.run(50)
    c1 = sim.conserved_sums()
    assert abs(c1[0] - c0[0]) < 1e-6 * abs(c0[0])
    assert np.all(np.abs(c1[1:] - c0[1:]) < 1e-6 * abs(c0[0]))


@pytest.mark.parametrize("kernel", ["tc", "warp"])
@pytest.mark.parametrize("bad", ["nan", "huge"])
def test_guard_keeps_the_plain_collision_for_a_broken_network(bad, kernel):
    """A network whose outputs are not finite (NaN weights) or absurdly large
    (weights scaled by 1e6) trips the fused step's guard at every node: each
    node keeps the plain MRT collision, so the run equals the plain run bit
    for bit, and the fallbacks are counted."""
    d = W.shear_layer(n=64, nu=1e-3, seed=5)
    a = Simulation(d, dtype="float32")
    b = Simulation(d, dtype="float32")
    p = init_params(11).astype(np.float32)
    p = np.full_like(p, np.nan) if bad == "nan" else p * 1e6
    b.set_closure(ClosureModel(p, _norm(scale_out=1e-3)))
    b.closure_kernel = kernel
    a.run(12)
    b.run(12)
    assert np.array_equal(_moments(a), _moments(b))
    assert b.closure_fallbacks() == 12 * 64 * 64


@pytest.mark.parametrize("kernel", ["tc", "warp"])
def test_rate_form_bounds_a_broken_network(kernel):
    """Rate form: NaN outputs trip the guard at every node (the run equals
    the plain run bit for bit); absurdly large outputs only saturate lam_j at
    its bounds, so the corrections stay within the relaxation's own change:
    no node falls back and the run stays finite."""
    from pylbm_gb300.closure_train import rate_bounds
    d = W.shear_layer(n=64, nu=1e-3, seed=5)
    plain = Simulation(d, dtype="float32")
    plain.run(12)
    for bad in ("nan", "huge"):
        sim = Simulation(d, dtype="float32")
        lo, hi = rate_bounds(sim.scheme.rates_numpy()[3:])
        p = init_params(11).astype(np.float32)
        p = np.full_like(p, np.nan) if bad == "nan" else p * 1e6
        norm = _norm(scale_out=1.0)
        sim.set_closure(ClosureModel(p, norm, rate=np.concatenate([lo, hi])))
        sim.closure_kernel = kernel
        sim.run(12)
        if bad == "nan":
            assert np.array_equal(_moments(plain), _moments(sim))
            assert sim.closure_fallbacks() == 12 * 64 * 64
        else:
            assert sim.closure_fallbacks() == 0
            assert np.all(np.isfinite(_moments(sim)))
        sim.free()


@pytest.mark.parametrize("form", ["additive", "rate"])
@pytest.mark.parametrize("kernel", ["tc", "warp"])
def test_closure_step_against_the_oracle(form, kernel):
    """Five fused closure steps (FP32 storage and arithmetic, BF16 network,
    both output forms) against the float64 CPU oracle of the same step
    (oracle/closure_oracle.py): the two differ by far less than the closure
    changes the flow, and conserve the same mass and momentum."""
    from closure_oracle import closure_step
    from pylbm_gb300.closure_train import rate_bounds
    d = W.shear_layer(n=48, nu=1e-3, seed=4)
    sim = Simulation(d, dtype="float32")
    plain = Simulation(d, dtype="float32")
    f = np.array([sim.F[k] for k in range(sim.scheme.nv)])
    p = (init_params(3) * 0.5).astype(np.float32)
    if form == "rate":
        lo, hi = rate_bounds(sim.scheme.rates_numpy()[3:])
        model = ClosureModel(p, _norm(scale_out=1.0), rate=np.concatenate([lo, hi]))
    else:
        model = ClosureModel(p, _norm(scale_out=1e-4))
    sim.set_closure(model)
    sim.closure_kernel = kernel
    steps = 5
    sim.run(steps)
    plain.run(steps)
    total = 0
    for _ in range(steps):
        f, fb = closure_step(f, sim.scheme, model.mlp.params_host().astype(np.float64), model.norm,
                             rate=model.rate, guard=model.guard)
        total += fb
    m_ref = np.einsum("ij,j...->i...", sim.scheme.M, f)
    got = np.array([sim.m[k] for k in range(sim.scheme.nv)])
    base = np.array([plain.m[k] for k in range(sim.scheme.nv)])
    effect = np.abs(m_ref[1:3] - base[1:3]).max()
    diff = np.abs(got[1:3] - m_ref[1:3]).max()
    assert total == 0 and sim.closure_fallbacks() == 0
    assert effect > 1e-7
    # the oracle accumulates each layer in float64, the kernels in FP32 in
    # their own order: a hidden activation can round to the neighbouring BF16
    # value (up to 5e-3 of the output scale, tests/test_gpu_closure.py), so
    # node corrections differ by a few per mille; a wrong formula would differ
    # by the whole effect
    assert diff < 1e-1 * effect, (diff, effect)
    assert np.abs(got[0] - m_ref[0]).max() < 1e-6
