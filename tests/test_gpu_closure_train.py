"""A-posteriori closure training (pylbm_gb300/closure_train.py) on the GPU:
the unrolled PyTorch step with the MLP on this package's kernels reproduces
the CUDA closure step, and its gradient reduces the unrolled loss."""
import numpy as np
import pytest
import torch

from pylbm_gb300.closure import ClosureModel, init_params, study_dicos
from pylbm_gb300.closure_train import CoarseStep, KernelClosure, segment_loss, train_aposteriori
from pylbm_gb300.simulation import Simulation

pytestmark = pytest.mark.gpu


def _model(scale=0.02, seed=3):
    norm = np.zeros(48, np.float32)
    norm[:9] = [1.0, 0, 0, -2.0, 1.0, 0, 0, 0, 0]
    norm[16:25] = [10.0, 20.0, 20.0, 10.0, 10.0, 20.0, 20.0, 50.0, 50.0]
    norm[40:46] = scale * np.array([1e-3, 1e-3, 5e-4, 5e-4, 5e-4, 5e-4])
    return ClosureModel(init_params(seed), norm, {})


def _populations(sim):
    return np.array([sim.F[k] for k in range(sim.scheme.nv)])


def _rate_model(sim, seed=3):
    """A random rate-form network with the training's bounds for this scheme."""
    from pylbm_gb300.closure_train import rate_bounds
    base = _model(seed=seed)
    lo, hi = rate_bounds(sim.scheme.rates_numpy()[3:])
    norm = base.norm.copy()
    norm[40:46] = 1.0
    return ClosureModel(base.mlp.params_host(), norm, {}, rate=np.concatenate([lo, hi]))


@pytest.mark.parametrize("form,kernel", [("additive", "tc"), ("additive", "warp"), ("rate", "tc"),
                                         ("rate", "warp")])
def test_unrolled_step_matches_cuda_closure_step(form, kernel):
    """The restatement (float64 step, MLP on lbm_mlp_forward_tc) against the
    fused CUDA closure step over 12 steps, in both output forms: the
    additive corrections, and the rate form (the node relaxes moment j at
    s_j (1 + lam_j), lam_j bounded)."""
    n, steps = 64, 12
    sim = Simulation(study_dicos(5, n, re=3000.0), dtype="float32")
    model = _model() if form == "additive" else _rate_model(sim)
    # the restatement in float64: absolute FP32 populations (~0.1-0.4 each)
    # would round q about as much as the closure changes it in 12 steps
    f0 = torch.tensor(_populations(sim), dtype=torch.float64, device="cuda")[None]
    sim.set_closure(model)
    sim.closure_kernel = kernel
    sim.run(steps)
    got = np.array([sim.m[k] for k in range(3)])
    step = CoarseStep(sim.scheme, device="cuda", dtype=torch.float64)
    closure = KernelClosure(model, "cuda")
    f = f0
    with torch.no_grad():
        for _ in range(steps):
            f = step(f, closure)
    ref = step.moments(f)[0, :3].cpu().numpy()
    plain = Simulation(study_dicos(5, n, re=3000.0), dtype="float32")
    plain.run(steps)
    base = np.array([plain.m[k] for k in range(3)])
    # the closure changes the flow by far more than the two restatements differ
    diff = np.abs(got[1:] - ref[1:]).max()
    effect = np.abs(got[1:] - base[1:]).max()
    assert effect > 1e-6
    assert diff < 2e-2 * effect, (diff, effect)
    assert np.abs(got[0] - ref[0]).max() < 1e-5
    assert sim.closure_fallbacks() == 0


def test_unrolled_training_reduces_the_segment_loss():
    """Targets from the same start state stepped at a ten times smaller
    viscosity; the closure learns to move the coarse run toward them (Adam
    steps on one segment)."""
    n, unroll = 32, 6
    sim = Simulation(study_dicos(2, n, re=3000.0), dtype="float64", parity=False)
    sim.run(20)
    start = torch.tensor(_populations(sim), dtype=torch.float32, device="cuda")[None]
    fine = CoarseStep(Simulation(study_dicos(2, n, re=30000.0), dtype="float64", parity=False).scheme,
                      device="cuda", dtype=torch.float64)
    f = start.to(torch.float64)
    tg = []
    with torch.no_grad():
        for _ in range(unroll):
            f = fine(f)
            tg.append(fine.moments(f)[0, :3].to(torch.float32))
    targets = torch.stack(tg)[None]
    model = _model(scale=1.0, seed=1)
    p = model.mlp.params_host()
    p[5248:5248 + 512] = 0.0  # W3 = 0: the closure starts as the plain step
    model.mlp.set_params(p)
    coarse = CoarseStep(sim.scheme, device="cuda")
    before = float(segment_loss(coarse, KernelClosure(model, "cuda"), start, targets))
    train_aposteriori(model, start, targets, iters=60, batch=1, lr=3e-3, report_every=1000, scheme=sim.scheme)
    after = float(segment_loss(coarse, KernelClosure(model, "cuda"), start, targets))
    assert after < 0.8 * before, (before, after)


def test_training_along_own_trajectories_runs_and_moves_the_rate_model():
    """train_on_trajectories on a small case (coarse 32^2 from 64^2 float64
    runs, 48 steps, 8-step segments): every segment's loss is finite, the
    parameters move, and the rate-form model stays a valid closure."""
    from pylbm_gb300.closure_train import rate_model, reference_trajectories, train_on_trajectories
    inits, refs = reference_trajectories([3, 4], t_end=48, every=4, n_fine=64, factor=2, re=3000.0)
    assert inits.shape == (2, 9, 32, 32) and refs.shape == (2, 12, 3, 32, 32)
    scheme = Simulation(study_dicos(3, 32, re=3000.0), dtype="float32").scheme
    step = CoarseStep(scheme, device="cuda")
    model = rate_model(step, inits)
    p0 = model.mlp.params_host()
    hist = train_on_trajectories(model, inits, refs, every=4, segment=8, episodes=3, batch=2, lr=1e-3,
                                 scheme=scheme)
    assert len(hist) == 3 and all(np.isfinite(h["loss_mean"]) for h in hist)
    assert np.abs(model.mlp.params_host() - p0).max() > 0
    sim = Simulation(study_dicos(3, 32, re=3000.0), dtype="float32")
    sim.set_closure(model)
    sim.run(20)
    assert sim.closure_fallbacks() == 0 and np.all(np.isfinite(sim.m[1]))
