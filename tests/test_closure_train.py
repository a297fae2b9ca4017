"""The PyTorch restatement of the coarse step used by the a-posteriori
closure training (pylbm_gb300/closure_train.py) against the oracle's step."""
import numpy as np
import pytest
import torch

from oracle import OracleSimulation
from pylbm_gb300.closure import study_dicos
from pylbm_gb300.closure_train import CoarseStep, vorticity
from pylbm_gb300.closure import vorticity as np_vorticity


def _interior(o):
    h = o.h
    return o.f[:, h[0]:h[0] + o.n[0], h[1]:h[1] + o.n[1]].copy()


@pytest.mark.parametrize("seed", [0, 7])
def test_coarse_step_matches_oracle_float64(seed):
    o = OracleSimulation(study_dicos(seed, 32, re=3000.0))
    o.initialize()
    step = CoarseStep(o.scheme, dtype=torch.float64)
    f = torch.tensor(_interior(o))[None]
    for _ in range(6):
        f = step(f)
        o.one_time_step()
    ref = _interior(o)
    assert np.abs(f[0].numpy() - ref).max() <= 1e-13 * np.abs(ref).max()


def test_coarse_step_closure_adds_to_non_conserved_moments_only():
    o = OracleSimulation(study_dicos(1, 16, re=3000.0))
    o.initialize()
    step = CoarseStep(o.scheme, dtype=torch.float64)
    f = torch.tensor(_interior(o))[None]
    corr = torch.full((1, 6, 16, 16), 1e-3, dtype=torch.float64)
    a = step.moments(step(f))
    b = step.moments(step(f, lambda m, relaxed: corr))
    assert torch.allclose(a[:, :3], b[:, :3], rtol=0, atol=1e-15)
    assert torch.allclose(b[:, 3:] - a[:, 3:], corr, rtol=0, atol=1e-14)


def test_vorticity_matches_numpy():
    rng = np.random.default_rng(0)
    cons = rng.normal(size=(3, 12, 10))
    cons[0] += 3.0
    got = vorticity(torch.tensor(cons)[None])[0].numpy()
    assert np.allclose(got, np_vorticity(cons[1:], cons[0]), rtol=1e-14, atol=1e-14)


def test_rate_bounds_keep_effective_rates_below_the_maximum():
    from pylbm_gb300.closure_train import rate_bounds
    rates = np.array([1.5, 1.5, 1.2, 1.2, 1.99489, 1.99489])
    lo, hi = rate_bounds(rates, rate_max=1.9995)
    assert np.all(lo[:6] <= 0.0) and np.all(hi[:6] >= 0.0) and np.all(lo <= hi) and np.all(lo >= -1.0)
    assert np.all(rates * (1.0 + hi[:6]) <= 1.9995 + 1e-6)
    assert np.all(rates * (1.0 + lo[:6]) > 0.0)
    # the stresses (rates near 2) get the tighter lower bound; padding outputs are closed
    assert np.all(lo[4:6] == np.float32(-0.02)) and np.all(lo[:4] == np.float32(-0.3))
    assert np.all(lo[6:] == 0.0) and np.all(hi[6:] == 0.0)
    # a rate already at the maximum cannot grow
    lo2, hi2 = rate_bounds(np.array([1.9995]), rate_max=1.9995)
    assert hi2[0] <= 1e-7


def _closure_case(form, seed=3, scale=0.5):
    import mlp_oracle as mo
    from pylbm_gb300.closure_train import rate_bounds
    o = OracleSimulation(study_dicos(seed, 16, re=3000.0))
    o.initialize()
    params = mo.init_params(seed) * scale
    norm = np.zeros(48)
    norm[:9] = [1.0, 0, 0, -2.0, 1.0, 0, 0, 0, 0]
    norm[16:25] = [10.0, 20.0, 20.0, 10.0, 10.0, 20.0, 20.0, 50.0, 50.0]
    rate = None
    if form == "rate":
        lo, hi = rate_bounds(o.scheme.rates_numpy()[3:])
        rate = np.concatenate([lo, hi]).astype(np.float64)
        norm[40:46] = 1.0
    else:
        norm[40:46] = 1e-4
    return o, params, norm, rate


@pytest.mark.parametrize("form", ["additive", "rate"])
def test_closure_oracle_matches_the_training_restatement(form):
    """The oracle's fused closure step and the PyTorch restatement (float64,
    same network through the MLP oracle) agree; corrections leave rho and q."""
    import mlp_oracle as mo
    from closure_oracle import closure_step
    o, params, norm, rate = _closure_case(form)
    f0 = _interior(o)
    ref, fallbacks = closure_step(f0, o.scheme, params, norm, rate=rate)
    assert fallbacks == 0

    def closure(m, relaxed):
        b, nv, n0, n1 = m.shape
        rows = m[0].reshape(nv, -1).T.numpy()
        x = np.zeros((rows.shape[0], mo.IN))
        x[:, :nv] = (rows - norm[:nv]) * norm[16:16 + nv]
        y, _ = mo.forward(params, x)
        z = y[:, :6] * norm[40:46] + norm[32:38]
        if rate is None:
            corr = z
        else:
            lam = rate[:6] + (rate[8:14] - rate[:6]) / (1.0 + np.exp(-z))
            corr = lam * (relaxed - m)[0, 3:].reshape(6, -1).T.numpy()
        return torch.tensor(corr.T.reshape(1, 6, n0, n1))

    step = CoarseStep(o.scheme, dtype=torch.float64)
    got = step(torch.tensor(f0)[None], closure)[0].numpy()
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    plain = step(torch.tensor(f0)[None])[0].numpy()
    m_ref = np.einsum("ij,j...->i...", o.scheme.M, ref)
    m_plain = np.einsum("ij,j...->i...", o.scheme.M, plain)
    assert np.abs(m_ref[:3] - m_plain[:3]).max() < 1e-14
    assert np.abs(m_ref[3:] - m_plain[3:]).max() > 1e-8  # the network changed the step


def test_closure_oracle_guard_keeps_the_plain_collision():
    from closure_oracle import closure_step
    o, params, norm, rate = _closure_case("additive")
    f0 = _interior(o)
    plain, _ = closure_step(f0, o.scheme, np.zeros_like(params), norm)
    bad, fallbacks = closure_step(f0, o.scheme, np.full_like(params, np.nan), norm, guard=(8.0, 1e-3))
    assert fallbacks == f0[0].size
    assert np.array_equal(bad, plain)


def test_shipped_closure_model_is_a_bounded_rate_model():
    """The model in pylbm_gb300/data: rate form, every effective rate of the
    study's coarse scheme at most 1.9995, finite parameters, and the study
    record beside it holds 20 held-out seeds with the learned run better than
    the plain one on each."""
    import json
    import os
    from pylbm_gb300.closure_study import DEFAULT_MODEL
    from pylbm_gb300.scheme import Scheme
    d = np.load(DEFAULT_MODEL, allow_pickle=False)
    assert d["params"].size == 5768 and np.all(np.isfinite(d["params"]))
    assert d["norm"].size == 48 and "rate" in d.files
    rate = d["rate"]
    rates = Scheme(study_dicos(0, 256)).rates_numpy()[3:]
    assert np.all(rate[:8] <= rate[8:]) and np.all(rate[:8] >= -1.0)
    assert np.all(rates * (1.0 + rate[8:14]) <= 1.9995 + 1e-6) and np.all(rates * (1.0 + rate[:6]) > 0.0)
    study = json.load(open(os.path.join(os.path.dirname(DEFAULT_MODEL), "closure_d2q9_shear_re30000_study.json")))
    rows = study["rows"]
    assert len(rows) == 20 and all(r["seed"] >= 100000 for r in rows)
    assert all(r["learned_256"]["vort_rel_l2"] < r["plain_256"]["vort_rel_l2"] for r in rows)
    assert all(r["learned_256"]["vort_rel_l2"] < 0.02 for r in rows)
