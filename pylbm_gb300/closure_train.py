"""A-posteriori training of the learned closure: the loss is the coarse
run's own error over several closure time steps.

A one-step target (the correction that maps one restricted fine state to the
next) only fixes what a single coarse step gets wrong, and at the shear rate
omega ~ 2 of the study the non-equilibrium moments flip sign every step, so
one-step targets are phase-sensitive.  Here the coarse D2Q9 step (periodic
pull, f -> m = M f, relaxation toward m_eq at rates s, the closure's
corrections of the non-conserved moments, f = M^-1 m) is restated with
PyTorch tensor operations, so that autograd carries the gradient of an
error accumulated over ``unroll`` coarse steps back to every step's
corrections; the MLP itself runs on this package's tensor-core kernels: the
forward pass on lbm_mlp_forward_tc, the backward pass on lbm_mlp_vjp_tc (the
vector-Jacobian product with the gradient autograd delivers for the
outputs), Adam on lbm_mlp_adam.  The network's inputs are constants of each
step: no gradient flows into the pre-collision moments through the network.

The step relaxes exactly as pylbm's MRT pull step (pylbm/algorithm/pull.py,
relaxation pylbm/algorithm/base.py:404-428) and the fused closure step of
the CUDA modules (k_step_periodic_closure): inputs are the normalised
pre-collision moments rounded to BF16, corrections are added after the
relaxation, rho and q are never changed.  The trained model is evaluated
with the CUDA closure step (closure_study.evaluate), not with this restatement.

Two ways to choose the unrolled segments:

* ``--mode trajectory`` (default): truncated backpropagation along the
  closure run's own trajectory.  Each episode advances a batch of coarse runs
  from their own initial states over the whole window; every ``--unroll``
  steps the error against the restricted fine moments is back-propagated
  through that segment and Adam steps.  The segments start from the states
  the closure meets when it runs.
* ``--mode segments``: unrolls started from restricted fine states.  Their
  short-horizon loss falls while the whole run gets worse: the network
  learns to undo the start-up transient of a restricted fine state, which a
  coarse run never has.

Two output forms (``--form``): ``additive`` (the correction is the scaled
output) and ``rate`` (the output sets lam_j in bounds and the node relaxes
moment j at s_j (1 + lam_j); with every effective rate below 2 the
collision cannot turn unstable, which the additive form did when its
corrections pushed the stress relaxation past 2).  Every report validates
the model over whole runs with the CUDA closure step and the best
parameters are kept.

    python -m pylbm_gb300.closure_train --out model.npz [--mode trajectory] [--form rate] [--seeds 24]
"""
import argparse
import ctypes
import json
import math
import time

import numpy as np
import sympy as sp
import torch

from .closure import IN, OUT, ClosureModel, _restrict, init_params, study_dicos
from .scheme import Scheme


class CoarseStep:
    """The periodic D2Q9 MRT step of a scheme as differentiable tensor operations.

    Populations are (batch, nv, n0, n1) absolute values; ``dtype`` float32
    (training) or float64 (checks against the oracle).
    """

    def __init__(self, scheme, device="cpu", dtype=torch.float32):
        if scheme.dim != 2 or scheme.Tu is not None or scheme.source_terms:
            raise ValueError("CoarseStep restates the plain 2D MRT step")
        self.scheme = scheme
        self.nv, self.nc = scheme.nv, scheme.nconsm
        self.device, self.dtype = device, dtype
        self.M = torch.tensor(np.asarray(scheme.M, dtype=np.float64), dtype=dtype, device=device)
        self.invM = torch.tensor(np.asarray(scheme.invM, dtype=np.float64), dtype=dtype, device=device)
        self.rates = torch.tensor(scheme.rates_numpy(), dtype=dtype, device=device)
        self.vel = [tuple(int(c) for c in v) for v in scheme.stencil.get_all_velocities()]
        syms = list(scheme.consm.keys())
        self._eq = [sp.lambdify(syms, e, "math") if e.free_symbols else float(e) for e in scheme.EQ]

    def pull(self, f):
        return torch.stack([torch.roll(f[:, k], shifts=self.vel[k], dims=(1, 2)) for k in range(self.nv)], dim=1)

    def moments(self, f):
        return torch.einsum("ij,bjxy->bixy", self.M, f)

    def populations(self, m):
        return torch.einsum("ij,bjxy->bixy", self.invM, m)

    def equilibrium(self, m):
        cons = [m[:, i] for i in range(self.nc)]
        out = []
        for e in self._eq:
            out.append(torch.full_like(cons[0], e) if isinstance(e, float) else e(*cons) + torch.zeros_like(cons[0]))
        return torch.stack(out, dim=1)

    def __call__(self, f, closure=None):
        """One time step; ``closure(m_pre, m_relaxed)`` returns corrections
        (batch, nv - nc, n0, n1) of the non-conserved moments."""
        m = self.moments(self.pull(f))
        meq = self.equilibrium(m)
        r = self.rates.view(1, -1, 1, 1)
        relaxed = m + r * (meq - m)
        if closure is not None:
            corr = closure(m, relaxed)
            relaxed = torch.cat([relaxed[:, :self.nc], relaxed[:, self.nc:] + corr], dim=1)
        return self.populations(relaxed)


def _torch_stream(device):
    """PyTorch's current stream on ``device`` as a raw handle for the C ABI, so
    the kernels are ordered with the tensor operations around them."""
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class _MlpOnKernels(torch.autograd.Function):
    """y = MLP(x) on lbm_mlp_forward_tc; backward accumulates the weight
    gradient with lbm_mlp_vjp_tc into the Mlp's gradient buffer (both on
    PyTorch's current stream)."""

    @staticmethod
    def forward(ctx, anchor, x, mlp):
        n = x.shape[0]
        y = torch.empty((n, OUT), dtype=torch.float32, device=x.device)
        mlp.forward_device(x.data_ptr(), n, y.data_ptr(), stream=_torch_stream(x.device))
        ctx.mlp, ctx.x = mlp, x
        return y

    @staticmethod
    def backward(ctx, gy):
        gy = gy.contiguous().to(torch.float32)
        ctx.mlp.vjp_device(ctx.x.data_ptr(), gy.data_ptr(), ctx.x.shape[0], stream=_torch_stream(gy.device))
        return torch.zeros(1, device=gy.device), None, None


class KernelClosure:
    """The closure of a ClosureModel as a differentiable map (m_pre, m_relaxed)
    -> corrections, in the additive or the rate form of the fused step."""

    def __init__(self, model, device):
        self.model = model
        nrm = torch.tensor(model.norm, dtype=torch.float32, device=device)
        self.mu_in, self.isig_in = nrm[0:16], nrm[16:32]
        self.mu_out, self.sig_out = nrm[32:40], nrm[40:48]
        self.rate = None if model.rate is None else torch.tensor(model.rate, dtype=torch.float32, device=device)
        self.anchor = torch.zeros(1, device=device, requires_grad=True)

    def inputs(self, m):
        """BF16 rows (nodes, 16) of normalised pre-collision moments, in node order."""
        b, nv, n0, n1 = m.shape
        rows = m.detach().to(torch.float32).permute(0, 2, 3, 1).reshape(-1, nv)
        x = torch.zeros((rows.shape[0], IN), dtype=torch.float32, device=m.device)
        x[:, :nv] = (rows - self.mu_in[:nv]) * self.isig_in[:nv]
        return x.to(torch.bfloat16).contiguous()

    def __call__(self, m, relaxed):
        b, nv, n0, n1 = m.shape
        nn = nv - 3
        y = _MlpOnKernels.apply(self.anchor, self.inputs(m), self.model.mlp)
        z = (y[:, :nn] * self.sig_out[:nn] + self.mu_out[:nn]).reshape(b, n0, n1, nn).permute(0, 3, 1, 2)
        if self.rate is None:
            return z.to(m.dtype)
        lo, hi = self.rate[:nn].view(1, -1, 1, 1), self.rate[8:8 + nn].view(1, -1, 1, 1)
        lam = lo + (hi - lo) * torch.sigmoid(z)
        return lam.to(m.dtype) * (relaxed[:, 3:] - m[:, 3:])


def vorticity(cons):
    """z-vorticity (batch, n0, n1) of u = q / rho, central differences, periodic."""
    ux, uy = cons[:, 1] / cons[:, 0], cons[:, 2] / cons[:, 0]
    duy_dx = (torch.roll(uy, -1, 1) - torch.roll(uy, 1, 1)) / 2
    dux_dy = (torch.roll(ux, -1, 2) - torch.roll(ux, 1, 2)) / 2
    return duy_dx - dux_dy


# ---------------------------------------------------------------------------
# trajectories of restricted fine runs
# ---------------------------------------------------------------------------
def trajectory_data(seeds, times, unroll, n_fine=1024, factor=4, re=30000.0, device="cuda", log=None, final=None):
    """Start states and targets of the unrolled segments.

    For every seed a float64 run on n_fine^2 nodes; at each coarse time t0 of
    ``times`` the populations restricted ``factor`` times (block averages,
    lbm_restrict) start a segment, and the restricted conserved moments after
    each of the next ``unroll`` coarse steps (``factor`` fine steps each) are
    its targets.  Returns (start (S, 9, n, n), targets (S, unroll, 3, n, n))
    as float32 tensors on ``device``; with ``final`` (a coarse time after the
    last segment) also the restricted conserved moments of every seed at
    that time (a list of float64 arrays (3, n, n)).
    """
    from .simulation import Simulation

    starts, targets, finals = [], [], []
    t0 = time.time()
    for s in seeds:
        sim = Simulation(study_dicos(int(s), n_fine, re), dtype="float64", parity=False)
        M3 = np.asarray(sim.scheme.M, dtype=np.float64)[:3]
        step = 0
        for tc in times:
            sim.run(factor * tc - step)
            step = factor * tc
            start = _restrict(sim, factor)
            tg = []
            for _ in range(unroll):
                sim.run(factor)
                step += factor
                r = _restrict(sim, factor)
                tg.append(np.einsum("ij,j...->i...", M3, r))
            starts.append(torch.tensor(start, dtype=torch.float32).to(device))
            targets.append(torch.tensor(np.array(tg), dtype=torch.float32).to(device))
        if final is not None:
            sim.run(factor * final - step)
            finals.append(np.einsum("ij,j...->i...", M3, _restrict(sim, factor)))
        sim.free()
        if log:
            log(f"seed {s}: {len(times)} segments, {time.time() - t0:.1f}s")
    if final is not None:
        return torch.stack(starts), torch.stack(targets), finals
    return torch.stack(starts), torch.stack(targets)


def rollout_errors(model, seeds, finals, t_coarse, n=256, re=30000.0):
    """Vorticity relative L2 error of the closure run (this package's CUDA
    closure step, FP32) after ``t_coarse`` steps from each seed's own
    initial state, against the restricted fine moments ``finals``; inf for a
    run that produced non-finite values."""
    from .closure import vorticity as np_vorticity
    from .simulation import Simulation

    errs = []
    for s, ref in zip(seeds, finals):
        sim = Simulation(study_dicos(int(s), n, re), dtype="float32")
        sim.set_closure(model)
        sim.run(t_coarse)
        m = np.array([sim.m[k] for k in range(3)])
        _, bad = sim.population_sums()
        sim.free()
        w, w_ref = np_vorticity(m[1:], m[0]), np_vorticity(ref[1:], ref[0])
        e = float(np.linalg.norm(w - w_ref) / np.linalg.norm(w_ref))
        errs.append(e if bad == 0 and np.isfinite(e) else float("inf"))
    return errs


def reference_trajectories(seeds, t_end, every, n_fine=1024, factor=4, re=30000.0, device="cuda", log=None):
    """The coarse runs' own initial populations and the restricted fine
    conserved moments every ``every`` coarse steps up to ``t_end``.

    Returns (inits (S, 9, n, n), refs (S, t_end // every, 3, n, n)) as
    float32 tensors on ``device``; refs[:, i] belongs to coarse step
    (i + 1) * every.
    """
    from .simulation import Simulation

    seeds = list(seeds)
    t0 = time.time()
    n = n_fine // factor
    snaps = t_end // every
    inits = None
    # filled in place: the snapshots of 200 seeds take about 59 GB
    refs = torch.empty((len(seeds), snaps, 3, n, n), dtype=torch.float32, device=device)
    for i, s in enumerate(seeds):
        coarse = Simulation(study_dicos(int(s), n, re), dtype="float32")
        f0 = torch.tensor(np.array([coarse.F[k] for k in range(coarse.scheme.nv)]), dtype=torch.float32)
        coarse.free()
        if inits is None:
            inits = torch.empty((len(seeds),) + tuple(f0.shape), dtype=torch.float32, device=device)
        inits[i] = f0.to(device)
        sim = Simulation(study_dicos(int(s), n_fine, re), dtype="float64", parity=False)
        M3 = np.asarray(sim.scheme.M, dtype=np.float64)[:3]
        for j in range(snaps):
            sim.run(factor * every)
            refs[i, j] = torch.from_numpy(np.einsum("ij,j...->i...", M3, _restrict(sim, factor))).to(device)
        sim.free()
        if log:
            log(f"seed {s}: {snaps} reference snapshots, {time.time() - t0:.1f}s")
    return inits, refs


def _snapshot_error(step, f, ref):
    """Relative squared vorticity error plus relative squared momentum error
    of the populations ``f`` against the conserved moments ``ref``, batch mean."""
    cons = step.moments(f)[:, :3]
    ref = ref.to(step.dtype)
    w, w_ref = vorticity(cons), vorticity(ref)
    ew = ((w - w_ref) ** 2).sum(dim=(1, 2)) / (w_ref ** 2).sum(dim=(1, 2))
    eq = ((cons[:, 1:] - ref[:, 1:]) ** 2).sum(dim=(1, 2, 3)) / (ref[:, 1:] ** 2).sum(dim=(1, 2, 3))
    return (ew + eq).mean()


def train_on_trajectories(model, inits, refs, every, segment=16, episodes=8, batch=4, lr=1e-3, clip=1.0,
                          log=None, seed=0, rollout=None, scheme=None):
    """Truncated backpropagation along the closure run's own trajectory.

    Each episode starts ``batch`` coarse runs from their own initial states
    and advances them with the closure over the whole reference window; every
    ``segment`` steps the error against the restricted fine moments at the
    snapshots inside the segment is back-propagated through that segment's
    steps only (the state entering it is a constant) and Adam takes a step.
    The start states are thus always states of the closure run itself, the
    ones the trained closure meets when it runs.  ``rollout``: as in
    train_aposteriori (validation over whole runs, best parameters kept).
    """
    if segment % every:
        raise ValueError("segment must be a multiple of the snapshot spacing")
    device = inits.device
    step = CoarseStep(scheme or Scheme(study_dicos(0, inits.shape[-1])), device=device)
    closure = KernelClosure(model, device)
    mlp = model.mlp
    saved_stream, mlp.stream = mlp.stream, _torch_stream(device)  # Adam and copies ordered with the tensors
    gen = torch.Generator(device="cpu").manual_seed(seed)
    t_end = refs.shape[1] * every
    nseg = t_end // segment
    total = episodes * nseg
    history, best, it = [], (float("inf"), None), 0
    if rollout is not None:
        errs = rollout(model)
        best = (float(np.mean(errs)), mlp.params_host())
        history.append({"episode": 0, "rollout": errs})
        if log:
            log(json.dumps(history[-1]))
    mlp.g.zero(mlp.stream)
    for ep in range(episodes):
        idx = torch.randperm(inits.shape[0], generator=gen)[:batch].to(device)
        f = inits[idx].clone()
        losses = []
        for sgi in range(nseg):
            f = f.detach()
            loss = 0.0
            for k in range(segment):
                f = step(f, closure)
                t = sgi * segment + k + 1
                if t % every == 0:
                    loss = loss + _snapshot_error(step, f, refs[idx, t // every - 1])
            loss.backward()
            torch.cuda.synchronize()
            g = mlp.grad_host()
            gn = float(np.linalg.norm(g))
            if math.isfinite(gn):
                if gn > clip:
                    mlp.set_grad(g * (clip / gn))
                mlp.adam_step(lr * 0.5 * (1.0 + math.cos(math.pi * it / total)))
            else:
                mlp.g.zero(mlp.stream)
            it += 1
            losses.append(float(loss.detach()))
        rec = {"episode": ep + 1, "loss_first": losses[0], "loss_last": losses[-1], "loss_mean": float(np.mean(losses))}
        if rollout is not None:
            torch.cuda.synchronize()  # the last Adam step landed before the runs read the weights
            errs = rollout(model)
            rec["rollout"] = errs
            if float(np.mean(errs)) < best[0]:
                best = (float(np.mean(errs)), mlp.params_host())
        history.append(rec)
        if log:
            log(json.dumps(rec))
    if best[1] is not None:
        mlp.set_params(best[1])
        history.append({"kept_rollout_mean": best[0]})
    mlp.stream = saved_stream
    return history


def segment_loss(step, closure, f0, targets):
    """Mean over the unrolled steps of the vorticity error (squared, relative
    to the target's norm), plus the momentum error in the same measure."""
    f = f0.to(step.dtype)
    total = 0.0
    unroll = targets.shape[1]
    for k in range(unroll):
        f = step(f, closure)
        total = total + _snapshot_error(step, f, targets[:, k])
    return total / unroll


def output_scales(step, starts, frac=0.1):
    """A correction scale per non-conserved moment: ``frac`` of the standard
    deviation of the relaxation's own change s_k (m_eq,k - m_k) on the start states."""
    with torch.no_grad():
        m = step.moments(step.pull(starts[: min(8, starts.shape[0])].to(step.dtype)))
        change = step.rates.view(1, -1, 1, 1) * (step.equilibrium(m) - m)
        return (frac * change[:, step.nc:].std(dim=(0, 2, 3))).cpu().numpy()


def train_aposteriori(model, starts, targets, iters=1500, batch=4, lr=3e-4, clip=1.0, val=None, log=None,
                      report_every=100, seed=0, scheme=None, rollout=None):
    """Adam on the unrolled loss; returns the history.  ``val`` = (starts,
    targets) held out; ``scheme``: the coarse scheme (default: the study's
    shear layer on the segments' grid).  ``rollout``: a function of the
    model giving its validation error over a whole run; with it, every
    report keeps the parameters of the lowest mean error so far, and they
    are the model's parameters at the end."""
    device = starts.device
    step = CoarseStep(scheme or Scheme(study_dicos(0, starts.shape[-1])), device=device)
    closure = KernelClosure(model, device)
    mlp = model.mlp
    saved_stream, mlp.stream = mlp.stream, _torch_stream(device)  # Adam and copies ordered with the tensors
    gen = torch.Generator(device="cpu").manual_seed(seed)
    history = []
    mlp.g.zero(mlp.stream)
    acc = []
    best = (float("inf"), None)
    if rollout is not None:
        errs = rollout(model)
        best = (float(np.mean(errs)), mlp.params_host())
        history.append({"iter": 0, "rollout": errs})
        if log:
            log(json.dumps(history[-1]))
    for it in range(iters):
        idx = torch.randint(0, starts.shape[0], (batch,), generator=gen).to(device)
        loss = segment_loss(step, closure, starts[idx], targets[idx])
        loss.backward()
        torch.cuda.synchronize()
        g = mlp.grad_host()
        gn = float(np.linalg.norm(g))
        if not math.isfinite(gn):
            mlp.g.zero(mlp.stream)
            continue
        if gn > clip:
            mlp.set_grad(g * (clip / gn))
        lr_s = lr * 0.5 * (1.0 + math.cos(math.pi * it / iters))
        mlp.adam_step(lr_s)
        acc.append(float(loss.detach()))
        if (it + 1) % report_every == 0 or it + 1 == iters:
            rec = {"iter": it + 1, "train": float(np.mean(acc)), "grad_norm": gn}
            if val is not None:
                rec["val"] = validation(step, closure, *val)
            if rollout is not None:
                torch.cuda.synchronize()  # the last Adam step landed before the runs read the weights
                errs = rollout(model)
                rec["rollout"] = errs
                if float(np.mean(errs)) < best[0]:
                    best = (float(np.mean(errs)), mlp.params_host())
            acc = []
            history.append(rec)
            if log:
                log(json.dumps(rec))
    if best[1] is not None:
        mlp.set_params(best[1])
        history.append({"kept_rollout_mean": best[0]})
    mlp.stream = saved_stream
    return history


def validation(step, closure, starts, targets, batch=8):
    with torch.no_grad():
        vals = [float(segment_loss(step, closure, starts[i:i + batch], targets[i:i + batch])) * min(batch, starts.shape[0] - i)
                for i in range(0, starts.shape[0], batch)]
    return sum(vals) / starts.shape[0]


def plain_validation(starts, targets, batch=8):
    step = CoarseStep(Scheme(study_dicos(0, starts.shape[-1])), device=starts.device)
    return validation(step, None, starts, targets, batch)


W3_AT, B3_AT = 16 * 64 + 64 + 64 * 64 + 64, 16 * 64 + 64 + 64 * 64 + 64 + 8 * 64


def rescale_outputs(model, scales, open_all=False):
    """The model with output scales ``scales`` (one per non-conserved moment).

    The corrections stay what they were: an output whose scale changes has
    its row of W3 and its b3 entry multiplied by old / new scale.  Outputs
    with scale zero (moments the model does not correct) stay closed unless
    ``open_all``: they then get their new scale and a zero row (no
    correction until training moves them).
    """
    norm = model.norm.copy()
    p = model.mlp.params_host()
    for j, new in enumerate(scales):
        old = float(norm[40 + j])
        row = slice(W3_AT + j * 64, W3_AT + (j + 1) * 64)
        if old > 0.0:
            p[row] *= old / new
            p[B3_AT + j] *= old / new
        elif open_all:
            p[row] = 0.0
            p[B3_AT + j] = 0.0
            norm[32 + j] = 0.0
        else:
            continue
        norm[40 + j] = new
    out = ClosureModel(p, norm, dict(model.meta))
    out.guard[1] = 8.0 * float(np.max(norm[40:48]))
    return out


def _input_norm(step, starts):
    norm = np.zeros(48, np.float32)
    with torch.no_grad():
        m = step.moments(step.pull(starts[:8]))
        mu = m.mean(dim=(0, 2, 3)).cpu().numpy()
        sd = m.std(dim=(0, 2, 3)).cpu().numpy()
    nv = mu.size
    norm[:nv] = mu
    norm[16:16 + nv] = np.where(sd > 0, 1.0 / np.maximum(sd, 1e-30), 0.0)
    return norm


def additive_model(step, starts):
    """A fresh additive-form network whose corrections start at zero."""
    norm = _input_norm(step, starts)
    norm[40:40 + step.nv - step.nc] = output_scales(step, starts)
    p = init_params(0)
    p[W3_AT:B3_AT] = 0.0  # zero last layer: the closure starts as the plain step
    return ClosureModel(p, norm, {"form": "additive"})


def rate_bounds(rates, rate_max=1.9995, lam_lo=-0.3, lam_lo_stress=-0.02, lam_hi=0.3):
    """(lo[8], hi[8]) of lam per non-conserved moment: the effective rate
    s (1 + lam) stays at most ``rate_max``; moments relaxed near 2 (above
    1.9: the stresses at low viscosity) get the tighter lower bound."""
    lo = np.zeros(8, np.float32)
    hi = np.zeros(8, np.float32)
    for j, sj in enumerate(rates):
        if sj <= 0.0:
            continue
        lo[j] = lam_lo_stress if sj > 1.9 else lam_lo
        hi[j] = min(lam_hi, rate_max / sj - 1.0)
        if hi[j] <= lo[j]:
            hi[j] = lo[j] = 0.0
    return lo, hi


def rate_model(step, starts, rate_max=1.9995, lam_lo=-0.3, lam_lo_stress=-0.02, lam_hi=0.3):
    """A fresh rate-form network: zero last layer and mu_out at the logit
    where lam = 0, so it starts as the plain step."""
    norm = _input_norm(step, starts)
    rates = step.rates[step.nc:].cpu().numpy()
    lo, hi = rate_bounds(rates, rate_max, lam_lo, lam_lo_stress, lam_hi)
    for j in range(rates.size):
        if hi[j] > lo[j]:
            frac = -lo[j] / (hi[j] - lo[j])
            norm[32 + j] = float(np.log(frac / (1.0 - frac)))
            norm[40 + j] = 1.0
    p = init_params(0)
    p[W3_AT:B3_AT] = 0.0
    model = ClosureModel(p, norm, {"form": "rate", "rate_max": rate_max}, rate=np.concatenate([lo, hi]))
    return model


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--seeds", type=int, default=48, help="training seeds (fine float64 runs)")
    ap.add_argument("--val-seeds", type=int, default=4)
    ap.add_argument("--times", default="100,300,500,700,900,1100,1300")
    ap.add_argument("--unroll", type=int, default=16)
    ap.add_argument("--iters", type=int, default=1500)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--report-every", type=int, default=100)
    ap.add_argument("--init", default=None, help="start from this model (else a fresh network)")
    ap.add_argument("--all-outputs", action="store_true", help="additive form: correct all six non-conserved moments")
    ap.add_argument("--form", default="rate", choices=["rate", "additive"])
    ap.add_argument("--rate-max", type=float, default=1.9995, help="rate form: largest effective rate")
    ap.add_argument("--lam-lo", type=float, default=-0.3, help="rate form: lower bound of lam")
    ap.add_argument("--lam-lo-stress", type=float, default=-0.02,
                    help="rate form: lower bound of lam for moments relaxed near 2 (the stresses)")
    ap.add_argument("--lam-hi", type=float, default=0.3, help="rate form: upper bound of lam (before --rate-max)")
    ap.add_argument("--out", required=True)
    ap.add_argument("--eval-seeds", type=int, default=20)
    ap.add_argument("--t-coarse", type=int, default=1500)
    ap.add_argument("--report", default=None)
    ap.add_argument("--mode", default="trajectory", choices=["trajectory", "segments"],
                    help="trajectory: truncated backpropagation along the closure run's own trajectory; "
                         "segments: unrolls started from restricted fine states")
    ap.add_argument("--episodes", type=int, default=8)
    ap.add_argument("--every", type=int, default=4, help="trajectory mode: coarse steps between reference snapshots")
    args = ap.parse_args()
    log = lambda s: print(s, flush=True)  # noqa: E731
    t0 = time.time()
    times = [int(t) for t in args.times.split(",")]
    vseeds = range(50000, 50000 + args.val_seeds)
    vstarts, vtargets, vfinals = trajectory_data(vseeds, times, args.unroll, final=args.t_coarse)
    if args.mode == "segments":
        starts, targets = trajectory_data(range(args.seeds), times, args.unroll, log=log)
        log(f"data: {starts.shape[0]} segments of {args.unroll} steps in {time.time() - t0:.1f}s")
    else:
        inits, refs = reference_trajectories(range(args.seeds), args.t_coarse, args.every, log=log)
        starts = vstarts  # normalisation statistics
        log(f"data: {inits.shape[0]} trajectories of {args.t_coarse} steps in {time.time() - t0:.1f}s")
    step = CoarseStep(Scheme(study_dicos(0, starts.shape[-1])), device=starts.device)
    if args.init:
        model = ClosureModel.load(args.init)
        if (model.rate is not None) != (args.form == "rate"):
            raise SystemExit(f"--init holds a model of the other form than --form {args.form}")
        if args.form == "additive":
            model = rescale_outputs(model, output_scales(step, starts), open_all=args.all_outputs)
    elif args.form == "rate":
        model = rate_model(step, starts, args.rate_max, args.lam_lo, args.lam_lo_stress, args.lam_hi)
    else:
        model = additive_model(step, starts)
    plain = plain_validation(vstarts, vtargets)
    closure = KernelClosure(model, starts.device)
    before = validation(step, closure, vstarts, vtargets)
    log(json.dumps({"val_plain": plain, "val_closure_before": before}))
    rollout = lambda mdl: rollout_errors(mdl, vseeds, vfinals, args.t_coarse)  # noqa: E731
    if args.mode == "segments":
        history = train_aposteriori(model, starts, targets, iters=args.iters, batch=args.batch, lr=args.lr,
                                    val=(vstarts, vtargets), log=log, report_every=args.report_every,
                                    rollout=rollout)
    else:
        history = train_on_trajectories(model, inits, refs, args.every, segment=args.unroll,
                                        episodes=args.episodes, batch=args.batch, lr=args.lr, log=log,
                                        rollout=rollout)
    model.meta.update({"training": "a-posteriori, " + args.mode, "unroll": args.unroll, "seeds": args.seeds,
                       "re": 30000.0, "n_fine": 1024, "factor": 4, "lr": args.lr,
                       **({"times": times, "iters": args.iters} if args.mode == "segments" else
                          {"episodes": args.episodes, "every": args.every, "t_coarse": args.t_coarse})})
    model.save(args.out)
    del starts
    torch.cuda.empty_cache()
    log(f"model saved to {args.out} after {time.time() - t0:.1f}s")
    rows, summary = [], {}
    if args.eval_seeds > 0:
        from .closure_study import evaluate
        rows, summary = evaluate(model, range(100000, 100000 + args.eval_seeds), t_coarse=args.t_coarse, log=log)
    report = {"summary": summary, "history": history, "val_plain": plain, "val_closure_before": before,
              "rows": rows}
    log(json.dumps({"summary": summary}))
    if args.report:
        with open(args.report, "w") as fh:
            json.dump(report, fh, indent=1)


if __name__ == "__main__":
    main()
