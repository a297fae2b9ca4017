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

    python -m pylbm_gb300.closure_train [--seeds 64] [--unroll 16] [--iters 1500] [--init model.npz] [--out model.npz]
"""
import argparse
import json
import math
import os
import time

import numpy as np
import sympy as sp
import torch

from . import runtime
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
        """One time step; ``closure(m_pre)`` returns corrections (batch, nv - nc, n0, n1)."""
        m = self.moments(self.pull(f))
        meq = self.equilibrium(m)
        r = self.rates.view(1, -1, 1, 1)
        relaxed = m + r * (meq - m)
        if closure is not None:
            corr = closure(m)
            relaxed = torch.cat([relaxed[:, :self.nc], relaxed[:, self.nc:] + corr], dim=1)
        return self.populations(relaxed)


class _MlpOnKernels(torch.autograd.Function):
    """y = MLP(x) on lbm_mlp_forward_tc; backward accumulates the weight
    gradient with lbm_mlp_vjp_tc into the Mlp's gradient buffer."""

    @staticmethod
    def forward(ctx, anchor, x, mlp):
        n = x.shape[0]
        y = torch.empty((n, OUT), dtype=torch.float32, device=x.device)
        mlp.forward_device(x.data_ptr(), n, y.data_ptr())
        ctx.mlp, ctx.x = mlp, x
        return y

    @staticmethod
    def backward(ctx, gy):
        gy = gy.contiguous().to(torch.float32)
        ctx.mlp.vjp_device(ctx.x.data_ptr(), gy.data_ptr(), ctx.x.shape[0])
        return torch.zeros(1, device=gy.device), None, None


class KernelClosure:
    """The closure of a ClosureModel as a differentiable map m_pre -> corrections."""

    def __init__(self, model, device):
        self.model = model
        nrm = torch.tensor(model.norm, dtype=torch.float32, device=device)
        self.mu_in, self.isig_in = nrm[0:16], nrm[16:32]
        self.mu_out, self.sig_out = nrm[32:40], nrm[40:48]
        self.anchor = torch.zeros(1, device=device, requires_grad=True)

    def inputs(self, m):
        """BF16 rows (nodes, 16) of normalised pre-collision moments, in node order."""
        b, nv, n0, n1 = m.shape
        rows = m.detach().to(torch.float32).permute(0, 2, 3, 1).reshape(-1, nv)
        x = torch.zeros((rows.shape[0], IN), dtype=torch.float32, device=m.device)
        x[:, :nv] = (rows - self.mu_in[:nv]) * self.isig_in[:nv]
        return x.to(torch.bfloat16).contiguous()

    def __call__(self, m):
        b, nv, n0, n1 = m.shape
        nn = nv - 3
        y = _MlpOnKernels.apply(self.anchor, self.inputs(m), self.model.mlp)
        corr = y[:, :nn] * self.sig_out[:nn] + self.mu_out[:nn]
        return corr.reshape(b, n0, n1, nn).permute(0, 3, 1, 2).to(m.dtype)


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


def segment_loss(step, closure, f0, targets):
    """Mean over the unrolled steps of the vorticity error (squared, relative
    to the target's norm), plus the momentum error in the same measure."""
    f = f0.to(step.dtype)
    total = 0.0
    unroll = targets.shape[1]
    for k in range(unroll):
        f = step(f, closure)
        cons = step.moments(f)[:, :3]
        ref = targets[:, k].to(step.dtype)
        w, w_ref = vorticity(cons), vorticity(ref)
        ew = ((w - w_ref) ** 2).sum(dim=(1, 2)) / (w_ref ** 2).sum(dim=(1, 2))
        eq = ((cons[:, 1:] - ref[:, 1:]) ** 2).sum(dim=(1, 2, 3)) / (ref[:, 1:] ** 2).sum(dim=(1, 2, 3))
        total = total + (ew + eq).mean()
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
    ap.add_argument("--all-outputs", action="store_true", help="correct all six non-conserved moments")
    ap.add_argument("--out", required=True)
    ap.add_argument("--eval-seeds", type=int, default=20)
    ap.add_argument("--t-coarse", type=int, default=1500)
    ap.add_argument("--report", default=None)
    args = ap.parse_args()
    log = lambda s: print(s, flush=True)  # noqa: E731
    t0 = time.time()
    times = [int(t) for t in args.times.split(",")]
    starts, targets = trajectory_data(range(args.seeds), times, args.unroll, log=log)
    vseeds = range(50000, 50000 + args.val_seeds)
    vstarts, vtargets, vfinals = trajectory_data(vseeds, times, args.unroll, final=args.t_coarse)
    log(f"data: {starts.shape[0]} segments of {args.unroll} steps in {time.time() - t0:.1f}s")
    step = CoarseStep(Scheme(study_dicos(0, starts.shape[-1])), device=starts.device)
    if args.init:
        model = ClosureModel.load(args.init)
    else:
        scales = output_scales(step, starts)
        norm = np.zeros(48, np.float32)
        with torch.no_grad():
            m = step.moments(step.pull(starts[:8]))
            mu = m.mean(dim=(0, 2, 3)).cpu().numpy()
            sd = m.std(dim=(0, 2, 3)).cpu().numpy()
        norm[:9] = mu
        norm[16:25] = np.where(sd > 0, 1.0 / np.maximum(sd, 1e-30), 0.0)
        norm[40:46] = scales
        p = init_params(0)
        p[W3_AT:B3_AT] = 0.0  # zero last layer: the closure starts as the plain step
        model = ClosureModel(p, norm, {})
    model = rescale_outputs(model, output_scales(step, starts), open_all=args.all_outputs)
    plain = plain_validation(vstarts, vtargets)
    closure = KernelClosure(model, starts.device)
    before = validation(step, closure, vstarts, vtargets)
    log(json.dumps({"val_plain": plain, "val_closure_before": before}))
    history = train_aposteriori(model, starts, targets, iters=args.iters, batch=args.batch, lr=args.lr,
                                val=(vstarts, vtargets), log=log, report_every=args.report_every,
                                rollout=lambda mdl: rollout_errors(mdl, vseeds, vfinals, args.t_coarse))
    model.meta.update({"training": "a-posteriori", "unroll": args.unroll, "seeds": args.seeds, "times": times,
                       "re": 30000.0, "n_fine": 1024, "factor": 4, "iters": args.iters})
    model.save(args.out)
    del starts, targets
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
