"""The learned-closure study: compare a trained closure with the plain method on held-out seeds.

    python -m pylbm_gb300.closure_study [--model model.npz] [--eval-seeds 20] [--report out.json]

Workload: D2Q9 MRT periodic double shear layer at Re = U0 L / nu = 30 000
(U0 = 0.05 in lattice units, same Mach number on every grid).  Evaluation on
held-out seeds (100000 on): vorticity relative L2 error against the float64
1024^2 run (restricted 4x to 256^2) after 1500 coarse steps, and the device
time of each run, for plain 256^2, learned-closure 256^2, plain 512^2, plain
1024^2 (FP32) and plain 256^2 with the viscosity lowered by the best uniform
factor.  The default model is trained by pylbm_gb300.closure_train (rate
form, a-posteriori along the closure run's own trajectory).

``--apriori-train`` runs the first formulation instead: the MLP fits
one-step sub-filter-flux targets of restricted fine runs
(closure.generate_training_data / closure.train, additive form).
"""
import argparse
import json
import os
import time

import numpy as np

from . import runtime
from .closure import (ClosureModel, generate_training_data, restrict_moments, study_dicos, train, vorticity)
from .simulation import Simulation

DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
DEFAULT_MODEL = os.path.join(DATA_DIR, "closure_d2q9_shear_re30000.npz")


def _timed_run(sim, steps):
    sim.run(2)
    sim.synchronize()
    e0, e1 = runtime.Event(), runtime.Event()
    e0.record(sim._stream)
    sim.run(steps - 2)
    e1.record(sim._stream)
    return e0.elapsed_ms(e1) * steps / max(steps - 2, 1)


def _velocity_vorticity(sim, factor):
    m = np.array([sim.m[k] for k in range(3)])
    if factor > 1:
        m = restrict_moments(m, factor)
    return vorticity(m[1:], m[0])


def evaluate(model, seeds, n_coarse=256, factor=4, t_coarse=1500, re=30000.0, log=print, retune=0.8):
    """Per seed: the float64 fine reference and the four runs of the study,
    plus plain 256^2 with the viscosity multiplied by ``retune`` (the best
    uniform change of the coarse method's viscosity: it tells how much of a
    closure's gain a constant retune would give)."""
    rows = []
    for s in seeds:
        ref = Simulation(study_dicos(int(s), n_coarse * factor, re), dtype="float64", parity=False)
        ref.run(factor * t_coarse)
        w_ref = _velocity_vorticity(ref, factor)
        ref.free()
        norm = np.linalg.norm(w_ref)
        row = {"seed": int(s)}
        runs = [("plain_256", n_coarse, 1, None, re), ("learned_256", n_coarse, 1, model, re),
                ("plain_512", 2 * n_coarse, 2, None, re), ("plain_1024", n_coarse * factor, factor, None, re)]
        if retune:
            runs.append(("retuned_256", n_coarse, 1, None, re / retune))
        for name, n, f, mdl, re_run in runs:
            sim = Simulation(study_dicos(int(s), n, re_run), dtype="float32")
            if mdl is not None:
                sim.set_closure(mdl)
            ms = _timed_run(sim, f * t_coarse)
            w = _velocity_vorticity(sim, f)
            sums, bad = sim.population_sums()
            row[name] = {"vort_rel_l2": float(np.linalg.norm(w - w_ref) / norm), "ms": ms, "nonfinite": bad}
            sim.free()
        rows.append(row)
        log(json.dumps(row))
    summary = {}
    for name in [r[0] for r in runs]:
        errs = [r[name]["vort_rel_l2"] for r in rows]
        ms = [r[name]["ms"] for r in rows]
        summary[name] = {"vort_rel_l2_mean": float(np.mean(errs)), "vort_rel_l2_median": float(np.median(errs)),
                         "ms_mean": float(np.mean(ms))}
    return rows, summary


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--model", default=DEFAULT_MODEL, help="the model to evaluate")
    ap.add_argument("--eval-seeds", type=int, default=20)
    ap.add_argument("--t-coarse", type=int, default=1500)
    ap.add_argument("--report", default=None)
    ap.add_argument("--apriori-train", action="store_true",
                    help="train the first (one-step, additive) formulation and save it to --model first")
    ap.add_argument("--train-seeds", type=int, default=200)
    ap.add_argument("--steps", type=int, default=6000, help="a-priori training: Adam steps of batch 2048")
    ap.add_argument("--corrected", default="4,5",
                    help="a-priori training: non-conserved moments the closure corrects (indices among moments "
                         "3..8 of the d'Humieres basis; 4,5 = the stresses pxx-pyy and pxy; 'all' for every one)")
    ap.add_argument("--nodes-per-pair", type=int, default=4096)
    args = ap.parse_args()
    log = lambda s: print(s, flush=True)  # noqa: E731
    t0 = time.time()
    history = None
    if args.apriori_train:
        if os.path.abspath(args.model) == os.path.abspath(DEFAULT_MODEL):
            raise SystemExit("--apriori-train: give --model a new path (the default model is the trained one)")
        times = tuple(range(300, args.t_coarse + 1, 200))
        x, y = generate_training_data(range(args.train_seeds), times=times, nodes_per_pair=args.nodes_per_pair)
        log(f"training data: {x.shape[0]} samples in {time.time() - t0:.1f}s")
        corrected = None if args.corrected == "all" else [int(c) for c in args.corrected.split(",")]
        model, history = train(x, y, steps=args.steps, log=log, corrected=corrected)
        model.meta["corrected"] = corrected
        model.meta.update({"training": "a-priori", "train_seeds": args.train_seeds, "times": list(times),
                           "re": 30000.0, "n_fine": 1024, "factor": 4})
        os.makedirs(os.path.dirname(os.path.abspath(args.model)), exist_ok=True)
        model.save(args.model)
        log(f"model saved to {args.model} after {time.time() - t0:.1f}s")
    else:
        model = ClosureModel.load(args.model)
    seeds = range(100000, 100000 + args.eval_seeds)
    rows, summary = evaluate(model, seeds, t_coarse=args.t_coarse, log=log)
    report = {"summary": summary, "history": history, "rows": rows}
    log(json.dumps({"summary": summary}))
    if args.report:
        with open(args.report, "w") as fh:
            json.dump(report, fh, indent=1)


if __name__ == "__main__":
    main()
