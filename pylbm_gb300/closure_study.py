"""The learned-closure study: train on restricted fine runs, compare on held-out seeds.

    python -m pylbm_gb300.closure_study [--train-seeds 200] [--eval-seeds 20] [--out model.npz]

Workload: D2Q9 MRT periodic double shear layer at Re = U0 L / nu = 30 000
(U0 = 0.05 in lattice units, same Mach number on every grid).  Training
data: float64 runs on 1024^2 for each training seed, restricted 4x (block
averages of the populations) onto 256^2 at a set of coarse times; the MLP
learns the correction of the non-conserved post-collision moments that maps
the restricted state at coarse step n to the one at n+1.  Evaluation on
held-out seeds: vorticity relative L2 error against the float64 1024^2 run
(restricted to 256^2) at the final time, and the device time of each run,
for plain 256^2, learned-closure 256^2, plain 512^2 and plain 1024^2 (FP32).
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


def evaluate(model, seeds, n_coarse=256, factor=4, t_coarse=1500, re=30000.0, log=print):
    rows = []
    for s in seeds:
        ref = Simulation(study_dicos(int(s), n_coarse * factor, re), dtype="float64", parity=False)
        ref.run(factor * t_coarse)
        w_ref = _velocity_vorticity(ref, factor)
        ref.free()
        norm = np.linalg.norm(w_ref)
        row = {"seed": int(s)}
        runs = [("plain_256", n_coarse, 1, None), ("learned_256", n_coarse, 1, model),
                ("plain_512", 2 * n_coarse, 2, None), ("plain_1024", n_coarse * factor, factor, None)]
        for name, n, f, mdl in runs:
            sim = Simulation(study_dicos(int(s), n, re), dtype="float32")
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
    for name in ("plain_256", "learned_256", "plain_512", "plain_1024"):
        errs = [r[name]["vort_rel_l2"] for r in rows]
        ms = [r[name]["ms"] for r in rows]
        summary[name] = {"vort_rel_l2_mean": float(np.mean(errs)), "vort_rel_l2_median": float(np.median(errs)),
                         "ms_mean": float(np.mean(ms))}
    return rows, summary


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train-seeds", type=int, default=200)
    ap.add_argument("--eval-seeds", type=int, default=20)
    ap.add_argument("--steps", type=int, default=6000, help="Adam steps of batch 2048")
    ap.add_argument("--corrected", default="4,5",
                    help="non-conserved moments the closure corrects (indices among moments 3..8 of the "
                         "d'Humieres basis; 4,5 = the stresses pxx-pyy and pxy; 'all' for every one)")
    ap.add_argument("--nodes-per-pair", type=int, default=4096)
    ap.add_argument("--t-coarse", type=int, default=1500)
    ap.add_argument("--out", default=DEFAULT_MODEL)
    ap.add_argument("--report", default=None)
    ap.add_argument("--skip-train", action="store_true", help="evaluate the model at --out")
    args = ap.parse_args()
    log = lambda s: print(s, flush=True)  # noqa: E731
    t0 = time.time()
    if args.skip_train:
        model = ClosureModel.load(args.out)
        history = None
    else:
        times = tuple(range(300, args.t_coarse + 1, 200))
        x, y = generate_training_data(range(args.train_seeds), times=times, nodes_per_pair=args.nodes_per_pair)
        log(f"training data: {x.shape[0]} samples in {time.time() - t0:.1f}s")
        corrected = None if args.corrected == "all" else [int(c) for c in args.corrected.split(",")]
        model, history = train(x, y, steps=args.steps, log=log, corrected=corrected)
        model.meta["corrected"] = corrected
        model.meta.update({"train_seeds": args.train_seeds, "times": list(times), "re": 30000.0,
                           "n_fine": 1024, "factor": 4})
        os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
        model.save(args.out)
        log(f"model saved to {args.out} after {time.time() - t0:.1f}s")
    seeds = range(100000, 100000 + args.eval_seeds)
    rows, summary = evaluate(model, seeds, t_coarse=args.t_coarse, log=log)
    report = {"summary": summary, "history": history, "rows": rows}
    log(json.dumps({"summary": summary}))
    if args.report:
        with open(args.report, "w") as fh:
            json.dump(report, fh, indent=1)


if __name__ == "__main__":
    main()
