"""Trains the learned GCG-correction network on pairs the solver itself
produces and writes its weights next to this file (data/lp_weights.f32,
raw float32 in ncgm_lp parameter order, and data/lp_weights.json).

Training pairs (r, exact d) are logged by the device HF driver
(ncgm_hf_config.lp_collect_every) from:
  * 16O, SLy4, 30^3 lattice, box 18 fm, no pairing (the plain HF ground state);
  * 24Mg, SkM*, 32^3 lattice, box 20 fm, HF+BCS with 24 states per isospin,
    at several points of the quadrupole-constrained deformation curve.
Every logged column gives 4 pairs (one per real component of the spinor).

  python -m nuclearcgm_gb300.train_lp [--steps 3000] [--batch 16]
"""
import argparse
import json
import os
import time

import numpy as np

from . import LearnedPreconditioner, abi, config, hf_run

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "data", "lp_weights.f32")

O16 = {"functional": "SLy4", "nucleus": {"A": 16, "Z": 8},
       "box": {"boxSize": 18.0, "axisMeshPoints": 30},
       "maxIterations": 40, "energyTol": 0.0}
MG24 = {"functional": "SKMstar", "nucleus": {"A": 24, "Z": 12},
        "box": {"boxSize": 20.0, "axisMeshPoints": 32},
        "pairing": {"type": "BCS", "HFbasisSize": 24, "V0": 300.0,
                    "window": 5.0},
        "maxIterations": 24, "energyTol": 0.0}


def collect(lp, every=3, mg_betas=(-0.2, 0.1, 0.4)):
    """Runs the HF loops with pair logging; returns a summary."""
    out = []
    cfg = config.from_input(O16)
    cfg.lp = lp.h.value
    cfg.lp_collect_every = every
    t = time.time()
    res, _ = hf_run(cfg)
    out.append({"run": "16O n=30", "iterations": res.iterations,
                "E": res.E_HF, "s": time.time() - t})
    for beta, mu in config.curve_points(24, mg_betas[0], mg_betas[-1],
                                        len(mg_betas)):
        cfg = config.from_input(MG24)
        cfg.curve_mode = 1
        cfg.mu20 = mu
        cfg.initial_beta = beta
        cfg.lp = lp.h.value
        cfg.lp_collect_every = every
        t = time.time()
        res, _ = hf_run(cfg)
        out.append({"run": "24Mg n=32 beta=%.2f" % beta,
                    "iterations": res.iterations, "E": res.E_HF,
                    "s": time.time() - t})
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default=WEIGHTS)
    args = ap.parse_args(argv)
    lp = LearnedPreconditioner(seed=args.seed)
    runs = collect(lp)
    sizes = {n: lp.dataset_size(n) for n in (30, 32)}
    before = {n: lp.eval(n) for n in sizes if sizes[n]}
    t = time.time()
    curve = lp.train(args.steps, args.batch, args.lr, args.seed)
    t_train = time.time() - t
    after = {n: lp.eval(n) for n in sizes if sizes[n]}
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    lp.params.astype(np.float32).tofile(args.out)
    meta = {"params": lp.P, "runs": runs, "pairs": sizes,
            "loss_before": before, "loss_after": after,
            "steps": args.steps, "batch": args.batch, "lr": args.lr,
            "train_s": t_train,
            "curve_first": float(curve[:50].mean()),
            "curve_last": float(curve[-50:].mean())}
    with open(os.path.splitext(args.out)[0] + ".json", "w") as fh:
        json.dump(meta, fh, indent=1)
    print(json.dumps(meta))
    lp.close()


if __name__ == "__main__":
    main()
