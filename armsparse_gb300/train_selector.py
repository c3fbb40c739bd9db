"""Train the learned SpMM kernel selector on this GPU and write its model file.

    python -m armsparse_gb300.train_selector [--matrices 300] [--holdout 60]
        [--out armsparse_gb300/selector_model.json] [--records PATH]

Sweeps the seeded synthetic matrices of selector.sweep_configs with the exhaustive
autotuner, trains the network on all but the last ``--holdout`` records with the project's
own GPU kernels, and prints one JSON line: the held-out picked/best time ratios of the
network and of the width-only rule, and the training summary.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import torch

from . import selector as SEL


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--matrices", type=int, default=300)
    ap.add_argument("--holdout", type=int, default=60)
    ap.add_argument("--max-nnz", type=int, default=6_000_000)
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--out", default=SEL.DEFAULT_MODEL)
    ap.add_argument("--records", default=None)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args(argv)
    t0 = time.time()
    cfgs = SEL.sweep_configs(args.matrices, seed=args.seed, max_nnz=args.max_nnz)
    recs = SEL.sweep(cfgs, reps=3, log=lambda m: print(m, file=sys.stderr, flush=True))
    t_sweep = time.time() - t0
    if args.records:
        with open(args.records, "w") as f:
            json.dump(recs, f)
    train, test = recs[: len(recs) - args.holdout], recs[len(recs) - args.holdout:]
    model = SEL.train(train, epochs=args.epochs, log=lambda m: print(m, file=sys.stderr))
    model["gpu"] = torch.cuda.get_device_name(0)
    ev_test = SEL.evaluate(model, test)
    ev_train = SEL.evaluate(model, train)
    model["heldout_eval"] = ev_test
    SEL.Selector(model).save(args.out)
    print(json.dumps({"heldout": ev_test, "train": ev_train, "sweep_s": round(t_sweep, 1),
                      "records": len(recs), "out": args.out}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
