"""Train the learned kernel selectors on this GPU and write their model files.

    python -m armsparse_gb300.train_selector [--matrices 300] [--holdout 60]
        [--out armsparse_gb300/selector_model.json] [--records PATH]
    python -m armsparse_gb300.train_selector --sddmm [--matrices 160] [--holdout 40]
        [--out armsparse_gb300/sddmm_selector_model.json]

SpMM: sweeps the seeded synthetic matrices of selector.sweep_configs with the exhaustive
autotuner, trains the network on all but the last ``--holdout`` records with the project's
own GPU kernels, and prints one JSON line: the held-out picked/best time ratios of the
network and of the width-only rule, and the training summary.

SDDMM (--sddmm): the same over selector.sddmm_sweep_configs and the SDDMM paths (CUDA-core
FP32 or one of the tcgen05 split-bf16 variants); the held-out summary compares the pick with
always taking the CUDA-core path (the reference's only kind) and with the default tensor-core
variant.
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
    ap.add_argument("--sddmm", action="store_true")
    args = ap.parse_args(argv)
    if args.sddmm:
        return _main_sddmm(args)
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


def _main_sddmm(args):
    t0 = time.time()
    n = args.matrices if args.matrices != 300 else 160
    hold = args.holdout if args.holdout != 60 else 40
    out = args.out if args.out != SEL.DEFAULT_MODEL else SEL.DEFAULT_SDDMM_MODEL
    cfgs = SEL.sddmm_sweep_configs(n, seed=args.seed, max_nnz=args.max_nnz)
    recs = SEL.sddmm_sweep(cfgs, reps=3, log=lambda m: print(m, file=sys.stderr, flush=True))
    t_sweep = time.time() - t0
    if args.records:
        with open(args.records, "w") as f:
            json.dump(recs, f)
    train, test = recs[: len(recs) - hold], recs[len(recs) - hold:]
    from . import tuner
    model = SEL.train(train, epochs=args.epochs, candidates=tuner.sddmm_paths(),
                      fmt=SEL.SDDMM_FORMAT, log=lambda m: print(m, file=sys.stderr))
    model["gpu"] = torch.cuda.get_device_name(0)
    ev_test = SEL.evaluate_sddmm(model, test)
    model["heldout_eval"] = ev_test
    SEL.SddmmSelector(model).save(out)
    print(json.dumps({"heldout": ev_test, "train": SEL.evaluate_sddmm(model, train),
                      "sweep_s": round(t_sweep, 1), "records": len(recs), "out": out}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
