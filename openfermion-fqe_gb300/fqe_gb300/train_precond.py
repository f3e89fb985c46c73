"""Train the learned Davidson preconditioner on correction-equation samples
from norb 10-12 sectors, select it on held-out sectors, and compare it with
the plain diagonal preconditioner.

    python -m fqe_gb300.train_precond --out DIR [--quick]

Writes DIR/precond_mlp.npz (parameters + metadata) and DIR/report.json.
Sectors use the seeded synthetic integrals (fqe_gb300.synthetic) with
2 * norb Cholesky vectors; training, validation and test seeds are disjoint.
"""

import argparse
import json
import os
import sys
import time

import numpy
import torch

from . import davidson as dav
from . import precond, synthetic
from .hamiltonians import RestrictedHamiltonian

TRAIN_SECTORS = [(10, 5, 5), (10, 5, 4), (10, 4, 4), (12, 6, 6)]
TRAIN_SEEDS = {10: range(1000, 1012), 12: range(1000, 1003)}
VAL_SEEDS = {10: range(2000, 2003), 12: range(2000, 2001)}
TEST_SEEDS = {10: range(3000, 3004), 12: range(3000, 3002)}


def _ham(norb, seed):
    h1, h2, _ = synthetic.integrals(norb, 2 * norb, seed)
    return RestrictedHamiltonian((h1, h2))


def collect(sectors, seeds, every, max_per_run, max_iter, log):
    samples = []
    for norb, na, nb in sectors:
        for seed in seeds[norb]:
            t0 = time.time()
            n0 = len(samples)
            res = dav.davidson(
                _ham(norb, seed), na, nb, block=4, max_iter=max_iter,
                callback=precond.correction_sampler(
                    samples, every=every, tol=1e-6, maxiter=200,
                    max_samples=len(samples) + max_per_run,
                    meta=dict(norb=norb, nalpha=na, nbeta=nb, seed=seed)))
            log(f"sector {(norb, na, nb)} seed {seed}: {len(samples) - n0} "
                f"samples, davidson {res.iterations} it, "
                f"{time.time() - t0:.1f} s")
    return samples


def compare(pre, sectors, seeds, log, precision=None):
    rows = []
    for norb, na, nb in sectors:
        for seed in seeds[norb]:
            ham = _ham(norb, seed)
            plain = dav.davidson(ham, na, nb, block=4, precision=precision)
            learned = dav.davidson(ham, na, nb, block=4, preconditioner=pre,
                                   precision=precision)
            row = dict(norb=norb, nalpha=na, nbeta=nb, seed=seed,
                       plain_iterations=plain.iterations,
                       plain_applies=plain.applies,
                       plain_seconds=plain.seconds,
                       learned_iterations=learned.iterations,
                       learned_applies=learned.applies,
                       learned_seconds=learned.seconds,
                       energy_difference=float(learned.eigenvalues[0]
                                               - plain.eigenvalues[0]),
                       both_converged=bool(plain.converged
                                           and learned.converged))
            rows.append(row)
            log(json.dumps(row))
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--quick", action="store_true",
                    help="norb 8-10 only, few seeds (a smoke run)")
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--lr", type=float, default=1e-3)
    args = ap.parse_args(argv)
    os.makedirs(args.out, exist_ok=True)
    logf = open(os.path.join(args.out, "train.log"), "w")

    def log(msg):
        print(msg, flush=True)
        logf.write(msg + "\n")
        logf.flush()

    train_sectors, val_sectors, test_sectors = (TRAIN_SECTORS,
                                                TRAIN_SECTORS,
                                                TRAIN_SECTORS)
    train_seeds, val_seeds, test_seeds = TRAIN_SEEDS, VAL_SEEDS, TEST_SEEDS
    if args.quick:
        train_sectors = val_sectors = test_sectors = [(8, 4, 4), (10, 5, 5)]
        train_seeds = {8: range(1000, 1004), 10: range(1000, 1002)}
        val_seeds = {8: range(2000, 2002), 10: range(2000, 2001)}
        test_seeds = {8: range(3000, 3002), 10: range(3000, 3001)}

    t0 = time.time()
    train = collect(train_sectors, train_seeds, every=3, max_per_run=8,
                    max_iter=60, log=log)
    val = collect(val_sectors, val_seeds, every=3, max_per_run=8,
                  max_iter=60, log=log)
    log(f"{len(train)} training and {len(val)} validation samples in "
        f"{time.time() - t0:.1f} s")

    pre = precond.LearnedPreconditioner(precond.init_params(0))
    plain_train = precond.mean_loss(pre, train)
    plain_val = precond.mean_loss(pre, val)
    log(f"plain preconditioner loss: train {plain_train:.6f} "
        f"validation {plain_val:.6f}")
    best = (plain_val, pre.params(), -1)
    history = []
    t1 = time.time()
    for ep in range(args.epochs):
        tr = precond.train(pre, train, epochs=1, lr=args.lr, batch=4,
                           seed=ep)[0]
        va = precond.mean_loss(pre, val)
        history.append((tr, va))
        log(f"epoch {ep}: train {tr:.6f} validation {va:.6f}")
        if va < best[0]:
            best = (va, pre.params(), ep)
    train_seconds = time.time() - t1
    pre.set_params(best[1])
    log(f"selected epoch {best[2]} (validation loss {best[0]:.6f} vs plain "
        f"{plain_val:.6f})")

    test = collect(test_sectors, test_seeds, every=3, max_per_run=8,
                   max_iter=60, log=log)
    plain_pre = precond.LearnedPreconditioner()
    test_plain = precond.mean_loss(plain_pre, test)
    test_learned = precond.mean_loss(pre, test)
    log(f"test correction-equation loss: plain {test_plain:.6f} learned "
        f"{test_learned:.6f}")
    rows = compare(pre, test_sectors, test_seeds, log)
    meta = dict(train_sectors=train_sectors,
                train_seeds={k: list(v) for k, v in train_seeds.items()},
                selected_epoch=best[2], validation_loss=best[0],
                plain_validation_loss=plain_val, epochs=args.epochs,
                lr=args.lr, samples=len(train))
    pre.save(os.path.join(args.out, "precond_mlp.npz"), **meta)
    report = dict(meta, history=history, train_seconds=train_seconds,
                  test_loss_plain=test_plain, test_loss_learned=test_learned,
                  davidson=rows,
                  device=torch.cuda.get_device_name(0))
    with open(os.path.join(args.out, "report.json"), "w") as f:
        json.dump(report, f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
