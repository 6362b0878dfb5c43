"""Train a variant selector on the GPU and write the model the library loads
by default (spira_gb300/spg_selector.bin for SpMV, spg_spgemm_selector.bin
for SpGEMM) plus a report.

    python -m spira_gb300.train_selector [--op spmv|spgemm] [--n 20000] [--held-out 2000] [--seed 7]

Steps: generate the corpus on the device, label every matrix with the
exhaustive autotuner, train the MLP with libspg's kernels on the first
n - held_out matrices, then report regret on the held-out ones against
exhaustive autotuning and against the fixed default variant.
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
MODELS = {"spmv": HERE / "spg_selector.bin", "spgemm": HERE / "spg_spgemm_selector.bin"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--op", default="spmv", choices=["spmv", "spgemm"])
    ap.add_argument("--n", type=int, default=20_000)
    ap.add_argument("--held-out", type=int, default=2_000)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--out", default=None)
    ap.add_argument("--report", default=None)
    ap.add_argument("--corpus-cache", default=None, help="npz to reuse / store features and timings")
    ap.add_argument("--refeature", action="store_true",
                    help="with a cached corpus: keep its timings, recompute the features of its matrices")
    args = ap.parse_args()

    import spira_gb300 as sg
    from spira_gb300 import selector as S

    ctx = sg.Context(0)
    t0 = time.time()
    if args.corpus_cache and Path(args.corpus_cache).exists():
        d = np.load(args.corpus_cache)
        X, T = d["X"], d["T"]
        if args.refeature:  # the matrices are pure functions of (seed, index): rebuild, re-measure features only
            X = S.features_of(ctx, range(len(T)), args.seed, op=args.op)
            np.savez_compressed(args.corpus_cache, X=X, T=T)
    else:
        X, T, _ = S.collect(ctx, range(args.n), args.seed, reps=args.reps, log_every=500, op=args.op)
        if args.corpus_cache:
            np.savez_compressed(args.corpus_cache, X=X, T=T)
    t_corpus = time.time() - t0
    n_train = len(X) - args.held_out
    Xtr, Ttr, Xte, Tte = X[:n_train], T[:n_train], X[n_train:], T[n_train:]
    t1 = time.time()
    blob, hist = S.train(ctx, Xtr, Ttr, epochs=args.epochs, log_every=50)
    t_train = time.time() - t1
    pred = S.predict(ctx, blob, Xte, op=args.op)
    choice = pred.argmin(axis=1)
    default = S.DEFAULT_SPMV if args.op == "spmv" else S.DEFAULT_SPGEMM
    rep = {
        "op": args.op,
        "corpus": {"n": int(len(X)), "train": int(n_train), "held_out": int(len(Xte)), "seed": args.seed,
                   "seconds": round(t_corpus, 1), "nnz_cap": S.NNZ_CAP if args.op == "spmv" else S.GEMM_NNZ_CAP},
        "train": {"epochs": args.epochs, "seconds": round(t_train, 1), "final_loss": hist[-1], "first_loss": hist[0]},
        "held_out": S.evaluate(Tte, choice, default),
        "train_fit": S.evaluate(Ttr, S.predict(ctx, blob, Xtr, op=args.op).argmin(axis=1), default),
        "variants": list((sg.SPMV_VARIANTS if args.op == "spmv" else sg.SPGEMM_VARIANTS).keys()),
        "best_variant_histogram": np.bincount(T.argmin(axis=1), minlength=T.shape[1]).tolist(),
    }
    blob.astype(np.float32).tofile(args.out or str(MODELS[args.op]))
    print(json.dumps(rep, indent=1))
    if args.report:
        Path(args.report).write_text(json.dumps(rep, indent=1))


if __name__ == "__main__":
    main()
