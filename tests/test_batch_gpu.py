"""Batched multi-RHS SpMV (one persistent launch from a CUDA graph) against
the oracle per matrix and per right-hand side, and against the plain
one-launch-per-matrix-per-column path."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import spira_gb300 as sg
from spira_gb300 import batched
from conftest import SPMV_TOL, spmv_rel_err

pytestmark = pytest.mark.gpu


def _check(mats, Xs, Ys, ks):
    for A, X, Y, k in zip(mats, Xs, Ys, ks):
        H = A.download()
        Xh = X.cpu().numpy().reshape(A.n_cols, k)
        Yh = Y.cpu().numpy().reshape(A.n_rows, k)
        for j in range(k):
            y_ref, sc = oracle.spmv_compensated(H, Xh[:, j].copy())
            assert spmv_rel_err(Yh[:, j], y_ref, sc) <= SPMV_TOL


@pytest.mark.parametrize("config", [-1, 0, 7])
def test_batch_matches_oracle(ctx, config):
    mats, Xs, Ys, ks, nnz = batched.build(ctx, 24, seed=3, rows_lo=50, rows_hi=20_000)
    assert set(ks) <= set(batched.KS)
    B = sg.Batch(ctx, mats, Xs, Ys, ks, config=config)
    cfg, n_items = B.config()
    assert 0 <= cfg < 8 and n_items >= len(mats)
    B.run()
    ctx.sync()
    _check(mats, Xs, Ys, ks)
    for Y in Ys:
        Y.zero_()
    B.run()  # graph replays
    ctx.sync()
    _check(mats, Xs, Ys, ks)


def test_batch_plain_path_matches(ctx):
    """Both paths run one FMA chain per (row, right-hand side) in column
    order: the same bits as each other and as the oracle's fused scalar
    SpMV of every column."""
    mats, Xs, Ys, ks, nnz = batched.build(ctx, 10, seed=4, rows_lo=100, rows_hi=5_000)
    B = sg.Batch(ctx, mats, Xs, Ys, ks, config=1)
    B.run_plain()
    ctx.sync()
    _check(mats, Xs, Ys, ks)
    plain = [Y.cpu().numpy().copy() for Y in Ys]
    for Y in Ys:
        Y.zero_()
    B.run()
    ctx.sync()
    for A, X, Y, k, want in zip(mats, Xs, Ys, ks, plain):
        got = Y.cpu().numpy()
        np.testing.assert_array_equal(got, want)
        H = A.download()
        Xh = X.cpu().numpy().reshape(A.n_cols, k)
        for j in range(k):
            np.testing.assert_array_equal(got.reshape(A.n_rows, k)[:, j],
                                          oracle.spmv_scalar(H, Xh[:, j].copy(), fused=True))


def test_batch_ragged_rows_every_k(ctx):
    """Row lengths from empty to long, row counts around the 256-row sort
    windows, every k: each Y entry is written (NaN-filled before the run)
    and matches the oracle."""
    import torch
    from spira_gb300 import gen
    shapes = [(1, 1), (255, 1), (257, 2), (256, 4), (1000, 8), (513, 16), (300, 32), (4000, 1), (777, 2)]
    mats, Xs, Ys, ks = [], [], [], []
    for i, (n, k) in enumerate(shapes):
        ctr = np.arange(n, dtype=np.uint64)
        lengths = gen.below(gen.hash3(90 + i, 1, ctr), 40).astype(np.int64)
        lengths[::7] = 0
        lengths[5::97] = 3000
        rows = np.repeat(np.arange(n, dtype=np.uint32), lengths)
        c2 = np.arange(len(rows), dtype=np.uint64)
        cols = gen.below(gen.hash3(90 + i, 2, c2), n)
        vals = gen.sym_unit(gen.hash3(90 + i, 3, c2))
        A = sg.Csr(ctx, n, n)
        A.lock(rows, cols, vals)
        mats.append(A)
        Xs.append(torch.from_numpy(gen.dense_x(n * k, 95 + i)).cuda())
        Ys.append(torch.full((n * k,), float("nan"), dtype=torch.float64, device="cuda"))
        ks.append(k)
    for config in (-1, 2):
        B = sg.Batch(ctx, mats, Xs, Ys, ks, config=config)
        B.run()
        ctx.sync()
        for Y in Ys:
            assert not torch.isnan(Y).any()
        _check(mats, Xs, Ys, ks)
        for Y in Ys:
            Y.fill_(float("nan"))
        B.close()


def test_batch_rejects_bad_k(ctx):
    mats, Xs, Ys, ks, nnz = batched.build(ctx, 2, seed=5, rows_lo=100, rows_hi=200)
    with pytest.raises(sg.InvalidArgument):
        sg.Batch(ctx, mats, Xs, Ys, [3, 1])
    with pytest.raises(sg.LogicError):
        sg.Batch(ctx, [sg.Csr(ctx, 10, 10)], Xs[:1], Ys[:1], [1])
