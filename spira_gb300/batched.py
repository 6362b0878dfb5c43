"""The batched multi-RHS workload: many independent square FP64 CSR matrices,
row counts log-uniform in [100, 200 000], Poisson(12) nonzeros per row at
uniform random columns, values uniform in [-1, 1), and k right-hand sides per
matrix with k uniform in {1, 2, 4, 8, 16, 32}. Everything is generated on the
device from (seed, matrix index)."""
from __future__ import annotations

import math

import numpy as np

from . import FAM_POISSON, GEN_SYM_F64, Context, Csr, gen_draw, gen_family
from . import gen

KS = (1, 2, 4, 8, 16, 32)


def specs(n: int, seed: int, rows_lo: int = 100, rows_hi: int = 200_000):
    u = gen.unit(gen.hash3(seed, 70, np.arange(2 * n, dtype=np.uint64))).reshape(n, 2)
    rows = np.rint(np.exp(np.log(rows_lo) + u[:, 0] * (np.log(rows_hi) - np.log(rows_lo)))).astype(np.int64)
    ks = np.array([KS[min(5, int(v * 6))] for v in u[:, 1]], np.int64)
    return rows, ks


def build(ctx: Context, n: int, seed: int, rows_lo: int = 100, rows_hi: int = 200_000, lam: float = 12.0):
    """(mats, Xs, Ys, ks, nnz list). X and Y are torch CUDA float64 tensors
    (row-major n x k); Y is zero-filled."""
    import torch
    rows, ks = specs(n, seed, rows_lo, rows_hi)
    mats, Xs, Ys, nnz = [], [], [], []
    for i in range(n):
        nr = int(rows[i])
        s = seed * 1_000_003 + i
        m = gen_family(ctx, FAM_POISSON, nr, 0, lam, None, s)
        r = torch.empty(max(m, 1), dtype=torch.int32, device="cuda")
        c = torch.empty(max(m, 1), dtype=torch.int32, device="cuda")
        v = torch.empty(max(m, 1), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        gen_family(ctx, FAM_POISSON, nr, 0, lam, None, s, r, c, v)
        A = Csr(ctx, nr, nr)
        A.lock_device(r, c, v, m)
        del r, c, v
        k = int(ks[i])
        X = torch.empty(nr * k, dtype=torch.float64, device="cuda")
        gen_draw(ctx, s, 14, nr * k, GEN_SYM_F64, 0, X)
        Y = torch.zeros(nr * k, dtype=torch.float64, device="cuda")
        ctx.sync()
        mats.append(A)
        Xs.append(X)
        Ys.append(Y)
        nnz.append(A.nnz)
    return mats, Xs, Ys, [int(k) for k in ks], nnz


def bytes_per_run(mats, ks, nnz) -> int:
    """Algorithmic bytes of one pass: 12 nnz + 8 (n + 1) + 8 k (n_cols + n_rows) per matrix."""
    tot = 0
    for A, k, z in zip(mats, ks, nnz):
        n = A.n_rows
        tot += 12 * z + 8 * (n + 1) + 8 * k * (2 * n)
    return tot
