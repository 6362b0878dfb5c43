"""Seeded synthetic matrices for the benchmark and the parity tests.

Every random draw is a pure function of (seed, stream, counter) through the
splitmix64 finaliser, so the same inputs come out on x86-64 and aarch64 and
in any order of generation. Values uniform in [-1, 1) are
2 * ((h >> 11) * 2**-53) - 1, exact in binary64. Generators return staged
inserts (rows, cols, vals) in insertion order, the way a Spira user feeds
matrix::insert before lock().

Workloads (no public dataset is involved; all are synthetic by construction):
  random_rows      n x n, `per_row` distinct uniform columns per row
  laplacian_2d     5-point stencil on a g x g grid (4 on the diagonal, -1)
  laplacian_3d     7-point stencil on a g^3 grid (6 on the diagonal, -1)
  zipf_rows        n x n, row lengths Zipf(alpha) truncated to [1, cap] and
                   scaled to a target mean by L = min(cap, max(1, round(Z*s)))
  uniform_rows     n x n, `per_row` uniform (possibly repeated) columns
  relock_batch     1% of nnz new entries spread over a random 10% of rows
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x: np.ndarray) -> np.ndarray:
    x = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def hash3(seed: int, stream: int, counter: np.ndarray) -> np.ndarray:
    """Independent 64-bit draws for (seed, stream, counter)."""
    with np.errstate(over="ignore"):
        k = splitmix64(np.uint64(seed) * np.uint64(0xD1B54A32D192ED03) + np.uint64(stream))
        return splitmix64(np.asarray(counter, dtype=np.uint64) ^ k)


def unit(h: np.ndarray) -> np.ndarray:
    """[0, 1) doubles from 64-bit draws."""
    return (h >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def sym_unit(h: np.ndarray) -> np.ndarray:
    """[-1, 1) doubles."""
    return 2.0 * unit(h) - 1.0


def below(h: np.ndarray, n: int) -> np.ndarray:
    """Integers in [0, n) (n < 2**32) by multiply-shift of the high word."""
    return (((h >> np.uint64(32)) * np.uint64(n)) >> np.uint64(32)).astype(np.uint32)


def random_rows(n_rows: int, n_cols: int, per_row: int, seed: int):
    """`per_row` distinct uniform columns per row (duplicates redrawn)."""
    r = np.repeat(np.arange(n_rows, dtype=np.uint64), per_row)
    k = np.tile(np.arange(per_row, dtype=np.uint64), n_rows)
    ctr = r * np.uint64(per_row) + k
    cols = below(hash3(seed, 1, ctr), n_cols).reshape(n_rows, per_row)
    attempt = 1
    while True:
        s = np.sort(cols, axis=1)
        dup_rows = np.nonzero((s[:, 1:] == s[:, :-1]).any(axis=1))[0]
        if len(dup_rows) == 0:
            break
        for rr in dup_rows:  # few rows; redraw later duplicates
            row = cols[rr]
            seen = set()
            for j in range(per_row):
                c = int(row[j])
                while c in seen:
                    c = int(below(hash3(seed, 100 + attempt, np.array([rr * per_row + j], np.uint64)), n_cols)[0])
                    attempt += 1
                seen.add(c)
                row[j] = c
    vals = sym_unit(hash3(seed, 2, ctr))
    return r.astype(np.uint32), cols.reshape(-1).astype(np.uint32), vals


def laplacian_2d(g: int):
    """5-point Laplacian, n = g*g, nnz = 5n - 4g; entries inserted row by row."""
    n = g * g
    i = np.arange(n, dtype=np.int64)
    x, y = i % g, i // g
    parts = []
    for (dx, dy, v) in ((0, -1, -1.0), (-1, 0, -1.0), (0, 0, 4.0), (1, 0, -1.0), (0, 1, -1.0)):
        ok = (x + dx >= 0) & (x + dx < g) & (y + dy >= 0) & (y + dy < g)
        parts.append((i[ok], (i + dx + dy * g)[ok], np.full(ok.sum(), v), dy * g + dx))
    rows = np.concatenate([p[0] for p in parts])
    cols = np.concatenate([p[1] for p in parts])
    vals = np.concatenate([p[2] for p in parts])
    order = np.lexsort((cols, rows))
    return rows[order].astype(np.uint32), cols[order].astype(np.uint32), vals[order]


def laplacian_3d(g: int):
    """7-point Laplacian, n = g^3; 6 on the diagonal, -1 for neighbours."""
    n = g ** 3
    i = np.arange(n, dtype=np.int64)
    x, y, z = i % g, (i // g) % g, i // (g * g)
    parts = []
    for (dx, dy, dz, v) in ((0, 0, -1, -1.0), (0, -1, 0, -1.0), (-1, 0, 0, -1.0), (0, 0, 0, 6.0),
                            (1, 0, 0, -1.0), (0, 1, 0, -1.0), (0, 0, 1, -1.0)):
        ok = (x + dx >= 0) & (x + dx < g) & (y + dy >= 0) & (y + dy < g) & (z + dz >= 0) & (z + dz < g)
        parts.append((i[ok], (i + dx + dy * g + dz * g * g)[ok], np.full(ok.sum(), v)))
    rows = np.concatenate([p[0] for p in parts])
    cols = np.concatenate([p[1] for p in parts])
    vals = np.concatenate([p[2] for p in parts])
    order = np.lexsort((cols, rows))
    return rows[order].astype(np.uint32), cols[order].astype(np.uint32), vals[order]


def zipf_lengths(n_rows: int, alpha: float, cap: int, mean: float, seed: int) -> np.ndarray:
    k = np.arange(1, cap + 1, dtype=np.float64)
    p = k ** (-alpha)
    cdf = np.cumsum(p) / p.sum()
    zmean = float((k * p).sum() / p.sum())
    s = mean / zmean
    u = unit(hash3(seed, 3, np.arange(n_rows, dtype=np.uint64)))
    z = np.searchsorted(cdf, u, side="right") + 1
    z = np.minimum(z, cap)
    return np.clip(np.rint(z * s), 1, cap).astype(np.int64)


def zipf_rows(n_rows: int, alpha: float = 1.8, cap: int = 10_000, mean: float = 16.0, seed: int = 42):
    L = zipf_lengths(n_rows, alpha, cap, mean, seed)
    rows = np.repeat(np.arange(n_rows, dtype=np.uint32), L)
    ctr = np.arange(len(rows), dtype=np.uint64)
    cols = below(hash3(seed, 4, ctr), n_rows)
    vals = sym_unit(hash3(seed, 5, ctr))
    return rows, cols, vals


def uniform_rows(n_rows: int, n_cols: int, per_row: int, seed: int):
    rows = np.repeat(np.arange(n_rows, dtype=np.uint32), per_row)
    ctr = np.arange(len(rows), dtype=np.uint64)
    return rows, below(hash3(seed, 6, ctr), n_cols), sym_unit(hash3(seed, 7, ctr))


def relock_batch(n_rows: int, n_cols: int, nnz: int, seed: int, row_frac: float = 0.10,
                 entry_frac: float = 0.01, zero_frac: float = 0.0):
    """entry_frac*nnz inserts with rows uniform over a random row_frac of the
    rows and uniform columns; collisions overwrite (buffer wins). With
    zero_frac > 0 that share of the values is 0.0 (deletes)."""
    pick = unit(hash3(seed, 8, np.arange(n_rows, dtype=np.uint64))) < row_frac
    dirty = np.nonzero(pick)[0].astype(np.uint32)
    m = int(round(entry_frac * nnz))
    ctr = np.arange(m, dtype=np.uint64)
    rows = dirty[below(hash3(seed, 9, ctr), len(dirty))] if len(dirty) else np.zeros(0, np.uint32)
    cols = below(hash3(seed, 10, ctr), n_cols)
    vals = sym_unit(hash3(seed, 11, ctr))
    if zero_frac > 0:
        vals = np.where(unit(hash3(seed, 12, ctr)) < zero_frac, 0.0, vals)
    return rows.astype(np.uint32), cols.astype(np.uint32), vals


def dense_x(n: int, seed: int) -> np.ndarray:
    return sym_unit(hash3(seed, 13, np.arange(n, dtype=np.uint64)))
