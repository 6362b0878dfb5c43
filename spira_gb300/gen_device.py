"""The large generators of spira_gb300.gen, drawn on the device (torch
tensors holding uint32 / float64 bits). Equal element for element to the host
versions (tests/test_gen.py)."""
from __future__ import annotations

import numpy as np

from . import GEN_BELOW_U32, GEN_SYM_F64, Context, gen_draw, gen_expand_rows
from . import gen


def _empty(n, dtype):
    import torch
    return torch.empty(max(n, 1), dtype=dtype, device="cuda")


def rows_from_lengths(ctx: Context, lengths: np.ndarray):
    import torch
    L = torch.from_numpy(np.ascontiguousarray(lengths, dtype=np.int64)).cuda()
    torch.cuda.synchronize()
    total = gen_expand_rows(ctx, L, len(lengths))
    rows = _empty(total, torch.int32)
    gen_expand_rows(ctx, L, len(lengths), rows)
    return rows, total


def zipf_rows(ctx: Context, n_rows: int, alpha: float = 1.8, cap: int = 10_000, mean: float = 16.0, seed: int = 42):
    """Device (rows, cols, vals, m) equal to gen.zipf_rows(n_rows, ...)."""
    import torch
    L = gen.zipf_lengths(n_rows, alpha, cap, mean, seed)
    rows, m = rows_from_lengths(ctx, L)
    cols = _empty(m, torch.int32)
    vals = _empty(m, torch.float64)
    gen_draw(ctx, seed, 4, m, GEN_BELOW_U32, n_rows, cols)
    gen_draw(ctx, seed, 5, m, GEN_SYM_F64, 0, vals)
    ctx.sync()
    return rows, cols, vals, m


def uniform_rows(ctx: Context, n_rows: int, n_cols: int, per_row: int, seed: int):
    """Device (rows, cols, vals, m) equal to gen.uniform_rows."""
    import torch
    rows, m = rows_from_lengths(ctx, np.full(n_rows, per_row, np.int64))
    cols = _empty(m, torch.int32)
    vals = _empty(m, torch.float64)
    gen_draw(ctx, seed, 6, m, GEN_BELOW_U32, n_cols, cols)
    gen_draw(ctx, seed, 7, m, GEN_SYM_F64, 0, vals)
    ctx.sync()
    return rows, cols, vals, m
