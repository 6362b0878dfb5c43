"""spg_spmv_noalloc: SpMV for callers that cannot allocate device memory.

It must give the same y as the regular entry point (spg_spmv with the MERGE
variant, within the SpMV tolerance the other tests use) on two calls in a
row, the second on a different matrix with a different number of tiles and
different tile starts (the shared scratch array then holds the first call's
starts and carries), must allocate nothing (the context's memory pool and the
device's free memory are unchanged across a warm call), and must refuse
matrices beyond its fixed scratch with a clear error. Called through the C
ABI with ctypes. This file sorts last so that a run stopping at the first
failure has run every other test before it.
"""
from __future__ import annotations

import numpy as np
import pytest

import spira_gb300 as sg
from spira_gb300 import gen
from conftest import SPMV_TOL, spmv_rel_err

pytestmark = pytest.mark.gpu


def _noalloc(ctx, A, xd, yd):
    st = sg.lib().spg_spmv_noalloc(ctx.h, A.h, xd.data_ptr(), yd.data_ptr(), None)
    if st != 0:
        raise sg.SpgError(sg.lib().spg_last_error().decode())


def _check_against_regular(ctx, A, H, x_seed):
    import torch
    import oracle
    n_rows, n_cols = H.n_rows, H.n_cols
    x = gen.dense_x(n_cols, x_seed)
    xd = torch.from_numpy(x).cuda()
    y_reg = torch.empty(n_rows, dtype=torch.float64, device="cuda")
    y_new = torch.full((n_rows,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    A.spmv(xd, y_reg, sg.SPMV_MERGE)
    _noalloc(ctx, A, xd, y_new)
    ctx.sync()
    y_c, scale = oracle.spmv_compensated(H, x)
    assert spmv_rel_err(y_new.cpu().numpy(), y_reg.cpu().numpy(), scale) <= SPMV_TOL
    assert spmv_rel_err(y_new.cpu().numpy(), y_c, scale) <= SPMV_TOL
    return xd, y_new


def test_noalloc_matches_regular_entry_point_twice():
    import torch
    ctx = sg.Context(0)  # a fresh context: the test also runs alone in a fresh process
    # first call: a 200 000-row Zipf matrix (long and short rows, many tiles)
    n1 = 200_000
    r, c, v = gen.zipf_rows(n1, seed=17)
    A1 = sg.Csr(ctx, n1, n1)
    A1.lock(r, c, v)
    H1 = A1.download()
    # second call: a 2D Laplacian of another size, so the tile count and every
    # tile start differ from what the first call left in the shared array
    g = 300
    r2, c2, v2 = gen.laplacian_2d(g)
    A2 = sg.Csr(ctx, g * g, g * g)
    A2.lock(r2, c2, v2)
    H2 = A2.download()
    limit = sg.lib().spg_spmv_noalloc_max()
    t1, t2 = n1 + A1.nnz, g * g + A2.nnz
    assert t1 <= limit and t2 <= limit and t1 != t2
    _check_against_regular(ctx, A1, H1, 18)
    xd, yd = _check_against_regular(ctx, A2, H2, 19)
    # a warm call allocates nothing: neither from the context's pool nor from
    # the driver (the pool's cached blocks would hide a pool allocation from
    # the free-memory count, so both are checked)
    torch.cuda.synchronize()
    ctx.sync()
    used0, reserved0 = ctx.pool_used()
    free0, _ = torch.cuda.mem_get_info()
    _noalloc(ctx, A2, xd, yd)
    ctx.sync()
    used1, reserved1 = ctx.pool_used()
    free1, _ = torch.cuda.mem_get_info()
    assert (used1, reserved1) == (used0, reserved0)
    assert free1 == free0
    ctx.close()


def test_noalloc_rejects_matrices_beyond_its_scratch():
    import torch
    ctx = sg.Context(0)
    limit = int(sg.lib().spg_spmv_noalloc_max())
    n = limit  # rows alone exceed the limit once nonzeros are added
    A = sg.Csr(ctx, n, 4)
    A.lock(np.array([0], np.uint32), np.array([1], np.uint32), np.array([2.0]))
    xd = torch.zeros(4, dtype=torch.float64, device="cuda")
    yd = torch.zeros(8, dtype=torch.float64, device="cuda")  # never written: the call is refused
    st = sg.lib().spg_spmv_noalloc(ctx.h, A.h, xd.data_ptr(), yd.data_ptr(), None)
    assert st == 1  # SPG_ERR_INVALID_ARGUMENT
    assert "scratch limit" in sg.lib().spg_last_error().decode()
    ctx.close()
