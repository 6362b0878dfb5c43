"""spg_spmv_noalloc: SpMV for callers that cannot allocate device memory.

It must give the same y as the regular entry point (spg_spmv with the MERGE
variant, within the SpMV tolerance the other tests use), on two calls in a
row (the shared scratch array keeps the previous call's contents), and must
refuse matrices beyond its fixed scratch with a clear error. Called through
the C ABI with ctypes. This file sorts last so that a run stopping at the
first failure has run every other test before it.
"""
from __future__ import annotations

import ctypes as C

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


def test_noalloc_matches_regular_entry_point_twice():
    import torch
    import oracle
    ctx = sg.Context(0)  # a fresh context: the test also runs alone in a fresh process
    n = 200_000
    r, c, v = gen.zipf_rows(n, seed=17)
    A = sg.Csr(ctx, n, n)
    A.lock(r, c, v)
    H = A.download()
    assert n + A.nnz <= sg.lib().spg_spmv_noalloc_max()
    for call, seed in enumerate((18, 19)):
        x = gen.dense_x(n, seed)
        xd = torch.from_numpy(x).cuda()
        y_ref_dev = torch.empty(n, dtype=torch.float64, device="cuda")
        y_new = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        A.spmv(xd, y_ref_dev, sg.SPMV_MERGE)
        _noalloc(ctx, A, xd, y_new)
        ctx.sync()
        y_regular = y_ref_dev.cpu().numpy()
        y_noalloc = y_new.cpu().numpy()
        _, scale = oracle.spmv_compensated(H, x)
        assert spmv_rel_err(y_noalloc, y_regular, scale) <= SPMV_TOL, f"call {call}"
        y_c, _ = oracle.spmv_compensated(H, x)
        assert spmv_rel_err(y_noalloc, y_c, scale) <= SPMV_TOL, f"call {call}"
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
