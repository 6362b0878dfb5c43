"""The three implementations of the seeded draws agree: numpy (gen.py), C
(oracle/gen_host.c) and CUDA (spg_gen_draw)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from spira_gb300 import gen


@pytest.mark.parametrize("kind,bound", [(0, 7), (0, 4_000_000), (0, 2**32), (1, 0), (2, 0)])
def test_c_draws_equal_numpy(kind, bound):
    ctr = np.arange(100_000, dtype=np.uint64) + np.uint64(12345)
    h = gen.hash3(77, 5, ctr)
    want = gen.below(h, bound) if kind == 0 else (gen.sym_unit(h) if kind == 1 else gen.unit(h))
    got = oracle.gen_draw(77, 5, 100_000, kind, bound, counter0=12345)
    np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8))


def test_zipf_host_equals_numpy():
    r, c, v = gen.zipf_rows(30_000, seed=9)
    r2, c2, v2 = oracle.zipf_rows_host(30_000, seed=9)
    np.testing.assert_array_equal(r, r2)
    np.testing.assert_array_equal(c, c2)
    np.testing.assert_array_equal(v.view(np.uint64), v2.view(np.uint64))


def test_zipf_length_distribution():
    L = gen.zipf_lengths(200_000, 1.8, 10_000, 16.0, seed=1)
    assert L.min() >= 1 and L.max() <= 10_000
    assert 13.0 < L.mean() < 17.0  # rounding of small Z pulls the mean a little under 16


def test_laplacian_shapes():
    r, c, v = gen.laplacian_2d(5)
    assert len(r) == 5 * 25 - 4 * 5
    r3, c3, v3 = gen.laplacian_3d(4)
    assert len(r3) == 7 * 64 - 6 * 16
    assert np.all(np.diff(r.astype(np.int64) * 25 + c) > 0)  # inserted in (row, col) order


@pytest.mark.gpu
def test_device_draws_equal_numpy(ctx):
    import torch
    import spira_gb300 as sg
    from spira_gb300 import gen_device
    out = torch.empty(50_000, dtype=torch.int32, device="cuda")
    sg.gen_draw(ctx, 5, 3, 50_000, sg.GEN_BELOW_U32, 1000, out, counter0=7)
    ctx.sync()
    want = gen.below(gen.hash3(5, 3, np.arange(50_000, dtype=np.uint64) + np.uint64(7)), 1000)
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), want)
    r, c, v, m = gen_device.zipf_rows(ctx, 30_000, seed=9)
    r2, c2, v2 = gen.zipf_rows(30_000, seed=9)
    assert m == len(r2)
    np.testing.assert_array_equal(r[:m].cpu().numpy().view(np.uint32), r2)
    np.testing.assert_array_equal(c[:m].cpu().numpy().view(np.uint32), c2)
    np.testing.assert_array_equal(v[:m].cpu().numpy(), v2)
