"""Element-wise operations and queries on the GPU against the oracle, bit for
bit: C = A + B, A * s and A / s (copy and in place), row sums, batched point
lookups and nnz-balanced partition boundaries."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import spira_gb300 as sg
from spira_gb300 import gen
from conftest import assert_csr_equal

pytestmark = pytest.mark.gpu


def _dev(ctx, H):
    """A device matrix holding the host CSR H exactly (explicit zeros kept)."""
    A = sg.Csr(ctx, H.n_rows, H.n_cols)
    A.load(H.off, H.cols, H.vals)
    return A


def _pair(n, seed, zeros=True):
    """A and B sharing positions, with exact cancellations (a + b == +-0) on
    some of them; A holds explicit zeros and NaNs as load_csr allows."""
    ra, ca, va = gen.uniform_rows(n, n, 6, seed=seed)
    A = oracle.lock_epochs(n, n, [(ra, ca, va)])
    rb, cb, vb = gen.uniform_rows(n, n, 4, seed=seed + 1)
    k = np.arange(0, len(A.cols), 3)
    rows_a = np.repeat(np.arange(n, dtype=np.uint32), np.diff(A.off).astype(np.int64))
    sv = np.where(np.arange(len(k)) % 2 == 0, -A.vals[k], 0.5 * A.vals[k])
    B = oracle.lock_epochs(n, n, [(np.concatenate([rb, rows_a[k]]), np.concatenate([cb, A.cols[k]]),
                                   np.concatenate([vb, sv]))])
    if zeros:
        A.vals[1::17] = 0.0
        A.vals[2::23] = -0.0
        A.vals[5::31] = np.nan
    return A, B


@pytest.mark.parametrize("n,seed", [(1, 1), (37, 2), (5000, 3), (120_000, 4)])
def test_add_matches_oracle(ctx, n, seed):
    Ah, Bh = _pair(n, seed)
    A, B = _dev(ctx, Ah), _dev(ctx, Bh)
    assert_csr_equal(A.add(B).download(), oracle.add(Ah, Bh))
    assert_csr_equal(B.add(A).download(), oracle.add(Bh, Ah))
    assert_csr_equal(A.add(A).download(), oracle.add(Ah, Ah))  # every entry collides


def test_add_long_rows_and_empty_rows(ctx):
    n = 60_000
    r, c, v = gen.zipf_rows(n, seed=5)
    Ah = oracle.lock_epochs(n, n, [(r, c, v)])
    # B: a few very long rows, many empty ones, and the negation of A's row 0
    lengths = np.zeros(n, np.int64)
    lengths[::9973] = 9000
    rb = np.repeat(np.arange(n, dtype=np.uint32), lengths)
    cb = gen.below(gen.hash3(6, 1, np.arange(len(rb), dtype=np.uint64)), n)
    vb = gen.sym_unit(gen.hash3(6, 2, np.arange(len(rb), dtype=np.uint64)))
    b0, e0 = int(Ah.off[0]), int(Ah.off[1])
    rb = np.concatenate([rb, np.zeros(e0 - b0, np.uint32)])
    cb = np.concatenate([cb, Ah.cols[b0:e0]])
    vb = np.concatenate([vb, -Ah.vals[b0:e0]])
    Bh = oracle.lock_epochs(n, n, [(rb, cb, vb)])
    A, B = _dev(ctx, Ah), _dev(ctx, Bh)
    assert_csr_equal(A.add(B).download(), oracle.add(Ah, Bh))


def test_add_laplacian_with_its_relock(ctx):
    """Config 2a's matrix plus its re-locked self: full size, all collisions
    on the stencil, new entries on 10 % of rows."""
    g = 1414
    r, c, v = gen.laplacian_2d(g)
    n = g * g
    b = gen.relock_batch(n, n, len(r), seed=21)
    Ah = oracle.lock_epochs(n, n, [(r, c, v)])
    Bh = oracle.lock_epochs(n, n, [(r, c, v), b])
    A, B = sg.Csr(ctx, n, n), sg.Csr(ctx, n, n)
    A.lock(r, c, v)
    B.lock(r, c, v)
    B.lock(*b)
    assert_csr_equal(A.add(B).download(), oracle.add(Ah, Bh))


def test_add_errors(ctx):
    Ah, Bh = _pair(50, 7, zeros=False)
    A, B = _dev(ctx, Ah), _dev(ctx, Bh)
    with pytest.raises(sg.InvalidArgument):
        A.add(sg.Csr(ctx, 50, 51))
    with pytest.raises(sg.LogicError):
        A.add(sg.Csr(ctx, 50, 50))
    E = sg.Csr(ctx, 50, 50)
    E.lock(np.array([], np.uint32), np.array([], np.uint32), np.array([]))
    assert_csr_equal(A.add(E).download(), oracle.add(Ah, oracle.lock_epochs(50, 50, [])))


@pytest.mark.parametrize("s,divide", [(2.5, False), (-3.0, False), (0.0, False), (1e-310, False), (np.nan, False),
                                      (3.0, True), (1e300, True), (-0.125, True), (np.inf, True)])
def test_scale_matches_oracle(ctx, s, divide):
    Ah, _ = _pair(30_000, 8)
    A = _dev(ctx, Ah)
    want = oracle.scale(Ah, s, divide)
    assert_csr_equal(A.scaled(s, divide).download(), want)
    # in place: the same entries; capacity by the merge rule of the staged
    # scaled values (kept while 2 nnz fits, else 1.5 x 2 nnz)
    A.scale_(s, divide)
    got = A.download()
    assert_csr_equal(got, want, check_capacity=False)
    m = len(Ah.cols)
    assert got.capacity == (Ah.capacity if 2 * m <= Ah.capacity else 3 * m)


def test_scale_in_place_drops_cached_plans(ctx):
    """SpMV after an in-place scale sees the new values (the interleaved copy
    and other cached plans are rebuilt)."""
    r, c, v = gen.zipf_rows(50_000, seed=9)
    A = sg.Csr(ctx, 50_000, 50_000)
    A.lock(r, c, v)
    x = gen.dense_x(50_000, 10)
    y0 = A.spmv_host(x, variant=sg.SPMV_INTERLEAVED)
    A.scale_(2.0)  # exact: every product doubles, every sum doubles
    np.testing.assert_array_equal(A.spmv_host(x, variant=sg.SPMV_INTERLEAVED), 2.0 * y0)


def test_scale_errors(ctx):
    Ah, _ = _pair(40, 11, zeros=False)
    A = _dev(ctx, Ah)
    for z in (0.0, -0.0):
        with pytest.raises(sg.DomainError):
            A.scaled(z, divide=True)
    with pytest.raises(sg.DomainError):  # the zero check comes before the mode check
        sg.Csr(ctx, 4, 4).scaled(0.0, divide=True)
    with pytest.raises(sg.LogicError):
        sg.Csr(ctx, 4, 4).scaled(2.0)


@pytest.mark.parametrize("kind", ["zipf", "laplacian", "loaded"])
def test_row_sums_bit_exact(ctx, kind):
    if kind == "zipf":
        r, c, v = gen.zipf_rows(200_000, seed=12)
        Ah = oracle.lock_epochs(200_000, 200_000, [(r, c, v)])
    elif kind == "laplacian":
        r, c, v = gen.laplacian_2d(700)
        Ah = oracle.lock_epochs(700 * 700, 700 * 700, [(r, c, v)])
    else:
        Ah, _ = _pair(20_000, 13)
    A = _dev(ctx, Ah)
    got = A.row_sums().cpu().numpy()
    np.testing.assert_array_equal(got.view(np.uint64), oracle.row_sums(Ah).view(np.uint64))


def test_lookup_matches_host(ctx):
    import torch
    Ah, _ = _pair(40_000, 14)
    A = _dev(ctx, Ah)
    n_q = 300_000
    ctr = np.arange(n_q, dtype=np.uint64)
    # half the queries hit stored entries, half are random (mostly misses),
    # a few are outside the shape
    pick = gen.below(gen.hash3(15, 1, ctr), len(Ah.cols)).astype(np.int64)
    rows_of = np.repeat(np.arange(Ah.n_rows, dtype=np.uint64), np.diff(Ah.off).astype(np.int64))
    qr = np.where(ctr % 2 == 0, rows_of[pick], gen.below(gen.hash3(15, 2, ctr), Ah.n_rows)).astype(np.uint64)
    qc = np.where(ctr % 2 == 0, Ah.cols[pick], gen.below(gen.hash3(15, 3, ctr), Ah.n_cols)).astype(np.uint32)
    qr[::1001] = Ah.n_rows + 5
    qc[7::1009] = Ah.n_cols
    d_r, d_c = torch.from_numpy(qr.view(np.int64)).cuda(), torch.from_numpy(qc.view(np.int32)).cuda()
    d_v = torch.empty(n_q, dtype=torch.float64, device="cuda")
    d_f = torch.empty(n_q, dtype=torch.uint8, device="cuda")
    A.lookup(d_r, d_c, d_v, d_f)
    ctx.sync()
    got_v, got_f = d_v.cpu().numpy(), d_f.cpu().numpy()
    want_f = np.zeros(n_q, np.uint8)
    want_v = np.zeros(n_q, np.float64)
    for i in range(n_q):
        r, c = int(qr[i]), int(qc[i])
        if r >= Ah.n_rows or c >= Ah.n_cols:
            continue
        b, e = int(Ah.off[r]), int(Ah.off[r + 1])
        p = b + int(np.searchsorted(Ah.cols[b:e], c))
        if p < e and Ah.cols[p] == c:
            want_f[i], want_v[i] = 1, Ah.vals[p]
    np.testing.assert_array_equal(got_f, want_f)
    np.testing.assert_array_equal(got_v.view(np.uint64), want_v.view(np.uint64))


@pytest.mark.parametrize("T", [1, 2, 3, 8, 152, 4096, 1_000_000])
def test_partition_matches_oracle(ctx, T):
    r, c, v = gen.zipf_rows(100_000, seed=16)
    Ah = oracle.lock_epochs(100_000, 100_000, [(r, c, v)])
    np.testing.assert_array_equal(_dev(ctx, Ah).partition(T), oracle.partition(Ah, T))
    Eh = oracle.lock_epochs(1000, 1000, [])
    E = sg.Csr(ctx, 1000, 1000)
    E.lock(np.array([], np.uint32), np.array([], np.uint32), np.array([]))
    np.testing.assert_array_equal(E.partition(T), oracle.partition(Eh, T))


def test_degenerate_shapes(ctx, tmp_path):
    """Zero rows, zero columns and empty matrices through every operation."""
    import torch
    for n_rows, n_cols in ((0, 0), (0, 5), (5, 0), (3, 3)):
        A = sg.Csr(ctx, n_rows, n_cols)
        A.lock(np.array([], np.uint32), np.array([], np.uint32), np.array([]))
        H = A.download()
        assert_csr_equal(A.add(A).download(), oracle.add(H, H))
        assert_csr_equal(A.scaled(3.0).download(), oracle.scale(H, 3.0))
        A.scale_(2.0)
        assert A.nnz == 0
        assert len(A.row_sums_host()) == n_rows
        np.testing.assert_array_equal(A.partition(4), oracle.partition(H, 4))
        p = tmp_path / f"e{n_rows}x{n_cols}.spgcsr"
        A.save(p)
        B = sg.Csr(ctx, 1, 1).load_file(p)
        assert (B.n_rows, B.n_cols, B.nnz) == (n_rows, n_cols, 0)
        q = torch.zeros(1, dtype=torch.int64, device="cuda")
        A.lookup(q[:0], q[:0].to(torch.int32), None, torch.zeros(0, dtype=torch.uint8, device="cuda"))


def test_lookup_and_partition_before_the_first_lock(ctx):
    import torch
    A = sg.Csr(ctx, 100, 100)
    d_r = torch.arange(10, dtype=torch.int64, device="cuda")
    d_c = torch.arange(10, dtype=torch.int32, device="cuda")
    d_v = torch.full((10,), 7.0, dtype=torch.float64, device="cuda")
    d_f = torch.ones(10, dtype=torch.uint8, device="cuda")
    A.lookup(d_r, d_c, d_v, d_f)
    ctx.sync()
    assert not d_f.any() and not d_v.any()
    np.testing.assert_array_equal(A.partition(4), [0, 25, 50, 75, 100])
    with pytest.raises(sg.LogicError):
        A.row_sums_host()
