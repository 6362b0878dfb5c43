"""lock() on the GPU: bit-exact against the oracle (structure, value bits and
Spira's capacity) and Spira's golden fixtures; error behaviour."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import oracle
import spira_gb300 as sg
from spira_gb300 import gen
from conftest import assert_csr_equal

pytestmark = pytest.mark.gpu

GOLD = json.loads((Path(__file__).parent / "golden" / "golden.json").read_text())


def _epochs(ep):
    out = []
    for e in ep:
        out.append((np.array([t[0] for t in e], np.uint32), np.array([t[1] for t in e], np.uint32),
                    np.array([float.fromhex(t[2]) for t in e], np.float64)))
    return out


def _gold_csr(d):
    return oracle.Csr(d["n_rows"], d["n_cols"], np.array(d["off"], np.uint64), np.array(d["cols"], np.uint32),
                      np.array([float.fromhex(v) for v in d["vals"]], np.float64), d["capacity"])


def gpu_lock(ctx, n_rows, n_cols, epochs):
    A = sg.Csr(ctx, n_rows, n_cols)
    for r, c, v in epochs:
        A.lock(r, c, v)
    return A


@pytest.mark.parametrize("kat", GOLD["kats"], ids=[k["name"] for k in GOLD["kats"]])
def test_lock_kats_match_spira(ctx, kat):
    A = gpu_lock(ctx, kat["n_rows"], kat["n_cols"], _epochs(kat["epochs"]))
    assert_csr_equal(A.download(), _gold_csr(kat["csr"]))


def _random_epochs(n_rows, n_cols, sizes, seed, zero_every=11, nan_every=0):
    eps = []
    for e, m in enumerate(sizes):
        ctr = np.arange(m, dtype=np.uint64)
        r = gen.below(gen.hash3(seed + e, 1, ctr), n_rows)
        c = gen.below(gen.hash3(seed + e, 2, ctr), n_cols)
        v = gen.sym_unit(gen.hash3(seed + e, 3, ctr))
        if zero_every:
            v[::zero_every] = 0.0
            v[5::zero_every * 3] = -0.0
        if nan_every:
            v[::nan_every] = np.nan
        eps.append((r, c, v))
    return eps


@pytest.mark.parametrize("n_rows,n_cols,sizes", [
    (1, 1, [5, 5]),
    (7, 3, [40, 0, 40]),
    (1000, 1000, [20_000, 3_000, 3_000, 500]),
    (3000, 50, [100_000, 10_000]),          # heavy duplicates (last write wins)
    (50, 100_000, [30_000, 30_000]),         # wide rows
    (200_000, 200_000, [300_000, 30_000]),   # many empty rows
])
def test_lock_random_epochs_bit_exact(ctx, n_rows, n_cols, sizes):
    eps = _random_epochs(n_rows, n_cols, sizes, seed=n_rows + 7, nan_every=997)
    A = gpu_lock(ctx, n_rows, n_cols, eps)
    assert_csr_equal(A.download(), oracle.lock_epochs(n_rows, n_cols, eps))


def test_lock_config1_full(ctx):
    r, c, v = gen.random_rows(10_000, 10_000, 10, seed=42)
    A = gpu_lock(ctx, 10_000, 10_000, [(r, c, v)])
    rec = {w["name"]: w for w in GOLD["workloads"]}["random_10k_10_per_row"]
    assert oracle.csr_digest(A.download()) == rec["csr_sha256"]


def test_lock_laplacian_relock_matches_oracle(ctx):
    r, c, v = gen.laplacian_2d(400)
    n = 400 * 400
    b = gen.relock_batch(n, n, len(r), seed=3, zero_frac=0.2)
    A = gpu_lock(ctx, n, n, [(r, c, v), b])
    assert_csr_equal(A.download(), oracle.lock_epochs(n, n, [(r, c, v), b]))


@pytest.mark.parametrize("vals", [[1.0, 2.5, 2.0, -3.0, 7.0], [1.0, 0.0, 2.0, -0.0, 7.0]])
def test_lock_strictly_sorted_input(ctx, vals):
    """Strictly increasing (row, col) inserts install the staged arrays as
    the CSR directly; a zero among them sends the lock down the general
    path, which drops it."""
    rows = np.array([0, 0, 1, 2, 4], np.uint32)
    cols = np.array([1, 3, 0, 2, 0], np.uint32)
    vals = np.array(vals)
    A = gpu_lock(ctx, 5, 4, [(rows, cols, vals)])
    assert_csr_equal(A.download(), oracle.lock_epochs(5, 4, [(rows, cols, vals)]))


def test_lock_presorted_input_with_duplicates(ctx):
    """Inserts already in (row, col) order skip the sort; duplicates still
    resolve to the last write and a last zero still deletes."""
    rows = np.array([0, 0, 0, 1, 1, 3, 3, 3], np.uint32)
    cols = np.array([1, 1, 2, 0, 0, 0, 5, 5], np.uint32)
    vals = np.array([1.0, 2.0, 3.0, 4.0, 0.0, 7.0, -1.0, 9.0])
    A = gpu_lock(ctx, 4, 6, [(rows, cols, vals)])
    assert_csr_equal(A.download(), oracle.lock_epochs(4, 6, [(rows, cols, vals)]))
    # a sorted second epoch merges too
    b = (np.array([0, 2, 3], np.uint32), np.array([2, 2, 5], np.uint32), np.array([0.0, 5.0, 8.0]))
    A.lock(*b)
    assert_csr_equal(A.download(), oracle.lock_epochs(4, 6, [(rows, cols, vals), b]))


@pytest.mark.parametrize("lengths,n_rows,n_cols", [
    ([13_000, 5, 0, 7], 4, 50_000),                    # a row longer than one on-chip tile: global sort
    ([3, 0, 0, 1, 2] * 4000, 20_000, 300),              # short rows, heavy duplicates
    ([9000, 1, 1, 2000, 4000, 1], 6, 1 << 22),          # long rows within a tile, 22-bit columns
])
def test_lock_row_grouped_inserts(ctx, lengths, n_rows, n_cols):
    """Inserts staged row by row with columns in any order (the on-chip
    per-row sort), duplicates and zeros included; also rows far apart."""
    lengths = np.asarray(lengths, np.int64)
    rows = np.repeat(np.arange(len(lengths), dtype=np.uint32), lengths)
    if n_rows > len(lengths):
        rows = (rows.astype(np.uint64) * (n_rows // len(lengths))).astype(np.uint32)
    ctr = np.arange(len(rows), dtype=np.uint64)
    cols = gen.below(gen.hash3(len(rows), 1, ctr), n_cols)
    vals = gen.sym_unit(gen.hash3(len(rows), 2, ctr))
    vals[::13] = 0.0
    A = gpu_lock(ctx, n_rows, n_cols, [(rows, cols, vals)])
    assert_csr_equal(A.download(), oracle.lock_epochs(n_rows, n_cols, [(rows, cols, vals)]))


@pytest.mark.parametrize("n_cols", [300, 1 << 22, 1 << 26, (1 << 26) + 1])
def test_lock_row_grouped_every_length_class(ctx, n_cols):
    """Grouped inserts with a row at every boundary of the on-chip sort's
    length classes (written through, bitonic in registers for 2..32 entries,
    a warp per row up to 512, a block per row up to 2048 / 4096 / 12 288),
    rows shuffled so the classes interleave; duplicates and zeros included.
    300 columns make duplicates dense; 2^26 columns is the widest key the
    on-chip sort takes, one more column sends the epoch to the global sort."""
    base = [0, 1, 2, 3, 4, 5, 7, 8, 9, 15, 16, 17, 31, 32, 33, 34, 100, 511, 512, 513, 2047, 2048, 2049, 4096,
            4097, 12288]
    lengths = np.array(base * 3, np.int64)
    lengths = lengths[np.argsort(gen.hash3(5, 0, np.arange(len(lengths), dtype=np.uint64)))]
    n_rows = len(lengths)
    rows = np.repeat(np.arange(n_rows, dtype=np.uint32), lengths)
    ctr = np.arange(len(rows), dtype=np.uint64)
    cols = gen.below(gen.hash3(n_cols, 1, ctr), n_cols)
    cols[7::50] = cols[6::50][: len(cols[7::50])]  # neighbours repeated: duplicates in every class
    vals = gen.sym_unit(gen.hash3(n_cols, 2, ctr))
    vals[::17] = 0.0
    A = gpu_lock(ctx, n_rows, n_cols, [(rows, cols, vals)])
    assert_csr_equal(A.download(), oracle.lock_epochs(n_rows, n_cols, [(rows, cols, vals)]))


def test_lock_row_grouped_nothing_dropped(ctx):
    """Grouped inserts with distinct columns in every row and no zeros: the
    rows sorted in place are the CSR as they stand (nothing moves after the
    sort); capacity stays exact."""
    lengths = np.array([1, 2, 5, 31, 32, 33, 300, 512, 513, 2048, 2049, 5000, 0, 7] * 2, np.int64)
    n_rows, n_cols = len(lengths), 1 << 20
    rows = np.repeat(np.arange(n_rows, dtype=np.uint32), lengths)
    start = np.repeat(np.cumsum(lengths) - lengths, lengths)
    j = np.arange(len(rows), dtype=np.int64) - start  # position inside the row
    cols = ((j * 40_503 + rows.astype(np.int64) * 977) % n_cols).astype(np.uint32)  # distinct within a row
    vals = 1.0 + gen.unit(gen.hash3(3, 2, np.arange(len(rows), dtype=np.uint64)))
    A = gpu_lock(ctx, n_rows, n_cols, [(rows, cols, vals)])
    ref = oracle.lock_epochs(n_rows, n_cols, [(rows, cols, vals)])
    assert int(ref.off[-1]) == len(rows)
    assert_csr_equal(A.download(), ref)


def test_lock_row_grouped_sparse_rows(ctx):
    """Grouped inserts whose rows are far apart (large row spans per tile)."""
    n = 3_000_000
    rows = np.repeat(np.array([0, 5, 1_000_000, 2_999_999], np.uint32), [700, 3000, 2, 40])
    ctr = np.arange(len(rows), dtype=np.uint64)
    cols = gen.below(gen.hash3(8, 1, ctr), n)
    vals = gen.sym_unit(gen.hash3(8, 2, ctr))
    A = gpu_lock(ctx, n, n, [(rows, cols, vals)])
    assert_csr_equal(A.download(), oracle.lock_epochs(n, n, [(rows, cols, vals)]))


@pytest.mark.parametrize("dups", [False, True])
def test_lock_long_empty_stretches(ctx, dups):
    """Row offsets across long runs of empty rows: more stretches of > 4096
    empty rows than the offsets pass lists for the whole grid (the rest are
    written warp by warp), a leading and a trailing stretch; strictly
    increasing inserts (direct path) and inserts with duplicates (sorted)."""
    n = 6_000_000
    hot = (7000 + 4999 * np.arange(1190, dtype=np.uint64)).astype(np.uint32)
    rows = np.repeat(hot, 2)
    cols = np.tile(np.array([3, 9], np.uint32), len(hot))
    if dups:
        cols[1::2] = 3
    vals = gen.sym_unit(gen.hash3(12, 2, np.arange(len(rows), dtype=np.uint64)))
    A = gpu_lock(ctx, n, n, [(rows, cols, vals)])
    assert_csr_equal(A.download(), oracle.lock_epochs(n, n, [(rows, cols, vals)]))


def test_lock_nothing_staged_on_many_rows(ctx):
    n = 5_000_000
    e = np.array([], np.uint32)
    A = gpu_lock(ctx, n, n, [(e, e, np.array([]))])
    H = A.download()
    assert A.nnz == 0 and len(H.off) == n + 1 and not H.off.any()


def test_lock_zipf_long_rows(ctx):
    r, c, v = gen.zipf_rows(100_000, seed=9)
    b = gen.relock_batch(100_000, 100_000, len(r), seed=10, zero_frac=0.05)
    A = gpu_lock(ctx, 100_000, 100_000, [(r, c, v), b])
    assert_csr_equal(A.download(), oracle.lock_epochs(100_000, 100_000, [(r, c, v), b]))


def test_out_of_range_leaves_matrix_unchanged(ctx):
    A = gpu_lock(ctx, 4, 4, [(np.array([0, 1], np.uint32), np.array([1, 2], np.uint32), np.array([1.0, 2.0]))])
    before = A.download()
    with pytest.raises(sg.OutOfRange):
        A.lock(np.array([4], np.uint32), np.array([0], np.uint32), np.array([1.0]))
    with pytest.raises(sg.OutOfRange):
        A.lock(np.array([0], np.uint32), np.array([4], np.uint32), np.array([1.0]))
    assert_csr_equal(A.download(), before)


def test_load_csr_validation(ctx):
    A = sg.Csr(ctx, 2, 3)
    with pytest.raises(sg.InvalidArgument, match="offsets\\[0\\]"):
        A.load([1, 1, 1], [0], [1.0])
    with pytest.raises(sg.InvalidArgument, match="does not equal nnz"):
        A.load([0, 1, 1], [0, 1], [1.0, 2.0])
    with pytest.raises(sg.InvalidArgument, match="non-decreasing"):
        A.load([0, 2, 1], [0], [1.0])
    with pytest.raises(sg.InvalidArgument, match="out of bounds"):
        A.load([0, 1, 1], [3], [1.0])
    with pytest.raises(sg.InvalidArgument, match="strictly sorted"):
        A.load([0, 2, 2], [1, 1], [1.0, 2.0])
    A.load([0, 2, 3], [0, 2, 1], [1.0, 2.0, 3.0])
    assert A.info()["built"] and A.nnz == 3 and A.get(1, 1) == 3.0 and A.get(1, 0) is None


def test_relock_after_load_with_explicit_zeros(ctx):
    """A loaded CSR may hold explicit zeros; Spira's merge drops them from the
    rows it touches (csr_build.hpp:274-276) and keeps them elsewhere."""
    off = np.array([0, 3, 5], np.uint64)
    cols = np.array([0, 1, 2, 0, 2], np.uint32)
    vals = np.array([0.0, 2.0, -0.0, 0.0, 5.0])
    A = sg.Csr(ctx, 2, 3)
    A.load(off, cols, vals)
    A.lock(np.array([0, 0], np.uint32), np.array([1, 2], np.uint32), np.array([7.0, 8.0]))
    got = A.download()
    # row 0 touched: its zero at col 0 is dropped, col 2 (-0.0) replaced by 8.0;
    # row 1 untouched: keeps its explicit zero
    np.testing.assert_array_equal(got.off, [0, 2, 4])
    np.testing.assert_array_equal(got.cols, [1, 2, 0, 2])
    np.testing.assert_array_equal(got.vals, [7.0, 8.0, 0.0, 5.0])


def test_context_destroyed_before_its_matrices():
    """Destroying a context frees its matrices' device memory; the handles
    stay safe to use (LogicError) and to destroy."""
    c2 = sg.Context(0)
    A = sg.Csr(c2, 10, 10)
    A.lock(np.array([1], np.uint32), np.array([2], np.uint32), np.array([3.0]))
    c2.close()
    c3 = sg.Context(0)
    r = np.array([1], np.uint32)
    v = np.array([3.0])
    st = sg.lib().spg_lock(c3.h, A.h, r.ctypes.data, r.ctypes.data, v.ctypes.data, 1)
    assert st == sg.LogicError.code  # the orphaned matrix refuses work
    A.close()
    c3.close()


def test_spmv_before_lock_is_logic_error(ctx):
    A = sg.Csr(ctx, 3, 3)
    with pytest.raises(sg.LogicError):
        A.spmv_host(np.zeros(3))
    A.lock(np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0))
    np.testing.assert_array_equal(A.spmv_host(np.ones(3)), np.zeros(3))
    with pytest.raises(sg.InvalidArgument):
        A.spmv_host(np.zeros(2))


@pytest.mark.parametrize("offset", [0, 1, 3])
def test_lock_device_arrays_at_any_alignment(ctx, offset):
    """Device-staged inserts whose arrays start 0, 4 or 12 bytes past a
    16-byte boundary (the range check reads 16 bytes at a time only when both
    index arrays are aligned); sizes not a multiple of 4, grouped and
    ungrouped epochs."""
    import torch
    for grouped in (True, False):
        n, m = 5000, 40_001
        ctr = np.arange(m, dtype=np.uint64)
        r = np.sort(gen.below(gen.hash3(offset, 1, ctr), n)) if grouped else gen.below(gen.hash3(offset, 1, ctr), n)
        c = gen.below(gen.hash3(offset, 2, ctr), n)
        v = gen.sym_unit(gen.hash3(offset, 3, ctr))
        pad = np.zeros(offset, np.uint32)
        dr = torch.from_numpy(np.concatenate([pad, r]).view(np.int32)).cuda()[offset:]
        dc = torch.from_numpy(np.concatenate([pad, c]).view(np.int32)).cuda()[offset:]
        dv = torch.from_numpy(v).cuda()
        assert (dr.data_ptr() % 16 == 0) == (offset == 0)
        A = sg.Csr(ctx, n, n)
        A.lock_device(dr, dc, dv, m)
        assert_csr_equal(A.download(), oracle.lock_epochs(n, n, [(r, c, v)]))


def test_lock_random_order_first_lock_scales(ctx):
    """A first lock of 2 M inserts in random order over 2 M rows: correct, and
    linear in the inserts (milliseconds; any per-insert work proportional to
    the gap between neighbouring rows would take minutes here)."""
    import time
    n, m = 2_000_000, 2_000_000
    ctr = np.arange(m, dtype=np.uint64)
    r = gen.below(gen.hash3(41, 1, ctr), n)
    c = gen.below(gen.hash3(41, 2, ctr), n)
    v = gen.sym_unit(gen.hash3(41, 3, ctr))
    A = sg.Csr(ctx, n, n)
    A.lock(r[:1000], c[:1000], v[:1000])  # warm the kernels and the pool
    A = sg.Csr(ctx, n, n)
    t0 = time.perf_counter()
    A.lock(r, c, v)
    ctx.sync()
    assert time.perf_counter() - t0 < 2.0
    assert_csr_equal(A.download(), oracle.lock_epochs(n, n, [(r, c, v)]))
