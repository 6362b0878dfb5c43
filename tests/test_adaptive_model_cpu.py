"""Host model of SPG_SPMV_ADAPTIVE's plan and thread ownership
(spira_gb300/csrc/spg_spmv_adaptive.cu), run on the CPU: every shared-memory
index and every aligned chunk load stays inside its buffer, and every row is
written exactly once with the right sum. Mirrors the kernel's integer logic
step by step."""
from __future__ import annotations

import numpy as np
import pytest

from spira_gb300 import gen

AD_BLOCK, AD_LONG, AD_ROWCAP = 256, 128, 1024


def plan(off, items):
    n = len(off) - 1
    BIN = AD_BLOCK * items - 16 - AD_LONG
    lens = np.diff(off)
    lng = lens > AD_LONG
    brk = np.zeros(n, bool)
    for r in range(n):
        b = lng[r] or r == 0 or r % AD_ROWCAP == 0
        if not b:
            b = lens[r - 1] > AD_LONG or (off[r - 1] // BIN) != (off[r] // BIN)
        brk[r] = b
    B = list(np.nonzero(brk)[0]) + [n]
    tiles = [(B[j], B[j + 1]) for j in range(len(B) - 1) if not lng[B[j]]]
    return tiles, list(np.nonzero(lng)[0])


def run_tile(off, cols, vals, x, r0, r1, items, alloc, y, writes):
    nr = r1 - r0
    assert 1 <= nr <= AD_ROWCAP
    k0, k1 = int(off[r0]), int(off[r1])
    s_end = [int(off[r0 + i + 1] - k0) for i in range(nr)]
    a0 = k0 & ~15
    span = ((k1 + 15) & ~15) - a0
    assert span <= AD_BLOCK * items, "bulk-copy window larger than a stage"
    assert a0 + span <= alloc, "bulk-copy window leaves the cols/vals allocation"
    ro = r0 & ~1
    nro = ((r1 + 1 - ro) + 1) & ~1
    assert nro <= AD_ROWCAP + 2 and ro + nro <= (len(off) - 1) + 3, "offsets window leaves its allocation"
    if k1 == k0:
        for i in range(nr):
            y[r0 + i] = 0.0
            writes[r0 + i] += 1
        return
    tails, heads = {}, {}
    for t in range(AD_BLOCK):
        ca = a0 + items * t
        lo, hi = max(ca, k0), min(ca + items, k1)
        if lo >= hi:
            continue
        assert ca % items == 0 and ca + items <= alloc  # aligned chunk inside the allocation
        plo, phi = lo - k0, hi - k0
        row, head = 0, False
        if plo > 0:
            l, h = 0, nr - 1
            while l < h:
                m = (l + h) >> 1
                if s_end[m] > plo:
                    h = m
                else:
                    l = m + 1
            row = l
            head = (0 if row == 0 else s_end[row - 1]) < plo
        rfirst, acc, head_row = row, 0.0, None
        for u in range(items):
            it = ca + u
            if it < lo or it >= hi:
                continue
            p = it - k0
            while s_end[row] <= p:
                assert row < nr
                if head and row == rfirst:
                    heads[t] = (row, acc)
                    head_row = row
                else:
                    y[r0 + row] = acc
                    writes[r0 + row] += 1
                acc = 0.0
                row += 1
            acc += x[cols[it]] * vals[it]
        while row < nr and s_end[row] <= phi:
            if head and row == rfirst:
                heads[t] = (row, acc)
                head_row = row
            else:
                y[r0 + row] = acc
                writes[r0 + row] += 1
            acc = 0.0
            row += 1
        if row < nr:
            tails[t] = (row, acc)
    for t, (hr, hv) in heads.items():
        j = t - 1
        while j >= 0 and j in tails and tails[j][0] == hr:
            j -= 1
        s = sum(tails[q][1] for q in range(j + 1, t))
        y[r0 + hr] = s + hv
        writes[r0 + hr] += 1


def check(lengths, items, seed=0):
    lengths = np.asarray(lengths, np.int64)
    off = np.zeros(len(lengths) + 1, np.int64)
    off[1:] = np.cumsum(lengths)
    nnz = int(off[-1])
    alloc = ((nnz + 15) & ~15) + 16
    n_cols = 1000
    ctr = np.arange(nnz, dtype=np.uint64)
    cols = gen.below(gen.hash3(seed, 1, ctr), n_cols)
    vals = gen.sym_unit(gen.hash3(seed, 2, ctr))
    x = gen.dense_x(n_cols, seed + 1)
    tiles, longs = plan(off, items)
    y = np.full(len(lengths), np.nan)
    writes = np.zeros(len(lengths), np.int64)
    for r0, r1 in tiles:
        run_tile(off, cols, vals, x, r0, r1, items, alloc, y, writes)
    for r in longs:
        b, e = int(off[r]), int(off[r + 1])
        a0 = b & ~(items - 1)
        assert ((e - a0 + items - 1) // items) * items + a0 <= alloc
        y[r] = float(np.dot(x[cols[b:e]], vals[b:e]))
        writes[r] += 1
    assert np.all(writes == 1), np.nonzero(writes != 1)[0][:10]
    ref = np.array([np.dot(x[cols[off[r]:off[r + 1]]], vals[off[r]:off[r + 1]]) for r in range(len(lengths))])
    np.testing.assert_allclose(y, ref, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("items", [8, 16])
@pytest.mark.parametrize("lengths", [
    [0], [1], [0, 0, 0], [5] * 3000, [0] * 2500 + [3] + [0] * 10,
    [128, 129, 127, 0, 1, 2000, 128, 3, 4095, 1],
    [1, 0, 2, 0, 0, 3] * 700,
    [16] * 1000, [15, 17] * 600,
])
def test_adaptive_model(items, lengths):
    check(lengths, items)


@pytest.mark.parametrize("items", [8, 16])
def test_adaptive_model_zipf(items):
    L = gen.zipf_lengths(20_000, 1.8, 10_000, 16.0, seed=3)
    check(L, items, seed=4)
