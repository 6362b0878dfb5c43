"""Host model of SPG_SPMV_ADAPTIVE (spira_gb300/csrc/spg_spmv_adaptive.cu),
run on the CPU before the kernel ever runs: it follows the kernel's integer
logic lane by lane (bitmap words, row-start prefix counts, vector-load
windows, direct writes, chunk records and the record fix-up) and checks that
every load window stays inside the padded CSR allocation, that only real
columns are gathered, and that every row's y is written exactly once with
the right sum."""
from __future__ import annotations

import numpy as np
import pytest

from spira_gb300 import gen

NONE = 0xFFFFFFFF


def model(off, cols, vals, x, items):
    n = len(off) - 1
    nnz = int(off[-1])
    alloc = ((nnz + 15) & ~15) + 16          # csr_alloc_elems(nnz)
    lens = np.diff(off)
    nonempty = np.nonzero(lens > 0)[0]
    nzrow = nonempty if len(nonempty) < n else None
    bitmap = np.zeros((nnz + 31) // 32 + 1, np.uint64)
    for r in nonempty:
        b = int(off[r])
        bitmap[b >> 5] |= np.uint64(1 << (b & 31))
    chunk = 32 * items
    n_chunks = (nnz + chunk - 1) // chunk
    pc = np.array([bin(int(w)).count("1") for w in bitmap], np.int64)
    pcs = np.concatenate([[0], np.cumsum(pc)])
    chunk_base = [int(pcs[c * items]) for c in range(n_chunks)]
    y = np.full(n, np.nan)
    writes = np.zeros(n, np.int64)

    def ywrite(i):
        return int(nzrow[i]) if nzrow is not None else i

    recs = [None] * (2 * n_chunks)
    for w in range(n_chunks):
        lanes = []
        for lane in range(32):
            p0 = w * chunk + lane * items
            word = 0
            if p0 < nnz:
                word = (int(bitmap[p0 >> 5]) >> (p0 & 31))
                if items < 32:
                    word &= (1 << items) - 1
                if nnz - p0 < items:
                    word &= (1 << (nnz - p0)) - 1
            lanes.append((p0, word))
        pcs_l = [bin(wd).count("1") for _, wd in lanes]
        excl = np.concatenate([[0], np.cumsum(pcs_l)])[:32]
        state = []
        for lane, (p0, word) in enumerate(lanes):
            sb = chunk_base[w] + int(excl[lane])
            cur = sb - 1
            acc, head, seen = 0.0, 0.0, False
            for h in range(items // 16):
                base = p0 + 16 * h
                nv = min(nnz - base, 16) if base < nnz else 0
                if nv:
                    assert base % 16 == 0 and base + 16 <= alloc, "vector load window leaves allocation"
                for u in range(16):
                    i = 16 * h + u
                    if (word >> i) & 1:
                        if not seen:
                            head, seen = acc, True
                        else:
                            assert 0 <= cur
                            r = ywrite(cur)
                            y[r] = acc
                            writes[r] += 1
                        acc = 0.0
                        cur += 1
                    if u < nv:
                        k = base + u
                        acc += x[cols[k]] * vals[k]
            state.append((sb, cur, acc, head, word != 0, word))
        has = [s[4] for s in state]
        carry = [0.0] * 32
        run = 0.0
        for lane in range(32):  # exclusive segmented scan of tails
            carry[lane] = run
            tail = state[lane][2]
            run = tail if has[lane] else run + tail
        for lane in range(32):
            sb, cur, tail, head, hs, word = state[lane]
            if not hs:
                continue
            total = carry[lane] + head
            if any(has[:lane]):
                r = ywrite(sb - 1)
                y[r] = total
                writes[r] += 1
            else:
                recs[2 * w] = (NONE if (lane == 0 and (word & 1)) else sb - 1, total)
        sb, cur, tail, head, hs, word = state[31]
        out = tail if hs else carry[31] + tail
        if not any(has):
            recs[2 * w] = (cur, out)
            recs[2 * w + 1] = (NONE, 0.0)
        else:
            recs[2 * w + 1] = (cur, out)
    assert all(r is not None for r in recs), "a chunk record was left unwritten"
    for q in range(len(recs)):  # seg_fixup
        row = recs[q][0]
        if row == NONE:
            continue
        if q > 0:
            p = q - 1
            if recs[p][0] == NONE and p > 0:
                p -= 1
            if recs[p][0] == row:
                continue
        s = recs[q][1]
        k = q + 1
        while k < len(recs):
            r = recs[k][0]
            if r == NONE and k + 1 < len(recs):
                k += 1
                r = recs[k][0]
            if r != row:
                break
            s += recs[k][1]
            k += 1
        rr = ywrite(row)
        y[rr] = s
        writes[rr] += 1
    for r in np.nonzero(lens == 0)[0]:
        y[r] = 0.0
        writes[r] += 1
    return y, writes


def check(lengths, items, seed=0):
    lengths = np.asarray(lengths, np.int64)
    off = np.zeros(len(lengths) + 1, np.int64)
    off[1:] = np.cumsum(lengths)
    nnz = int(off[-1])
    ctr = np.arange(nnz, dtype=np.uint64)
    cols = gen.below(gen.hash3(seed, 1, ctr), 1000)
    vals = gen.sym_unit(gen.hash3(seed, 2, ctr))
    x = gen.dense_x(1000, seed + 1)
    y, writes = model(off, cols, vals, x, items)
    assert np.all(writes == 1), (np.nonzero(writes != 1)[0][:10], writes[writes != 1][:10])
    ref = np.array([np.dot(x[cols[off[r]:off[r + 1]]], vals[off[r]:off[r + 1]]) for r in range(len(lengths))])
    np.testing.assert_allclose(y, ref, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("items", [16, 32])
@pytest.mark.parametrize("lengths", [
    [0], [1], [0, 0, 0], [5] * 700, [0] * 50 + [3] + [0] * 10,
    [128, 129, 127, 0, 1, 2000, 128, 3, 4095, 1],
    [1, 0, 2, 0, 0, 3] * 300,
    [16] * 300, [15, 17] * 200, [32] * 100, [1024] * 3, [1023, 1025, 1],
    [5000], [0, 5000, 0],
])
def test_adaptive_model(items, lengths):
    check(lengths, items)


@pytest.mark.parametrize("items", [16, 32])
def test_adaptive_model_zipf(items):
    L = gen.zipf_lengths(3000, 1.8, 10_000, 16.0, seed=3)
    check(L, items, seed=4)


@pytest.mark.parametrize("sub", [2, 4, 8, 16])
def test_interleaved_layout_is_a_bijection_read_in_order(sub):
    """INTERLEAVED's plan-time copy: nonzero p = 512 w + 16 l + u (chunk w,
    lane l, item u) is written to 512 w + 64 (u // 2) + 2 l + u % 2 (values
    and columns alike), and the kernel's sub-batch h of SUB items reads pairs
    at 64 ((SUB h + u) // 2) + 2 l, u = 0, 2, ...: every slot of a chunk is
    written once, and each lane reads back its own 16 nonzeros in order."""
    w = 3
    dst = {}
    for lane in range(32):
        for u in range(16):
            p = 512 * w + 16 * lane + u
            d = 512 * w + 64 * (u >> 1) + 2 * lane + (u & 1)
            assert d not in dst
            dst[d] = p
    assert sorted(dst) == list(range(512 * w, 512 * w + 512))
    for lane in range(32):
        got = []
        for h in range(16 // sub):
            for u in range(0, sub, 2):
                at = 512 * w + 64 * ((sub * h + u) >> 1) + 2 * lane
                got += [dst[at], dst[at + 1]]
        assert got == [512 * w + 16 * lane + u for u in range(16)]
