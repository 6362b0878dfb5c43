"""Host model of SPG_SPGEMM_WARPSORT_* (spira_gb300/csrc/spg_spgemm_sort.cu).

Restates the kernel's index arithmetic in Python, step by step, and checks
it on the CPU: the tile plan (every tile's rows and products fit the block's
shared memory and the block scan's threads, the launch's tile bound holds), the
per-row expansion (owner max-scan, slots inside the warp's arrays; or, for
rows of at most 32 A entries whose B rows fit power-of-two blocks, the
presorted runs placed block by block, odd blocks reversed, and the network
started at the first stage that merges blocks), the bitonic network as the
kernel runs it (element 32 e + lane; partners 32 or more apart inside a
lane, nearer ones by shuffles), the left-to-right run
sums (run boundaries from the neighbours' columns; rows without equal
columns keep every product as its own sum) with in-place compaction, and the
ordered copy-out (a warp per row). The result must be
bit-identical to the oracle's Spira-order SpGEMM. Every shared-memory index
the model touches is asserted inside its buffer.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from spira_gb300 import gen

RB = 128          # rows per tile (one thread each in the block scan)
WARPS = 4
CONFIGS = {"warpsort_64": (64, 1024), "warpsort_128": (128, 2048), "warpsort_256": (256, 4096)}


def csr(n_rows, n_cols, rows, cols, vals):
    return oracle.lock_epochs(n_rows, n_cols, [(rows, cols, vals)])


def products(A, B):
    off, cols = A.off.astype(np.int64), A.cols.astype(np.int64)
    blen = np.diff(B.off.astype(np.int64))
    per_entry = blen[cols]
    cs = np.concatenate([[0], np.cumsum(per_entry)])
    return cs[off[1:]] - cs[off[:-1]]


def heavy(A, P, hb):
    r = np.diff(A.off.astype(np.int64))
    return (P > hb) | (r > hb)


def tile_plan(A, P, hb, tpb):
    m = A.n_rows
    pofs = np.concatenate([[0], np.cumsum(P)])
    W = tpb - hb
    hv = heavy(A, P, hb)
    starts = []
    for i in range(m):
        st = (i % RB == 0) or hv[i] or hv[i - 1] or (pofs[i] // W != pofs[i - 1] // W)
        if st:
            starts.append(i)
    n_heavy = int(hv.sum())
    t_max = (m + RB - 1) // RB + int(pofs[m]) // W + 2 * n_heavy + 3
    return pofs, starts + [m], t_max


def bitonic_warp(key, E, k0=2):
    """key: list of 32*E ints, element i = 32 e + lane; the kernel's network
    (stages below k0 skipped)."""
    N = 32 * E
    k = 2
    while k <= N:
        if k < k0:
            k <<= 1
            continue
        j = k >> 1
        while j > 0:
            new = list(key)
            if j >= 32:
                jj = j >> 5
                for lane in range(32):
                    for e in range(E):
                        if e & jj == 0:
                            f = e | jj
                            up = ((32 * e) & k) == 0
                            a, b = key[32 * e + lane], key[32 * f + lane]
                            sw = (a > b) if up else (a < b)
                            new[32 * e + lane], new[32 * f + lane] = (b, a) if sw else (a, b)
            else:
                for e in range(E):
                    for lane in range(32):
                        i = 32 * e + lane
                        o = key[32 * e + (lane ^ j)]
                        keep_min = ((i & k) == 0) == ((i & j) == 0)
                        new[i] = min(o, key[i]) if keep_min else max(o, key[i])
            key = new
            j >>= 1
        k <<= 1
    return key


def model(A, B, hb, tpb, n_runs=None):
    """n_runs: [rows sorted as presorted runs, rows sorted in full, rows with
    a run longer than one product], counted."""
    if n_runs is None:
        n_runs = [0, 0, 0]
    SB = hb.bit_length() - 1
    P = products(A, B)
    pofs, starts, t_max = tile_plan(A, P, hb, tpb)
    assert len(starts) - 1 <= t_max
    hv = heavy(A, P, hb)
    Cref_heavy = oracle.spgemm(A, B)  # heavy rows' results come from expand-sort-compress
    out_cols, out_vals, out_off = [], [], np.zeros(A.n_rows + 1, np.uint64)
    aoff, acols, avals = A.off.astype(np.int64), A.cols.astype(np.int64), A.vals
    boff, bcols, bvals = B.off.astype(np.int64), B.cols.astype(np.int64), B.vals
    base = 0
    for t in range(len(starts) - 1):
        row0, row1 = starts[t], starts[t + 1]
        nr = row1 - row0
        assert 1 <= nr <= RB
        p0 = pofs[row0]
        if nr == 1 and hv[row0]:
            b, e = int(Cref_heavy.off[row0]), int(Cref_heavy.off[row0 + 1])
            out_off[row0] = base
            out_cols.append(Cref_heavy.cols[b:e])
            out_vals.append(Cref_heavy.vals[b:e])
            base += e - b
            continue
        assert pofs[row1] - p0 <= tpb, "tile products exceed the shared-memory budget"
        slots = tpb + RB  # one slot of skew per row
        s_col = np.full(slots, -1, np.int64)
        s_prod = np.full(slots, np.nan)
        counts = []
        for j in range(nr):
            i = row0 + j
            assert not hv[i]
            reg = int(pofs[i] - p0) + j
            Pi = int(P[i])
            assert reg + Pi <= slots
            if Pi == 0:
                counts.append((reg, 0))
                continue
            E = 1 if Pi <= 32 else 2 if Pi <= 64 else 4 if Pi <= 128 else 8
            assert Pi <= hb and 32 * E <= max(hb, 32)
            r = int(aoff[i + 1] - aoff[i])
            assert r <= hb
            own = np.zeros(hb, np.int64)
            w_a = np.zeros(hb)
            w_b = np.zeros(hb, np.int64)
            ex = 0
            exs, Ls = [], []
            for tt in range(r):
                k = acols[aoff[i] + tt]
                L = int(boff[k + 1] - boff[k])
                w_a[tt] = avals[aoff[i] + tt]
                w_b[tt] = boff[k] - ex
                if L:
                    assert ex < Pi <= hb
                    own[ex] = tt
                exs.append(ex)
                Ls.append(L)
                ex += L
            assert ex == Pi
            lmax = max(Ls) if r <= 32 else 0
            lg = 0 if lmax <= 1 else (lmax - 1).bit_length()
            runs = r <= 32 and lg >= 1 and (r << lg) <= 32 * E
            keys = []
            if runs:
                bm = (1 << lg) - 1
                for q in range(32 * E):
                    t = q >> lg
                    assert t < 32  # the shuffle source lane
                    u = bm - (q & bm) if t & 1 else q & bm
                    if t < r and u < Ls[t]:
                        s = exs[t] + u
                        assert 0 <= s < Pi
                        bi = int(w_b[t] + s)
                        assert boff[acols[aoff[i] + t]] <= bi < boff[acols[aoff[i] + t] + 1]
                        s_prod[reg + s] = np.float64(w_a[t]) * np.float64(bvals[bi])
                        keys.append((int(bcols[bi]) << SB) | s)
                    else:
                        keys.append((1 << 64) - 1)
                assert sorted(k for k in keys if k != (1 << 64) - 1) == sorted(set(keys) - {(1 << 64) - 1})
                n_runs[0] += 1
            else:
                for s in range(32 * E):
                    if s < Pi:
                        o = int(own[:s + 1].max())  # inclusive max-scan
                        bi = int(w_b[o] + s)
                        assert boff[acols[aoff[i] + o]] <= bi < boff[acols[aoff[i] + o] + 1]
                        s_prod[reg + s] = np.float64(w_a[o]) * np.float64(bvals[bi])
                        keys.append((int(bcols[bi]) << SB) | s)
                    else:
                        keys.append((1 << 64) - 1)
                n_runs[1] += 1
            skeys = bitonic_warp(keys, E, (2 << lg) if runs else 2)
            assert skeys == sorted(keys)
            # the same warp: products gathered into sorted order (registers)
            pv = [s_prod[reg + (kk & ((1 << SB) - 1))] for kk in skeys[:Pi]]
            col = [kk >> SB for kk in skeys[:Pi]]
            # run boundaries from the neighbours' columns (the kernel's shuffles)
            head = [q == 0 or col[q - 1] != col[q] for q in range(Pi)]
            cont = [q + 1 < Pi and col[q + 1] == col[q] for q in range(Pi)]
            if any(cont):  # the warp vote: some run is longer than one product
                n_runs[2] += 1
                for q in range(Pi):  # the sorted copy in shared memory
                    s_col[reg + q] = col[q]
                    s_prod[reg + q] = pv[q]
                keep = [False] * Pi
                for q in range(Pi):
                    if head[q]:  # the head lane sums its run left to right
                        acc, r = pv[q], q + 1
                        while r < Pi and s_col[reg + r] == col[q]:
                            acc = np.float64(acc) + np.float64(s_prod[reg + r])
                            r += 1
                        pv[q] = acc
                        keep[q] = not abs(acc) <= 0.0  # spgemm.hpp:44: v != V{}
            else:
                keep = [head[q] and not abs(pv[q]) <= 0.0 for q in range(Pi)]
            # ballot ranking: kept sums in element order, compacted from reg
            w = reg
            for q in range(Pi):
                if keep[q]:
                    s_col[w], s_prod[w] = col[q], pv[q]
                    w += 1
            counts.append((reg, w - reg))
        kept = [k for _, k in counts]
        excl = np.concatenate([[0], np.cumsum(kept)])
        total = int(excl[-1])
        for j in range(nr):
            out_off[row0 + j] = base + excl[j]
        oc, ov = np.full(total, -1, np.int64), np.full(total, np.nan)
        for j in range(nr):  # a warp per row, lanes over its kept entries
            e0, n = int(excl[j]), int(excl[j + 1] - excl[j])
            src = counts[j][0]
            assert 0 <= src and src + n <= slots and e0 + n <= total
            assert (oc[e0:e0 + n] == -1).all()  # every output entry written once
            oc[e0:e0 + n], ov[e0:e0 + n] = s_col[src:src + n], s_prod[src:src + n]
        assert (oc >= 0).all()
        out_cols.append(oc)
        out_vals.append(ov)
        base += total
    out_off[A.n_rows] = base
    return (out_off, np.concatenate(out_cols).astype(np.uint32) if out_cols else np.zeros(0, np.uint32),
            np.concatenate(out_vals) if out_vals else np.zeros(0))


def _check(A, B, name):
    hb, tpb = CONFIGS[name]
    n_runs = [0, 0, 0]
    off, cols, vals = model(A, B, hb, tpb, n_runs)
    C = oracle.spgemm(A, B)
    np.testing.assert_array_equal(off, C.off.astype(np.uint64))
    np.testing.assert_array_equal(cols, C.cols)
    np.testing.assert_array_equal(vals.view(np.uint64), C.vals.view(np.uint64))
    return n_runs


@pytest.mark.parametrize("name", list(CONFIGS))
def test_model_uniform_rows(name):
    n = 600
    r, c, v = gen.uniform_rows(n, n, 8, seed=3)
    A = csr(n, n, r, c, v)
    n_runs = _check(A, A, name)
    assert n_runs[0] > 0.9 * n  # 8 runs of <= 8: the presorted-run path


@pytest.mark.parametrize("name", list(CONFIGS))
def test_model_mixed_rows_heavy_and_cancellations(name):
    """Row lengths 0..60 and a few long rows (heavy), integer values so that
    exact cancellations drop entries; rectangular B."""
    n_rows, n_inner, n_cols = 300, 200, 500
    lengths = np.array([0, 1, 3, 8, 9, 20, 2, 33, 5, 12] * (n_rows // 10))
    lengths[7::40] = 90
    rows = np.repeat(np.arange(n_rows, dtype=np.uint32), lengths)
    ctr = np.arange(len(rows), dtype=np.uint64)
    cols = gen.below(gen.hash3(8, 1, ctr), n_inner)
    vals = (gen.below(gen.hash3(8, 2, ctr), 5).astype(np.int64) - 2).astype(np.float64)
    A = csr(n_rows, n_inner, rows, cols, vals)
    blen = np.array([0, 2, 5, 1, 9, 3] * (n_inner // 6) + [4] * (n_inner % 6))
    brows = np.repeat(np.arange(n_inner, dtype=np.uint32), blen)
    ctr2 = np.arange(len(brows), dtype=np.uint64)
    bcols = gen.below(gen.hash3(9, 1, ctr2), n_cols)
    bvals = (gen.below(gen.hash3(9, 2, ctr2), 5).astype(np.int64) - 2).astype(np.float64)
    bvals[::4] = gen.sym_unit(gen.hash3(9, 3, ctr2[::4]))
    B = csr(n_inner, n_cols, brows, bcols, bvals)
    n_runs = _check(A, B, name)
    assert n_runs[0] > 0 and n_runs[1] > 0  # both expansions ran
    assert 0 < n_runs[2] < n_runs[0] + n_runs[1]  # rows with and without equal columns


@pytest.mark.parametrize("E", [1, 2, 4, 8])
def test_network_from_presorted_runs(E):
    """Blocks of 2^lg sorted keys, odd blocks reversed, padding anywhere after
    a block's real keys: the network started at stage 2^(lg+1) sorts them."""
    rng = np.random.default_rng(E)
    N = 32 * E
    for lg in range(1, N.bit_length()):
        if (1 << lg) > N:
            break
        for _ in range(6):
            n_blocks = int(rng.integers(1, N // (1 << lg) + 1))
            keys = [(1 << 64) - 1] * N
            for t in range(n_blocks):
                L = int(rng.integers(0, (1 << lg) + 1))
                run = sorted(int(x) for x in rng.choice(1 << 20, L, replace=False))
                block = run + [(1 << 64) - 1] * ((1 << lg) - L)
                if t & 1:
                    block = block[::-1]
                keys[t << lg:(t + 1) << lg] = block
            assert bitonic_warp(keys, E, 2 << lg) == sorted(keys)


def test_model_tile_bound_many_empty_rows():
    """Long runs of rows without products still give tiles of <= 128 rows."""
    n = 1000
    rows = np.array([5, 500, 501, 999], np.uint32)
    A = csr(n, n, rows, np.array([1, 2, 3, 4], np.uint32), np.ones(4))
    for name in CONFIGS:
        _check(A, A, name)


PER_LANE = 1


def lookback_model(states, t):
    """The kernel's warp look-back: states[q] = (status, value) of tile q
    (status 1 aggregate, 2 inclusive prefix); returns tile t's exclusive
    prefix, reading windows of 32 * PER_LANE predecessors (lane l, word j:
    tile p - PER_LANE l - j), and the number of windows read."""
    excl, p = 0, t - 1
    steps = 0
    while True:
        steps += 1
        words = {}
        for lane in range(32):
            for j in range(PER_LANE):
                q = p - (PER_LANE * lane + j)
                words[(lane, j)] = states[q] if q >= 0 else (0, 0)
        jp = {lane: min([j for j in range(PER_LANE) if words[(lane, j)][0] == 2], default=PER_LANE)
              for lane in range(32)}
        pref = [lane for lane in range(32) if jp[lane] < PER_LANE]
        lp = pref[0] if pref else 32
        for lane in range(32):
            upto = PER_LANE if lane < lp else jp[lane] + 1 if lane == lp else 0
            for j in range(upto):
                st, val = words[(lane, j)]
                assert st != 0
                excl += val
        if pref:
            return excl, steps
        p -= 32 * PER_LANE


def test_lookback_model_sums_every_predecessor_once():
    rng = np.random.default_rng(0)
    for trial in range(200):
        T = int(rng.integers(1, 400))
        counts = rng.integers(0, 50, T)
        incl = np.cumsum(counts)
        states = []
        for q in range(T):
            if q == 0 or rng.random() < 0.03:
                states.append((2, int(incl[q])))
            else:
                states.append((1, int(counts[q])))
        t = T - 1
        if t == 0:
            continue
        excl, steps = lookback_model(states, t)
        assert excl == int(incl[t - 1])
        # the walk stops at the nearest published prefix
        nearest = max(q for q in range(t) if states[q][0] == 2)
        assert steps == (t - 1 - nearest) // (32 * PER_LANE) + 1
