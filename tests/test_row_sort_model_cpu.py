"""CPU model of the row-grouped sort that lock() and transpose use when the
staged rows are already grouped (spira_gb300/csrc/spg_prims.cu,
sort_grouped_rows): the length classes, the segmented bitonic network of the
short rows (lane by lane, as the warp runs it), the span tiles of the medium
rows and the bounds the kernels rely on (rows per tile, entries per tile, key
bits). The order it must give is Spira's: stable (row, col) order, the
staging position deciding among duplicates so that the last write wins
(include/spira/matrix/buffer/aos_array_buffer.hpp:76-101, driven by
include/spira/matrix/matrix.hpp:277-342)."""
from __future__ import annotations

import numpy as np
import pytest

SEG_SPAN, SEG_TILE_ROWS, TS_SMALL, TS_MAX, SEG_MAX_CBITS = 2048, 64, 4096, 12288, 26


def seg_class(L: int) -> int:
    if L <= 1:
        return 0
    if L <= 32:
        return int(L - 1).bit_length()
    if L <= SEG_SPAN:
        return 6
    if L <= TS_SMALL:
        return 7
    if L <= TS_MAX:
        return 8
    return 9


def segment_bitonic(keys: np.ndarray, P: int) -> np.ndarray:
    """The warp network: 32 lanes, aligned P-lane segments, shfl_xor partners."""
    key = keys.astype(np.uint32).copy()
    lane = np.arange(32)
    k = 2
    while k <= P:
        j = k >> 1
        while j > 0:
            other = key[lane ^ j]
            up = np.full(32, True) if k == P else (lane & k) == 0
            low = (lane & j) == 0
            key = np.where(low == up, np.minimum(key, other), np.maximum(key, other))
            j >>= 1
        k <<= 1
    return key


def test_length_classes():
    assert [seg_class(L) for L in (0, 1, 2, 3, 4, 5, 8, 9, 16, 17, 32)] == [0, 0, 1, 2, 2, 3, 3, 4, 4, 5, 5]
    assert [seg_class(L) for L in (33, 2048, 2049, 4096, 4097, 12288, 12289)] == [6, 6, 7, 7, 8, 8, 9]
    # the padded length 2^c holds the row
    for L in range(2, 33):
        c = seg_class(L)
        assert 2 ** (c - 1) < L <= 2 ** c


@pytest.mark.parametrize("P", [2, 4, 8, 16, 32])
def test_segment_bitonic_gives_stable_column_order(P):
    rng = np.random.default_rng(P)
    for trial in range(200):
        ncols = [3, 50, 1 << 26][trial % 3]  # heavy duplicates .. 26-bit columns
        keys = np.full(32, 0xFFFFFFFF, np.uint64)
        want = []
        for g in range(32 // P):
            L = int(rng.integers(P // 2 + 1, P + 1)) if P > 2 else 2
            cols = rng.integers(0, ncols, L)
            for j in range(L):
                keys[g * P + j] = (int(cols[j]) << 5) | j
            want.append(sorted(range(L), key=lambda j: (cols[j], j)))  # stable column order
        out = segment_bitonic(keys, P)
        for g in range(32 // P):
            got = [int(k) & 31 for k in out[g * P: g * P + len(want[g])]]
            assert got == want[g]
            # the padding sorts behind the row
            assert all(int(k) == 0xFFFFFFFF for k in out[g * P + len(want[g]): (g + 1) * P])


def test_short_keys_stay_below_the_padding():
    assert (((1 << SEG_MAX_CBITS) - 1) << 5 | 31) < 0xFFFFFFFF


def _spans(lengths):
    """Span tiles of the medium rows: span -> [(row, start, length)]."""
    off = np.concatenate([[0], np.cumsum(lengths)])
    tiles = {}
    for r, L in enumerate(lengths):
        if seg_class(L) == 6:
            tiles.setdefault(int(off[r]) // SEG_SPAN, []).append((r, int(off[r]), int(L)))
    return tiles


@pytest.mark.parametrize("pattern", ["all33", "mixed", "zipf_like", "one_long_between"])
def test_span_tiles_fit_the_small_kernel(pattern):
    rng = np.random.default_rng(7)
    if pattern == "all33":
        lengths = np.full(5000, 33)
    elif pattern == "mixed":
        lengths = rng.choice([1, 2, 33, 40, 2048, 2047, 5000], 3000)
    elif pattern == "zipf_like":
        lengths = np.minimum(rng.zipf(1.8, 20000), 10000)
    else:
        lengths = np.array([2048, 33, 2048, 1, 2048, 4096, 33] * 50)
    tiles = _spans(lengths)
    for rows in tiles.values():
        assert len(rows) <= SEG_TILE_ROWS - 1  # 33 apart in a 2048 span: <= 63
        E = sum(L for _, _, L in rows)
        assert E < 2 * SEG_SPAN <= TS_SMALL
        rbits = (len(rows) - 1).bit_length()
        assert rbits + SEG_MAX_CBITS <= 32


def tile_sort_model(cols_in, rows_in_tile, cbits):
    """One tile: keys (rank << cbits | col), stable sort, outputs by rank."""
    pref = np.concatenate([[0], np.cumsum([L for _, _, L in rows_in_tile])])
    keys, pos = [], []
    for i, (_, b, L) in enumerate(rows_in_tile):
        for e in range(L):
            keys.append((i << cbits) | int(cols_in[b + e]))
            pos.append(pref[i] + e)
    order = np.argsort(np.array(keys, np.uint64), kind="stable")
    out = {}
    for q, o in enumerate(order):
        i = keys[o] >> cbits
        r, b, _ = rows_in_tile[i]
        out[b + (q - pref[i])] = (r, keys[o] & ((1 << cbits) - 1), b + (pos[o] - pref[i]))
    return out


def test_tile_sort_model_matches_stable_row_column_order():
    rng = np.random.default_rng(3)
    lengths = rng.choice([33, 50, 200, 1000, 2048], 60)
    n_cols = 1 << 22
    cbits = (n_cols - 1).bit_length()
    off = np.concatenate([[0], np.cumsum(lengths)])
    cols = rng.integers(0, 64, off[-1])  # many duplicates inside every row
    for rows in _spans(lengths).values():
        got = tile_sort_model(cols, rows, cbits)
        for r, b, L in rows:
            want = sorted(range(L), key=lambda e: (cols[b + e], e))
            for q in range(L):
                rr, c, src = got[b + q]
                assert rr == r and c == cols[b + want[q]] and src == b + want[q]
