"""CPU model of the row-grouped sort that lock() and transpose use when the
staged rows are already grouped (spira_gb300/csrc/spg_prims.cu,
sort_grouped_rows and dedup_grouped_rows): the length classes, the segmented
bitonic network of the short rows and the warp network of the medium rows
(lane by lane, as the warp runs them), the block radix rank of the long rows,
and the bounds the kernels rely on (key bits, bank conflicts). The order it must give is Spira's: stable (row, col) order, the
staging position deciding among duplicates so that the last write wins
(include/spira/matrix/buffer/aos_array_buffer.hpp:76-101, driven by
include/spira/matrix/matrix.hpp:277-342)."""
from __future__ import annotations

import numpy as np
import pytest

SEG_MEDIUM, SEG_MAX_CBITS = 512, 26
TS0, TS1, TS_MAX = 128 * 16, 256 * 16, 768 * 16


def seg_class(L: int) -> int:
    if L <= 1:
        return 0
    if L <= 32:
        return int(L - 1).bit_length()
    if L <= SEG_MEDIUM:
        return 6
    if L <= TS0:
        return 7
    if L <= TS1:
        return 8
    if L <= TS_MAX:
        return 9
    return 10


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
    assert [seg_class(L) for L in (33, 512, 513, 2048, 2049, 4096, 4097, 12288, 12289)] == [6, 6, 7, 7, 8, 8, 9, 9, 10]
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


def warp_bitonic(keys: np.ndarray, E: int) -> np.ndarray:
    """The warp network over 32 E elements (element 32 e + lane in key[e] of
    that lane): partners 32 or more apart within a lane's registers, nearer
    ones by shuffles; as the kernels run it."""
    key = keys.reshape(E, 32).copy()  # key[e][lane]
    lane = np.arange(32)
    k = 2
    while k <= 32 * E:
        j = k >> 1
        while j > 0:
            if j >= 32:
                jj = j >> 5
                for e in range(E):
                    if e & jj == 0:
                        f = e | jj
                        up = ((32 * e) & k) == 0
                        a, b = key[e].copy(), key[f].copy()
                        sw = (a > b) if up else (a < b)
                        key[e] = np.where(sw, b, a)
                        key[f] = np.where(sw, a, b)
            else:
                for e in range(E):
                    o = key[e][lane ^ j]
                    i = 32 * e + lane
                    keep_min = ((i & k) == 0) == ((i & j) == 0)
                    key[e] = np.where(keep_min, np.minimum(o, key[e]), np.maximum(o, key[e]))
            j >>= 1
        k <<= 1
    return key.reshape(-1)


@pytest.mark.parametrize("E", [2, 4, 8, 16])
def test_medium_row_network_gives_stable_column_order(E):
    """Rows of 33..512 entries: keys col << 9 | position, padding all ones;
    32-bit keys while the columns need at most 22 bits."""
    rng = np.random.default_rng(E)
    for trial in range(20):
        L = int(rng.integers(16 * E + 1, 32 * E + 1)) if E > 2 else int(rng.integers(33, 65))
        cbits = [6, 22][trial % 2]
        cols = rng.integers(0, 1 << cbits, L)
        cols[1::9] = cols[0]  # duplicates: the position orders them
        keys = np.full(32 * E, 0xFFFFFFFF, np.uint64)
        keys[:L] = (cols.astype(np.uint64) << np.uint64(9)) | np.arange(L, dtype=np.uint64)
        out = warp_bitonic(keys, E)
        want = sorted(range(L), key=lambda p: (cols[p], p))
        assert [int(k) & 511 for k in out[:L]] == want
        assert (out[L:] == 0xFFFFFFFF).all()
    # the largest real key stays below the padding only up to 22 column bits
    assert (((1 << 22) - 1) << 9 | 511) < 0xFFFFFFFF
    assert (((1 << 23) - 1) << 9 | 511) == 0xFFFFFFFF


RS_DBITS, RS_WORDS = 6, 32


def pad33(p):
    return p + (p >> 5)


def block_radix_pass(keys, idxs, T, I, shift):
    """One pass of the tile kernel's ranking, index for index: packed 16-bit
    counters (digit d in word d % 32, half d // 32) in a column per thread,
    a raking scan over flat (word, thread) order, rank = prefix + earlier
    same digit in the thread. Returns the scattered (keys, idxs)."""
    E = len(keys)
    col_stride = T + T // 32
    ctr = np.zeros(RS_WORDS * T + RS_WORDS * T // 32, np.uint64)
    local = {}
    for t in range(T):
        for i in range(I):
            e = t * I + i
            if e >= E:
                break
            d = (int(keys[e]) >> shift) & 63
            a = pad33(t) + (d & 31) * col_stride
            assert a == pad33((d & 31) * T + t)
            sh = (d // 32) * 16
            cv = int(ctr[a])
            ctr[a] = cv + (1 << sh)
            local[e] = (cv >> sh) & 0xFFFF
    sums = [sum(int(ctr[33 * t + j]) for j in range(RS_WORDS)) for t in range(T)]
    assert all(33 * t + j == pad33(RS_WORDS * t + j) for t in range(T) for j in range(RS_WORDS))
    total = sum(sums)
    run = 0
    for t in range(T):
        for j in range(RS_WORDS):
            a = 33 * t + j
            x = int(ctr[a])
            ctr[a] = run
            run += x
    low_total = total & 0xFFFF
    out_k = np.zeros(E, np.uint64)
    out_i = np.zeros(E, np.int64)
    for e in range(E):
        t = e // I
        d = (int(keys[e]) >> shift) & 63
        a = pad33(t) + (d & 31) * col_stride
        hi = d // 32
        rank = ((int(ctr[a]) >> (16 * hi)) & 0xFFFF) + (low_total if hi else 0) + local[e]
        out_k[rank] = keys[e]
        out_i[rank] = idxs[e]
    return out_k, out_i


@pytest.mark.parametrize("T,I,E,bits", [(32, 4, 128, 12), (32, 4, 77, 18), (64, 3, 190, 28), (32, 8, 256, 6)])
def test_block_radix_rank_model_is_a_stable_sort(T, I, E, bits):
    rng = np.random.default_rng(E + bits)
    keys = rng.integers(0, 1 << bits, E).astype(np.uint64)
    keys[::7] = keys[0]  # ties: order must stay the input order
    idxs = np.arange(E)
    k, i = keys.copy(), idxs.copy()
    for p in range((bits + RS_DBITS - 1) // RS_DBITS):
        k, i = block_radix_pass(k, i, T, I, p * RS_DBITS)
    order = np.argsort(keys, kind="stable")
    assert (k == keys[order]).all() and (i == idxs[order]).all()


@pytest.mark.parametrize("I", [8, 16, 24])
def test_blocked_reads_and_raking_are_bank_conflict_free(I):
    lanes = np.arange(32)
    for i in range(I):  # a warp's lanes reading their i-th of I consecutive entries
        banks = [pad33(int(t) * I + i) % 32 for t in lanes]
        # 8 or 16 entries per lane (the kernels' sizes): one bank per lane; 24: two lanes at most
        assert max(np.bincount(banks, minlength=32)) <= (1 if I in (8, 16) else 2)
    for j in range(RS_WORDS):  # raking: lane t reads word j of its own segment
        assert len({(33 * int(t) + j) % 32 for t in lanes}) == 32
