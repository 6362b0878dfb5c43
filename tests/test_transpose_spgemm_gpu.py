"""Transpose and SpGEMM on the GPU: bit-exact structure and values against
the oracle (itself pinned to Spira) and Spira's golden fixtures, at the
SpGEMM/transpose configurations' full sizes (3D Laplacian 100^3 and a
200 000^2 matrix with 8 uniform columns per row) and on edge shapes."""
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


def _gold_csr(d):
    return oracle.Csr(d["n_rows"], d["n_cols"], np.array(d["off"], np.uint64), np.array(d["cols"], np.uint32),
                      np.array([float.fromhex(v) for v in d["vals"]], np.float64), d["capacity"])


def dev(ctx, H):
    A = sg.Csr(ctx, H.n_rows, H.n_cols)
    A.load(H.off, H.cols, H.vals)
    return A


def locked(ctx, n_rows, n_cols, r, c, v):
    A = sg.Csr(ctx, n_rows, n_cols)
    A.lock(r, c, v)
    return A


@pytest.mark.parametrize("case", GOLD["transpose"], ids=[k["name"] for k in GOLD["transpose"]])
def test_transpose_kats(ctx, case):
    T = dev(ctx, _gold_csr(case["A"])).transpose()
    assert_csr_equal(T.download(), _gold_csr(case["T"]))


VARIANTS = list(sg.SPGEMM_VARIANTS.values())
VARIANT_IDS = list(sg.SPGEMM_VARIANTS.keys())


@pytest.mark.parametrize("variant", VARIANTS, ids=VARIANT_IDS)
@pytest.mark.parametrize("case", GOLD["spgemm"], ids=[k["name"] for k in GOLD["spgemm"]])
def test_spgemm_kats(ctx, case, variant):
    Cm = dev(ctx, _gold_csr(case["A"])).spgemm(dev(ctx, _gold_csr(case["B"])), variant)
    assert_csr_equal(Cm.download(), _gold_csr(case["C"]))


@pytest.mark.parametrize("rec", [w for w in GOLD["workloads"] if "spgemm_sha256" in w],
                         ids=[w["name"] for w in GOLD["workloads"] if "spgemm_sha256" in w])
def test_golden_workload_digests(ctx, rec):
    from test_oracle_pin import _workloads
    name, nr, nc, ep, x = _workloads()[rec["name"]]
    A = sg.Csr(ctx, nr, nc)
    for e in ep:
        A.lock(*e)
    assert oracle.csr_digest(A.transpose().download()) == rec["transpose_sha256"]
    for v in VARIANTS:
        Cm = A.spgemm(A, v)
        assert Cm.nnz == rec["spgemm_nnz"], sg.SPGEMM_NAMES[v]
        assert oracle.csr_digest(Cm.download()) == rec["spgemm_sha256"], sg.SPGEMM_NAMES[v]


@pytest.mark.parametrize("shape", [(1, 1), (5, 9), (9, 5), (1, 70_000), (70_000, 1), (3000, 3000)])
def test_transpose_shapes(ctx, shape):
    n_rows, n_cols = shape
    m = min(4 * max(n_rows, n_cols), 200_000)
    ctr = np.arange(m, dtype=np.uint64)
    r = gen.below(gen.hash3(1, 1, ctr), n_rows)
    c = gen.below(gen.hash3(1, 2, ctr), n_cols)
    v = gen.sym_unit(gen.hash3(1, 3, ctr))
    A = locked(ctx, n_rows, n_cols, r, c, v)
    H = A.download()
    T = A.transpose()
    assert_csr_equal(T.download(), oracle.transpose(H))
    assert_csr_equal(T.transpose().download(), H, check_capacity=False)  # double transpose


@pytest.mark.parametrize("longest", [16, 32, 33])
def test_transpose_row_length_tiers(ctx, longest):
    """Output rows of every length up to `longest`: up to 16 entries are
    sorted in a thread's registers, 17..32 across a warp, and one longer row
    sends every row through the per-tile sort."""
    n_rows, n_cols = 10_000, 700
    rows, cols = [], []
    for col in range(n_cols):
        cnt = col % (longest + 1)
        pick = np.unique(gen.below(gen.hash3(50 + col, 1, np.arange(4 * cnt + 4, dtype=np.uint64)), n_rows))
        pick = pick[gen.below(gen.hash3(60 + col, 2, np.arange(len(pick), dtype=np.uint64)), 1 << 30).argsort()]
        pick = pick[:cnt]
        rows.append(pick.astype(np.uint32))
        cols.append(np.full(len(pick), col, np.uint32))
    r, c = np.concatenate(rows), np.concatenate(cols)
    v = gen.sym_unit(gen.hash3(70, 3, np.arange(len(r), dtype=np.uint64)))
    A = locked(ctx, n_rows, n_cols, r, c, v)
    H = A.download()
    T = A.transpose()
    assert max(np.diff(T.download().off)) == longest
    assert_csr_equal(T.download(), oracle.transpose(H))


def test_transpose_zipf_long_rows(ctx):
    r, c, v = gen.zipf_rows(200_000, seed=12)
    A = locked(ctx, 200_000, 200_000, r, c, v)
    assert_csr_equal(A.transpose().download(), oracle.transpose(A.download()))


@pytest.mark.parametrize("variant", VARIANTS, ids=VARIANT_IDS)
def test_spgemm_cancellation_and_rectangular(ctx, variant):
    # integer values: exact products, cancellations produce exact zeros to drop
    ctr = np.arange(60_000, dtype=np.uint64)
    r = gen.below(gen.hash3(2, 1, ctr), 3000)
    c = gen.below(gen.hash3(2, 2, ctr), 500)
    v = (gen.below(gen.hash3(2, 3, ctr), 5).astype(np.int64) - 2).astype(np.float64)
    A = locked(ctx, 3000, 500, r, c, v)
    ctr2 = np.arange(20_000, dtype=np.uint64)
    B = locked(ctx, 500, 4000, gen.below(gen.hash3(3, 1, ctr2), 500), gen.below(gen.hash3(3, 2, ctr2), 4000),
               (gen.below(gen.hash3(3, 3, ctr2), 5).astype(np.int64) - 2).astype(np.float64))
    Cm = A.spgemm(B, variant)
    assert_csr_equal(Cm.download(), oracle.spgemm(A.download(), B.download()))


@pytest.mark.parametrize("variant", VARIANTS, ids=VARIANT_IDS)
def test_spgemm_every_row_class(ctx, variant):
    """Rows for each SpGEMM path: merge with <= 8 A entries, merge with 9..32,
    expand-sort for > 32 entries and for > 4096 products; warp sorts of 1, 2,
    4 and 8 items per lane and heavy rows for the warp-sort tiles; exact
    cancellations (integer values) included. Bit-exact against the oracle."""
    n = 3000
    lengths = np.array([0, 1, 3, 8, 9, 20, 32, 33, 60, 5] * (n // 10), np.int64)
    lengths[7::50] = 2000  # long rows: as B rows they push products past 4096
    rows = np.repeat(np.arange(n, dtype=np.uint32), lengths)
    ctr = np.arange(len(rows), dtype=np.uint64)
    cols = gen.below(gen.hash3(5, 1, ctr), n)
    vals = (gen.below(gen.hash3(5, 2, ctr), 7).astype(np.int64) - 3).astype(np.float64)
    vals[::5] = gen.sym_unit(gen.hash3(5, 3, ctr[::5]))
    A = locked(ctx, n, n, rows, cols, vals)
    H = A.download()
    Cm = A.spgemm(A, variant)
    assert_csr_equal(Cm.download(), oracle.spgemm(H, H))


@pytest.mark.parametrize("variant", VARIANTS, ids=VARIANT_IDS)
def test_spgemm_edge_shapes(ctx, variant):
    """Empty matrices, no products at all, one row, rows without products
    between long runs, and a B with more than 2^26 columns (the warp sort's
    64-bit keys)."""
    E = locked(ctx, 0, 0, np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0))
    C0 = E.spgemm(E, variant)
    assert C0.nnz == 0 and C0.n_rows == 0
    Z = locked(ctx, 50, 50, np.array([3], np.uint32), np.array([7], np.uint32), np.array([1.5]))
    Cz = Z.spgemm(Z, variant)  # row 3 names B row 7, which is empty
    assert_csr_equal(Cz.download(), oracle.spgemm(Z.download(), Z.download()))
    n = 5000
    rows = np.array([0, 0, 1, 2500, 2500, 4999], np.uint32)
    cols = np.array([0, 2500, 4999, 0, 1, 2500], np.uint32)
    A = locked(ctx, n, n, rows, cols, np.array([1.0, -2.0, 3.0, 0.5, 0.25, 4.0]))
    H = A.download()
    assert_csr_equal(A.spgemm(A, variant).download(), oracle.spgemm(H, H))
    wide = (1 << 26) + 5
    ctr = np.arange(3000, dtype=np.uint64)
    B = locked(ctx, 300, wide, gen.below(gen.hash3(4, 1, ctr), 300), gen.below(gen.hash3(4, 2, ctr), wide),
               gen.sym_unit(gen.hash3(4, 3, ctr)))
    A2 = locked(ctx, 200, 300, gen.below(gen.hash3(5, 1, ctr), 200), gen.below(gen.hash3(5, 2, ctr), 300),
                gen.sym_unit(gen.hash3(5, 3, ctr)))
    assert_csr_equal(A2.spgemm(B, variant).download(), oracle.spgemm(A2.download(), B.download()))


def test_spgemm_against_fused_order_within_tolerance(ctx):
    """Spira built with FMA contraction (GCC's default on aarch64) sums
    acc = fma(a, b, acc); the engine reproduces the uncontracted build bit for
    bit, and stays within 1e-12 (relative to sum |a_ik b_kj|) of the
    contracted order, with the same structure on generic values."""
    n = 20_000
    r, c, v = gen.uniform_rows(n, n, 12, seed=88)
    A = locked(ctx, n, n, r, c, v)
    H = A.download()
    F = oracle.spgemm(H, H, fused=True)
    Habs = H._replace(vals=np.abs(H.vals))
    S = oracle.spgemm(Habs, Habs)  # per entry: sum of |a_ik b_kj|
    for variant in VARIANTS:
        G = A.spgemm(A, variant).download()
        np.testing.assert_array_equal(G.off, F.off)
        np.testing.assert_array_equal(G.cols, F.cols)
        np.testing.assert_array_equal(S.cols, G.cols)
        assert np.all(np.abs(G.vals - F.vals) <= 1e-12 * S.vals)


def test_spgemm_selection(ctx):
    """AUTO resolves to a valid variant under each policy; the autotuner
    times every variant; the features describe the products per row."""
    n = 30_000
    r, c, v = gen.uniform_rows(n, n, 8, seed=3)
    A = locked(ctx, n, n, r, c, v)
    t, best = A.spgemm_autotune(A, 2)
    assert len(t) == len(VARIANTS) and np.all(t > 0) and best == int(np.argmin(t))
    f = A.spgemm_features(A)
    H = A.download()
    blen = np.diff(H.off.astype(np.int64))
    cs = np.concatenate([[0], np.cumsum(blen[H.cols.astype(np.int64)])])
    prods = cs[H.off[1:].astype(np.int64)] - cs[H.off[:-1].astype(np.int64)]
    bins = np.where(prods > 0, 1 + np.floor(np.log2(np.maximum(prods, 1))).astype(np.int64), 0)
    np.testing.assert_allclose(f[:32], np.bincount(np.minimum(bins, 31), minlength=32) / n, atol=1e-6)
    assert abs(f[38] - np.log2(prods.max() + 1) / 32) < 1e-6
    for policy in (sg.POLICY_AUTOTUNE, sg.POLICY_FIXED, sg.POLICY_SELECTOR):
        ctx.set_spgemm_policy(policy)
        B = locked(ctx, n, n, r, c, v)
        assert 0 <= B.spgemm_selected(B) < len(VARIANTS)
        assert_csr_equal(B.spgemm(B).download(), oracle.spgemm(B.download(), B.download()))
    ctx.set_spgemm_policy(sg.POLICY_SELECTOR)


def test_spgemm_errors(ctx):
    A = locked(ctx, 3, 4, np.array([0], np.uint32), np.array([1], np.uint32), np.array([1.0]))
    B = sg.Csr(ctx, 3, 3)
    with pytest.raises(sg.InvalidArgument):
        A.spgemm(B)
    B2 = sg.Csr(ctx, 4, 2)
    with pytest.raises(sg.LogicError):
        A.spgemm(B2)
    with pytest.raises(sg.LogicError):
        sg.Csr(ctx, 2, 2).transpose()


def test_spgemm_transpose_laplacian_3a_full(ctx):
    """3D 7-point Laplacian on 100^3: C = A*A and A^T, bit-exact."""
    r, c, v = gen.laplacian_3d(100)
    n = 100 ** 3
    A = locked(ctx, n, n, r, c, v)
    assert A.nnz == 6_940_000
    H = A.download()
    ref = oracle.spgemm(H, H)
    assert ref.cols.size <= 24_581_200
    for v in VARIANTS:
        assert_csr_equal(A.spgemm(A, v).download(), ref)
    assert_csr_equal(A.transpose().download(), oracle.transpose(H))


def test_spgemm_transpose_uniform_3b_full(ctx):
    """200 000^2 with 8 uniform columns per row: C = A*A and A^T, bit-exact."""
    n = 200_000
    r, c, v = gen.uniform_rows(n, n, 8, seed=77)
    A = locked(ctx, n, n, r, c, v)
    H = A.download()
    ref = oracle.spgemm(H, H)
    for v in VARIANTS:
        assert_csr_equal(A.spgemm(A, v).download(), ref)
    assert_csr_equal(A.transpose().download(), oracle.transpose(H))
