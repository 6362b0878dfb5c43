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


@pytest.mark.parametrize("case", GOLD["spgemm"], ids=[k["name"] for k in GOLD["spgemm"]])
def test_spgemm_kats(ctx, case):
    Cm = dev(ctx, _gold_csr(case["A"])).spgemm(dev(ctx, _gold_csr(case["B"])))
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
    Cm = A.spgemm(A)
    assert Cm.nnz == rec["spgemm_nnz"]
    assert oracle.csr_digest(Cm.download()) == rec["spgemm_sha256"]


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


def test_spgemm_cancellation_and_rectangular(ctx):
    # integer values: exact products, cancellations produce exact zeros to drop
    ctr = np.arange(60_000, dtype=np.uint64)
    r = gen.below(gen.hash3(2, 1, ctr), 3000)
    c = gen.below(gen.hash3(2, 2, ctr), 500)
    v = (gen.below(gen.hash3(2, 3, ctr), 5).astype(np.int64) - 2).astype(np.float64)
    A = locked(ctx, 3000, 500, r, c, v)
    ctr2 = np.arange(20_000, dtype=np.uint64)
    B = locked(ctx, 500, 4000, gen.below(gen.hash3(3, 1, ctr2), 500), gen.below(gen.hash3(3, 2, ctr2), 4000),
               (gen.below(gen.hash3(3, 3, ctr2), 5).astype(np.int64) - 2).astype(np.float64))
    Cm = A.spgemm(B)
    assert_csr_equal(Cm.download(), oracle.spgemm(A.download(), B.download()))


def test_spgemm_every_row_class(ctx):
    """Rows for each SpGEMM path: merge with <= 8 A entries, merge with 9..32,
    expand-sort for > 32 entries and for > 4096 products; exact cancellations
    (integer values) included. Bit-exact against the oracle."""
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
    Cm = A.spgemm(A)
    assert_csr_equal(Cm.download(), oracle.spgemm(H, H))


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
    Cm = A.spgemm(A)
    assert Cm.nnz <= 24_581_200
    assert_csr_equal(Cm.download(), oracle.spgemm(H, H))
    assert_csr_equal(A.transpose().download(), oracle.transpose(H))


def test_spgemm_transpose_uniform_3b_full(ctx):
    """200 000^2 with 8 uniform columns per row: C = A*A and A^T, bit-exact."""
    n = 200_000
    r, c, v = gen.uniform_rows(n, n, 8, seed=77)
    A = locked(ctx, n, n, r, c, v)
    H = A.download()
    Cm = A.spgemm(A)
    assert_csr_equal(Cm.download(), oracle.spgemm(H, H))
    assert_csr_equal(A.transpose().download(), oracle.transpose(H))
