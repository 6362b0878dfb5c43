"""Pin the oracle before trusting it: against Spira's own outputs in the
committed golden fixtures (always) and against Spira compiled from its
sources in oracle/_ref (where Spira's source tree is present)."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from spira_gb300 import gen
from conftest import assert_csr_equal

GOLD = json.loads((Path(__file__).parent / "golden" / "golden.json").read_text())
GOLD_Y = np.load(Path(__file__).parent / "golden" / "golden_y.npz")


def _csr(d):
    return oracle.Csr(d["n_rows"], d["n_cols"], np.array(d["off"], np.uint64), np.array(d["cols"], np.uint32),
                      np.array([float.fromhex(v) for v in d["vals"]], np.float64), d["capacity"])


def _epochs(ep):
    out = []
    for e in ep:
        r = np.array([t[0] for t in e], np.uint32)
        c = np.array([t[1] for t in e], np.uint32)
        v = np.array([float.fromhex(t[2]) for t in e], np.float64)
        out.append((r, c, v))
    return out


@pytest.mark.parametrize("kat", GOLD["kats"], ids=[k["name"] for k in GOLD["kats"]])
def test_oracle_lock_matches_spira_kats(kat):
    A = oracle.lock_epochs(kat["n_rows"], kat["n_cols"], _epochs(kat["epochs"]))
    assert_csr_equal(A, _csr(kat["csr"]))
    if "y" in kat:
        x = np.array([float.fromhex(v) for v in kat["x"]])
        y = oracle.spmv_blocked(A, x, lanes=8, tail_fused=0)
        np.testing.assert_array_equal(y, np.array([float.fromhex(v) for v in kat["y"]]))


def test_kat_expected_values_from_spira_tests():
    """The assertions Spira's own tests make on these cases."""
    k = {d["name"]: d for d in GOLD["kats"]}
    y = [float.fromhex(v) for v in k["spmv_rect_out_of_order"]["y"]]
    assert y == [9.0, 9.0, 33.0]  # tests/serial/spmv_tests.cpp:161
    assert k["build_offsets_cols_vals"]["csr"]["off"] == [0, 2, 3, 4]  # tests/compaction_tests.cpp:86-89
    assert k["build_first_last_rows_empty"]["csr"]["off"] == [0, 0, 2, 2]
    assert k["merge_zero_deletes_all"]["csr"]["off"] == [0, 0, 0]
    s = {d["name"]: d for d in GOLD["spgemm"]}
    C = _csr(s["spgemm_small_example"]["C"])  # C(0,1)=16, C(1,0)=15 (spgemm_tests.cpp:144-147)
    assert list(C.off) == [0, 1, 2] and list(C.cols) == [1, 0] and list(C.vals) == [16.0, 15.0]


@pytest.mark.parametrize("case", GOLD["spgemm"], ids=[k["name"] for k in GOLD["spgemm"]])
def test_oracle_spgemm_matches_spira(case):
    Cm = oracle.spgemm(_csr(case["A"]), _csr(case["B"]), fused=False)
    assert_csr_equal(Cm, _csr(case["C"]))


@pytest.mark.parametrize("case", GOLD["transpose"], ids=[k["name"] for k in GOLD["transpose"]])
def test_oracle_transpose_matches_spira(case):
    assert_csr_equal(oracle.transpose(_csr(case["A"])), _csr(case["T"]))


def _workloads():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", Path(__file__).parent / "golden" / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return {w[0]: w for w in mg.workloads()}


WL = None


@pytest.mark.parametrize("rec", GOLD["workloads"], ids=[w["name"] for w in GOLD["workloads"]])
def test_oracle_workloads_match_spira_digests(rec):
    global WL
    if WL is None:
        WL = _workloads()
    name, nr, nc, ep, x = WL[rec["name"]]
    A = oracle.lock_epochs(nr, nc, ep)
    assert len(A.cols) == rec["nnz"] and A.capacity == rec["capacity"]
    assert oracle.csr_digest(A) == rec["csr_sha256"]
    y = oracle.spmv_blocked(A, x, lanes=8, tail_fused=0)
    np.testing.assert_array_equal(y, GOLD_Y[rec["name"] + "__y"])
    if "transpose_sha256" in rec:
        assert oracle.csr_digest(oracle.transpose(A)) == rec["transpose_sha256"]
        Cm = oracle.spgemm(A, A, fused=False)
        assert len(Cm.cols) == rec["spgemm_nnz"]
        assert oracle.csr_digest(Cm) == rec["spgemm_sha256"]


def test_compensated_oracle_is_tight():
    r, c, v = gen.random_rows(2000, 2000, 30, seed=3)
    A = oracle.lock_epochs(2000, 2000, [(r, c, v)])
    x = gen.dense_x(2000, 4)
    y, sc = oracle.spmv_compensated(A, x)
    # exact reference through Python's correctly rounded fsum over products
    import math
    for row in range(0, 2000, 97):
        b, e = int(A.off[row]), int(A.off[row + 1])
        from fractions import Fraction
        exact = sum(Fraction(float(A.vals[k])) * Fraction(float(x[A.cols[k]])) for k in range(b, e))
        assert abs(Fraction(y[row]) - exact) <= Fraction(2.3e-16) * Fraction(sc[row])


needs_ref = pytest.mark.skipif(not oracle.ref_available(), reason="Spira sources not present (oracle/_ref)")


@needs_ref
@pytest.mark.parametrize("layout", [0, 1, 2])
def test_oracle_lock_matches_spira_random_epochs(layout):
    n = 1500
    rng_eps = []
    for e in range(4):
        ctr = np.arange(4000, dtype=np.uint64)
        r = gen.below(gen.hash3(90 + e, 1, ctr), n)
        c = gen.below(gen.hash3(90 + e, 2, ctr), n)
        v = (gen.below(gen.hash3(90 + e, 3, ctr), 7).astype(np.int64) - 3).astype(np.float64)
        v[::13] = -0.0
        v[::29] = np.nan
        rng_eps.append((r, c, v))
    A = oracle.lock_epochs(n, n, rng_eps)
    R = oracle.ref_lock_epochs(n, n, rng_eps, layout=layout, n_threads=3)
    assert_csr_equal(A, R, check_capacity=(layout != 2))


@needs_ref
@pytest.mark.parametrize("n_threads", [1, 2, 3, 4])
def test_oracle_parallel_spmv_matches_spira(n_threads):
    r, c, v = gen.zipf_rows(20_000, seed=5)
    A = oracle.lock_epochs(20_000, 20_000, [(r, c, v)])
    x = gen.dense_x(20_000, 6)
    y_ref = oracle.ref_spmv(A, x, mode=2, n_threads=n_threads)
    y = oracle.spmv_parallel(A, x, n_threads, lanes=8, tail_fused=0)
    np.testing.assert_array_equal(y, y_ref)


@needs_ref
def test_oracle_spgemm_transpose_parallel_match_spira():
    r, c, v = gen.uniform_rows(3000, 3000, 8, seed=7)
    A = oracle.lock_epochs(3000, 3000, [(r, c, v)])
    for par in (False, True):
        assert_csr_equal(oracle.spgemm(A, A), oracle.ref_spgemm(A, A, parallel=par, n_threads=3),
                         check_capacity=not par)
        assert_csr_equal(oracle.transpose(A), oracle.ref_transpose(A, parallel=par, n_threads=3),
                         check_capacity=not par)


def _ops_pair(n=2500, seed=11):
    """A and B with shared positions, exact cancellations on some of them and
    explicit zeros (as load_csr may install) in A."""
    ra, ca, va = gen.uniform_rows(n, n, 6, seed=seed)
    A = oracle.lock_epochs(n, n, [(ra, ca, va)])
    rb, cb, vb = gen.uniform_rows(n, n, 4, seed=seed + 1)
    # B also holds every third entry of A, negated on half of them (sum +-0)
    k = np.arange(0, len(A.cols), 3)
    rows_a = np.repeat(np.arange(n, dtype=np.uint32), np.diff(A.off).astype(np.int64))
    sv = np.where(np.arange(len(k)) % 2 == 0, -A.vals[k], 0.5 * A.vals[k])
    B = oracle.lock_epochs(n, n, [(np.concatenate([rb, rows_a[k]]), np.concatenate([cb, A.cols[k]]),
                                   np.concatenate([vb, sv]))])
    Az = oracle.Csr(A.n_rows, A.n_cols, A.off.copy(), A.cols.copy(), A.vals.copy(), A.capacity)
    Az.vals[1::17] = 0.0
    Az.vals[2::23] = -0.0
    Az.vals[5::31] = np.nan
    return Az, B


@needs_ref
def test_oracle_add_matches_spira():
    A, B = _ops_pair()
    got = oracle.add(A, B)
    assert_csr_equal(got, oracle.ref_add(A, B))
    assert_csr_equal(got, oracle.ref_add(A, B, parallel=True, n_threads=3), check_capacity=False)
    assert_csr_equal(oracle.add(B, A), oracle.ref_add(B, A))
    with pytest.raises(ValueError):
        oracle.ref_add(A, oracle.lock_epochs(10, 10, []))


@needs_ref
@pytest.mark.parametrize("s,divide", [(2.5, False), (-3.0, False), (0.0, False), (1e-310, False), (np.nan, False),
                                      (3.0, True), (1e300, True), (-0.125, True)])
def test_oracle_scale_matches_spira(s, divide):
    A, _ = _ops_pair(seed=21)
    got = oracle.scale(A, s, divide)
    assert_csr_equal(got, oracle.ref_scale(A, s, divide))


@needs_ref
def test_spira_in_place_scale_is_lost_at_lock():
    """Spira's in-place scalers (serial/scalars.hpp:10-18, 37-49) insert the
    scaled values through row::insert, which leaves the matrix's dirty flags
    unset; the next lock() copies every clean row's old slice
    (csr_build.hpp:190-215), so the values come back unscaled. Only the
    capacity moves, by the merge rule over the buffered entries: kept while
    2 nnz fits, else 1.5 x 2 nnz. Recorded here because libspg's in-place
    scale installs the scaled values instead."""
    A, _ = _ops_pair(seed=21)
    m = len(A.cols)
    for s, divide in ((2.5, False), (3.0, True)):
        ip = oracle.ref_scale(A, s, divide, in_place=True)
        assert_csr_equal(ip, A, check_capacity=False)
        assert ip.capacity == (A.capacity if 2 * m <= A.capacity else 3 * m)


@needs_ref
def test_oracle_division_by_zero_is_a_domain_error():
    A, _ = _ops_pair(n=50)
    for z in (0.0, -0.0):
        with pytest.raises(ArithmeticError):
            oracle.ref_scale(A, z, divide=True)


@needs_ref
def test_oracle_row_sums_match_spira():
    r, c, v = gen.zipf_rows(20_000, seed=23)
    A = oracle.lock_epochs(20_000, 20_000, [(r, c, v)])
    np.testing.assert_array_equal(oracle.row_sums(A).view(np.uint64), oracle.ref_row_sums(A).view(np.uint64))


@needs_ref
@pytest.mark.parametrize("T", [1, 2, 3, 7, 64, 5000])
def test_oracle_partition_matches_spira(T):
    r, c, v = gen.zipf_rows(3000, seed=24)
    A = oracle.lock_epochs(3000, 3000, [(r, c, v)])
    np.testing.assert_array_equal(oracle.partition(A, T), oracle.ref_partition(A, T))
    E = oracle.lock_epochs(100, 100, [])  # nnz == 0: uniform split
    np.testing.assert_array_equal(oracle.partition(E, T), oracle.ref_partition(E, T))
    few = oracle.lock_epochs(100, 100, [(np.array([99], np.uint32), np.array([0], np.uint32), np.array([1.0]))])
    np.testing.assert_array_equal(oracle.partition(few, T), oracle.ref_partition(few, T))
