"""Regenerate the golden fixtures in tests/golden/ by running Spira itself.

Spira is compiled from its own sources by oracle/Makefile (target `ref`) into
oracle/_ref/libspira_ref.so; this script drives it through its public API
(matrix insert/lock/open, serial spmv through sparse_dot_double, spgemm,
transpose) on
  * known-answer cases taken from Spira's own tests (the file:line each case
    restates is recorded with it), and
  * seeded synthetic workloads (spira_gb300.gen), stored as sha256 digests of
    the CSR plus the SpMV output vector.
The fixtures are what the tests compare the oracle and the GPU engine with on
machines where Spira's sources are absent.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import platform
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from spira_gb300 import gen  # noqa: E402

# (name, source, n_rows, n_cols, epochs [[(r, c, v), ...], ...], x or None)
KATS = [
    ("spmv_rect_out_of_order", "tests/serial/spmv_tests.cpp:141-187", 3, 5,
     [[(0, 0, 1.0), (0, 3, 2.0), (1, 2, 3.0), (2, 4, 5.0), (2, 1, 4.0)]], [1.0, 2.0, 3.0, 4.0, 5.0]),
    ("spmv_mixed_last_write_wins", "tests/serial/spmv_tests.cpp:189-237", 5, 6,
     [[(0, 1, 2.0), (0, 4, -1.0), (1, 0, 3.5), (2, 5, 7.0), (3, 2, 1.25), (3, 2, 4.0), (4, 3, -2.0)]],
     [1.0, 2.0, 3.0, 4.0, 5.0, 6.0]),
    ("spmv_empty_matrix", "tests/serial/spmv_tests.cpp:239-269", 4, 5, [[]], [3.14] * 5),
    ("lock_last_write_wins", "tests/flush_behaviour_tests.cpp:17-31", 1, 10,
     [[(0, 3, 3.0), (0, 1, 1.0), (0, 1, 9.0)]], None),
    ("lock_last_write_wins_soa", "tests/flush_behaviour_tests.cpp:33-52", 1, 10,
     [[(0, 1, 1.0), (0, 2, 2.0), (0, 3, 3.0), (0, 4, 4.0), (0, 1, 5.0)]], None),
    ("merge_slab_preserved", "tests/flush_behaviour_tests.cpp:96-137", 1, 10,
     [[(0, 3, 4.0), (0, 5, 99.0)], [(0, 9, 7.0)]], None),
    ("merge_buffer_overwrites_slab", "tests/flush_behaviour_tests.cpp:140-176", 1, 10,
     [[(0, 5, 2.0)], [(0, 5, 99.0)]], None),
    ("lock_zero_filtered", "tests/flush_behaviour_tests.cpp:178-210", 1, 10,
     [[(0, 1, 5.0), (0, 2, 0.0)]], None),
    ("merge_zero_deletes", "tests/flush_behaviour_tests.cpp:211-232", 1, 10,
     [[(0, 3, 7.0)], [(0, 3, 0.0)]], None),
    ("merge_zero_deletes_one_of_two", "tests/flush_behaviour_tests.cpp:234-253", 1, 10,
     [[(0, 5, 3.0), (0, 6, 4.0)], [(0, 5, 0.0)]], None),
    ("merge_zero_deletes_all", "tests/flush_behaviour_tests.cpp:255-276", 2, 10,
     [[(0, 1, 1.0), (0, 2, 2.0), (1, 3, 3.0)], [(0, 1, 0.0), (0, 2, 0.0), (1, 3, 0.0)]], None),
    ("build_offsets_cols_vals", "tests/compaction_tests.cpp:71-100", 3, 5,
     [[(0, 0, 1.0), (0, 3, 2.0), (1, 1, 3.0), (2, 2, 4.0)]], None),
    ("build_first_last_rows_empty", "tests/compaction_tests.cpp:102-125", 3, 5,
     [[(1, 0, 9.0), (1, 4, 8.0)]], None),
    ("build_cols_sorted", "tests/compaction_tests.cpp:127-141", 1, 6,
     [[(0, 4, 4.0), (0, 1, 1.0), (0, 2, 2.0)]], None),
    ("build_zero_rows", "tests/compaction_tests.cpp:143-152", 0, 5, [[]], None),
]

SPGEMM_KATS = [
    ("spgemm_small_example", "tests/serial/spgemm_tests.cpp:130-151",
     (2, 3, [(0, 0, 1.0), (0, 2, 2.0), (1, 1, 3.0)]), (3, 2, [(0, 1, 4.0), (1, 0, 5.0), (2, 1, 6.0)])),
    ("spgemm_rectangular", "tests/serial/spgemm_tests.cpp:153-163",
     (4, 3, [(0, 0, 1.0), (0, 2, 2.0), (2, 1, 3.0), (3, 0, 4.0)]),
     (3, 5, [(0, 1, 7.0), (0, 4, 1.0), (1, 2, 2.0), (2, 1, 3.0), (2, 3, 5.0)])),
    ("spgemm_accumulates", "tests/serial/spgemm_tests.cpp:189-202",
     (1, 3, [(0, 0, 1.0), (0, 1, 1.0), (0, 2, 1.0)]), (3, 1, [(0, 0, 2.0), (1, 0, 3.0), (2, 0, 4.0)])),
    ("spgemm_double", "tests/serial/spgemm_tests.cpp:205-214",
     (2, 2, [(0, 0, 0.5), (1, 1, 2.0)]), (2, 2, [(0, 1, 4.0), (1, 0, -1.5)])),
    ("spgemm_cancellation_drops_zero", "spgemm.hpp:42-48 (v != V{})",
     (1, 2, [(0, 0, 1.0), (0, 1, 1.0)]), (2, 2, [(0, 0, 2.0), (0, 1, 3.0), (1, 0, -2.0)])),
]

TRANSPOSE_KATS = [
    ("transpose_empty", "tests/serial/transpose_tests.cpp:42-60", (3, 5, [])),
    ("transpose_single", "tests/serial/transpose_tests.cpp:62-74", (4, 6, [(2, 5, 7.5)])),
    ("transpose_multiple", "tests/serial/transpose_tests.cpp:76-100",
     (3, 4, [(0, 0, 1.0), (0, 3, 2.0), (2, 1, 3.0)])),
]


def _csr_json(A):
    return {"n_rows": int(A.n_rows), "n_cols": int(A.n_cols), "off": [int(v) for v in A.off],
            "cols": [int(v) for v in A.cols], "vals": [float(v).hex() for v in A.vals], "capacity": int(A.capacity)}


def _epochs(ep):
    out = []
    for e in ep:
        if e:
            r, c, v = zip(*e)
        else:
            r, c, v = (), (), ()
        out.append((np.array(r, np.uint32), np.array(c, np.uint32), np.array(v, np.float64)))
    return out


def _lock(n_rows, n_cols, triples):
    return oracle.ref_lock_epochs(n_rows, n_cols, _epochs([triples]), layout=1)


def workloads():
    """Seeded synthetic cases: (name, n_rows, n_cols, epochs, x)."""
    out = []
    r, c, v = gen.random_rows(10_000, 10_000, 10, seed=42)
    out.append(("random_10k_10_per_row", 10_000, 10_000, [(r, c, v)], gen.dense_x(10_000, 7)))
    # Stress in the shape of tests/large_matrix_stress_tests.cpp:12-90:
    # 10k x 10k, 100k inserts, integer values in [-10, 10] (about 1/21 zeros
    # = deletes), the second half overwriting keys of the first half.
    m = 100_000
    ctr = np.arange(m, dtype=np.uint64)
    rr = gen.below(gen.hash3(43, 1, ctr), 10_000)
    cc = gen.below(gen.hash3(43, 2, ctr), 10_000)
    vv = (gen.below(gen.hash3(43, 3, ctr), 21).astype(np.int64) - 10).astype(np.float64)
    half = m // 2
    pick = gen.below(gen.hash3(43, 4, ctr[half:]), half)
    rr[half:] = np.where(ctr[half:] % 2 == 0, rr[pick], rr[half:])
    cc[half:] = np.where(ctr[half:] % 2 == 0, cc[pick], cc[half:])
    out.append(("stress_10k_100k_inserts", 10_000, 10_000,
                [(rr[:half], cc[:half], vv[:half]), (rr[half:], cc[half:], vv[half:])], gen.dense_x(10_000, 8)))
    # Laplacian 2D, small grid, then a re-lock of 1% of nnz over 10% of rows
    r, c, v = gen.laplacian_2d(300)
    nnz = len(r)
    b = gen.relock_batch(300 * 300, 300 * 300, nnz, seed=44, zero_frac=0.1)
    out.append(("laplacian2d_300_relock", 90_000, 90_000, [(r, c, v), b], gen.dense_x(90_000, 9)))
    # Zipf rows, small
    r, c, v = gen.zipf_rows(50_000, seed=45)
    out.append(("zipf_50k", 50_000, 50_000, [(r, c, v)], gen.dense_x(50_000, 10)))
    return out


def main():
    oracle.build()
    assert oracle.ref_available(), "Spira's sources are needed to build oracle/_ref"
    doc = {"generator": "tests/golden/make_golden.py", "host": platform.machine(),
           "spira_flags": "-std=gnu++23 -O3 -DNDEBUG; dot_avx512.cpp -mavx512f -mavx512vl -mavx512bw -mavx512dq",
           "kats": [], "spgemm": [], "transpose": [], "workloads": []}
    for name, src, nr, nc, ep, x in KATS:
        A = oracle.ref_lock_epochs(nr, nc, _epochs(ep), layout=1)
        rec = {"name": name, "source": src, "n_rows": nr, "n_cols": nc,
               "epochs": [[[int(t[0]), int(t[1]), float(t[2]).hex()] for t in e] for e in ep],
               "csr": _csr_json(A)}
        if x is not None:
            y = oracle.ref_spmv(A, np.array(x, np.float64), mode=0)
            rec["x"] = [float(v).hex() for v in x]
            rec["y"] = [float(v).hex() for v in y]
        doc["kats"].append(rec)
    for name, src, (ar, ac, at), (br, bc, bt) in SPGEMM_KATS:
        A, B = _lock(ar, ac, at), _lock(br, bc, bt)
        Cm = oracle.ref_spgemm(A, B)
        doc["spgemm"].append({"name": name, "source": src, "A": _csr_json(A), "B": _csr_json(B), "C": _csr_json(Cm)})
    for name, src, (nr, nc, t) in TRANSPOSE_KATS:
        A = _lock(nr, nc, t)
        T = oracle.ref_transpose(A)
        doc["transpose"].append({"name": name, "source": src, "A": _csr_json(A), "T": _csr_json(T)})
    arrays = {}
    for name, nr, nc, ep, x in workloads():
        A = oracle.ref_lock_epochs(nr, nc, ep, layout=1)
        y = oracle.ref_spmv(A, x, mode=0)
        rec = {"name": name, "n_rows": nr, "n_cols": nc, "nnz": int(len(A.cols)), "capacity": int(A.capacity),
               "csr_sha256": oracle.csr_digest(A)}
        if nr == nc and len(A.cols) <= 200_000:
            At = oracle.ref_transpose(A)
            rec["transpose_sha256"] = oracle.csr_digest(At)
            Cm = oracle.ref_spgemm(A, A)
            rec["spgemm_sha256"] = oracle.csr_digest(Cm)
            rec["spgemm_nnz"] = int(len(Cm.cols))
        arrays[name + "__y"] = y
        doc["workloads"].append(rec)
    (HERE / "golden.json").write_text(json.dumps(doc, indent=1))
    np.savez_compressed(HERE / "golden_y.npz", **arrays)
    print("wrote", HERE / "golden.json", HERE / "golden_y.npz")


if __name__ == "__main__":
    main()
