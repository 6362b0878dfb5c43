"""Binary CSR files on the GPU: save / load round trips are bit-exact, files
written by an independent numpy writer load, and corrupt or malformed files
are refused with the matrix left unchanged."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import spira_gb300 as sg
from spira_gb300 import gen
from conftest import assert_csr_equal
import csr_file

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["zipf", "empty", "one_row", "zeros_nan", "odd_nnz"])
def test_round_trip(ctx, tmp_path, kind):
    if kind == "zipf":
        r, c, v = gen.zipf_rows(300_000, seed=41)
        H = oracle.lock_epochs(300_000, 300_000, [(r, c, v)])
    elif kind == "empty":
        H = oracle.lock_epochs(1000, 700, [])
    elif kind == "one_row":
        H = oracle.lock_epochs(1, 10, [(np.zeros(3, np.uint32), np.array([9, 0, 4], np.uint32), np.array([1., 2., 3.]))])
    elif kind == "zeros_nan":
        r, c, v = gen.uniform_rows(5000, 5000, 7, seed=42)
        H = oracle.lock_epochs(5000, 5000, [(r, c, v)])
        H.vals[::11] = 0.0
        H.vals[3::13] = np.nan
    else:
        H = oracle.lock_epochs(3, 3, [(np.array([0, 1, 2], np.uint32), np.array([0, 1, 2], np.uint32),
                                       np.array([1.0, 2.0, 3.0]))])
    A = sg.Csr(ctx, H.n_rows, H.n_cols)
    A.load(H.off, H.cols, H.vals)
    p = tmp_path / "m.spgcsr"
    A.save(p)
    assert sg.csr_file_info(p) == (H.n_rows, H.n_cols, len(H.cols))
    B = sg.Csr(ctx, 1, 1).load_file(p)
    assert_csr_equal(B.download(), A.download())
    # the numpy writer makes the same bytes
    q = tmp_path / "n.spgcsr"
    csr_file.write(q, H.n_rows, H.n_cols, H.off, H.cols, H.vals, flags=int(kind == "zeros_nan"))
    assert q.read_bytes() == p.read_bytes()


def test_refusals_leave_the_matrix_unchanged(ctx, tmp_path):
    r, c, v = gen.uniform_rows(2000, 2000, 5, seed=43)
    H = oracle.lock_epochs(2000, 2000, [(r, c, v)])
    keep = sg.Csr(ctx, 4, 4)
    keep.load(np.array([0, 1, 1, 1, 2], np.uint64), np.array([2, 3], np.uint32), np.array([5.0, 6.0]))
    before = keep.download()
    p = tmp_path / "x.spgcsr"
    # a flipped value bit: checksum mismatch
    csr_file.write(p, H.n_rows, H.n_cols, H.off, H.cols, H.vals)
    raw = bytearray(p.read_bytes())
    raw[-3] ^= 0x10
    p.write_bytes(bytes(raw))
    with pytest.raises(sg.InvalidArgument, match="checksum"):
        keep.load_file(p)
    # consistent checksums over broken CSRs
    bad_cols = H.cols.copy()
    bad_cols[1], bad_cols[0] = H.cols[0], H.cols[1]  # row 0 not ascending
    csr_file.write(p, H.n_rows, H.n_cols, H.off, bad_cols, H.vals)
    with pytest.raises(sg.InvalidArgument, match="strictly sorted"):
        keep.load_file(p)
    oob = H.cols.copy()
    oob[5] = H.n_cols
    csr_file.write(p, H.n_rows, H.n_cols, H.off, oob, H.vals)
    with pytest.raises(sg.InvalidArgument, match="out of bounds"):
        keep.load_file(p)
    off = H.off.copy()
    off[10], off[11] = off[11], off[10]
    csr_file.write(p, H.n_rows, H.n_cols, off, H.cols, H.vals)
    with pytest.raises(sg.InvalidArgument, match="non-decreasing"):
        keep.load_file(p)
    off = H.off.copy()
    off[0] = 1
    csr_file.write(p, H.n_rows, H.n_cols, off, H.cols, H.vals)
    with pytest.raises(sg.InvalidArgument, match="offsets\\[0\\]"):
        keep.load_file(p)
    assert_csr_equal(keep.download(), before)
    with pytest.raises(sg.LogicError):
        sg.Csr(ctx, 3, 3).save(tmp_path / "unlocked.spgcsr")
