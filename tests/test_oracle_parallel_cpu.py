"""The oracle's parallel forms (the multi-core CPU baseline of lock, SpGEMM
and transpose) give exactly the serial oracle's results, which are pinned to
Spira: parallel_matrix's t*n/T partitions change who computes a row, never
what it holds."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from spira_gb300 import gen


@pytest.mark.parametrize("threads", [1, 3, 8])
def test_parallel_spgemm_and_transpose_equal_serial(threads):
    r, c, v = gen.zipf_rows(4000, seed=9)
    A = oracle.lock_epochs(4000, 4000, [(r, c, v)])
    assert oracle.csr_digest(oracle.spgemm_parallel(A, A, threads)) == oracle.csr_digest(oracle.spgemm(A, A))
    assert oracle.csr_digest(oracle.spgemm_parallel(A, A, threads, fused=True)) == \
        oracle.csr_digest(oracle.spgemm(A, A, fused=True))
    assert oracle.csr_digest(oracle.transpose_parallel(A, threads)) == oracle.csr_digest(oracle.transpose(A))


@pytest.mark.parametrize("threads", [1, 4, 7])
def test_parallel_lock_counts_equal_serial(threads):
    n = 5000
    r, c, v = gen.random_rows(n, n, 6, seed=4)
    d = gen.relock_batch(n, n, len(r), seed=5)
    secs, nnz = oracle.lock_parallel_time(n, n, [(r, c, v), d], threads)
    assert len(secs) == 2 and np.all(secs >= 0)
    assert nnz == len(oracle.lock_epochs(n, n, [(r, c, v), d]).cols)


def test_parallel_lock_rejects_out_of_range():
    with pytest.raises(IndexError):
        oracle.lock_parallel_time(10, 10, [(np.array([10], np.uint32), np.array([0], np.uint32), np.ones(1))], 2)
