"""Shared fixtures. Tests marked `gpu` need a GB300 and libspg.so; the rest
run on any CPU (the oracle, the golden fixtures, host-side logic and the C ABI
surface without compute calls)."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built libspg.so")


@pytest.fixture(scope="session")
def ctx():
    import spira_gb300 as sg

    c = sg.Context(0)
    yield c
    c.close()


def assert_csr_equal(got, ref, check_capacity=True):
    """Bit-exact structure and value bits."""
    assert got.n_rows == ref.n_rows and got.n_cols == ref.n_cols
    np.testing.assert_array_equal(np.asarray(got.off, np.uint64), np.asarray(ref.off, np.uint64))
    np.testing.assert_array_equal(np.asarray(got.cols, np.uint32), np.asarray(ref.cols, np.uint32))
    np.testing.assert_array_equal(np.asarray(got.vals, np.float64).view(np.uint64),
                                  np.asarray(ref.vals, np.float64).view(np.uint64))
    if check_capacity:
        assert got.capacity == ref.capacity


# FP64 SpMV parity bound: |y - y_ref| <= TOL * sum_k |a_rk x_k| per row.
SPMV_TOL = 1e-12


def spmv_rel_err(y, y_ref, scale):
    y, y_ref = np.asarray(y), np.asarray(y_ref)
    d = np.abs(y - y_ref)
    s = np.where(scale > 0, scale, 1.0)
    e = d / s
    # rows with no entries must be exactly zero
    e = np.where(scale > 0, e, np.where(d == 0, 0.0, np.inf))
    return float(e.max()) if len(e) else 0.0
