"""Failure detection without a GPU fault: the one kind of kernel that waits
(SpGEMM's ordered scan of tile counts) bounds every wait. The self-test runs
that wait against a predecessor that never publishes (a flag nothing sets)
with a ~10 ms bound: the kernel must give up and return, the context must
report SPG_ERR_DEVICE_TIMEOUT once, and then keep working."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle
import spira_gb300 as sg
from spira_gb300 import gen
from conftest import assert_csr_equal

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_context_stays_usable():
    ctx = sg.Context(0)
    gave_up = C.c_int(0)
    sg._check(sg.lib().spg_selftest_wait_timeout(ctx.h, 20_000_000, C.byref(gave_up)))
    assert gave_up.value == 1
    with pytest.raises(sg.DeviceTimeout):
        ctx.sync()
    ctx.sync()  # reported once, then cleared
    n = 3000
    r, c, v = gen.uniform_rows(n, n, 6, seed=2)
    A = sg.Csr(ctx, n, n)
    A.lock(r, c, v)
    H = A.download()
    assert_csr_equal(A.spgemm(A, sg.SPGEMM_VARIANTS["warpsort_64"]).download(), oracle.spgemm(H, H))
    ctx.close()


def test_selftest_rejects_unbounded_waits():
    ctx = sg.Context(0)
    gave_up = C.c_int(0)
    assert sg.lib().spg_selftest_wait_timeout(ctx.h, 0, C.byref(gave_up)) == 1
    assert sg.lib().spg_selftest_wait_timeout(ctx.h, 1 << 40, C.byref(gave_up)) == 1
    ctx.close()
