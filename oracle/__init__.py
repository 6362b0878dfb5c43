"""The oracle: CPU restatement of Spira's hot path (spira_oracle.c) and, where
the Spira source tree is present, Spira itself compiled from its sources
(oracle/_ref/libspira_ref.so via oracle/Makefile).

TEST INFRASTRUCTURE ONLY. Imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline / reference arm as the reference results and the
CPU baseline; never by the product (spira_gb300), which has no CPU path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from collections import namedtuple
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "_build" / "liboracle.so"
REF_SO = HERE / "_ref" / "libspira_ref.so"
# The Spira source tree to compile the reference from: $SPIRA_REF, no default.


def ref_src() -> Path | None:
    p = os.environ.get("SPIRA_REF")
    return Path(p) if p else None

Csr = namedtuple("Csr", "n_rows n_cols off cols vals capacity")


class _OrcCsr(C.Structure):
    _fields_ = [("n_rows", C.c_uint64), ("n_cols", C.c_uint64), ("nnz", C.c_uint64), ("capacity", C.c_uint64),
                ("off", C.POINTER(C.c_uint64)), ("cols", C.POINTER(C.c_uint32)), ("vals", C.POINTER(C.c_double))]


def build(ref: bool | None = None) -> None:
    """Compile liboracle.so; and Spira itself when its sources are here."""
    subprocess.run(["make", "-s", "-C", str(HERE), "liboracle"], check=True)
    src = ref_src()
    if ref is None:
        ref = src is not None and (src / "include" / "spira" / "spira.hpp").exists()
    if ref:
        if src is None:
            raise RuntimeError("SPIRA_REF must name the Spira source tree to build the reference")
        subprocess.run(["make", "-s", "-j8", "-C", str(HERE), "ref", f"REF={src}"], check=True)


_orc = None
_ref = None


def orc():
    global _orc
    if _orc is None:
        if not ORACLE_SO.exists():
            build(ref=False)
        _orc = C.CDLL(str(ORACLE_SO))
        P = C.POINTER(_OrcCsr)
        _orc.orc_lock.argtypes = [P, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64]
        _orc.orc_csr_free.argtypes = [P]
        for n in ("orc_spmv_scalar",):
            getattr(_orc, n).argtypes = [C.c_void_p] * 3 + [C.c_uint64, C.c_void_p, C.c_void_p, C.c_int]
        _orc.orc_spmv_blocked.argtypes = [C.c_void_p] * 3 + [C.c_uint64, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        _orc.orc_spmv_parallel.argtypes = [C.c_void_p] * 3 + [C.c_uint64, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                                              C.c_int]
        _orc.orc_spmv_compensated.argtypes = [C.c_void_p] * 3 + [C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p]
        _orc.orc_spgemm.argtypes = [P, P, P, C.c_int]
        _orc.orc_spgemm_products.argtypes = [P, P]
        _orc.orc_spgemm_products.restype = C.c_uint64
        _orc.orc_transpose.argtypes = [P, P]
        _orc.orc_spgemm_parallel.argtypes = [P, P, P, C.c_int, C.c_int]
        _orc.orc_transpose_parallel.argtypes = [P, P, C.c_int]
        _orc.orc_lock_parallel_time.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64)]
        _orc.orc_add.argtypes = [P, P, P]
        _orc.orc_scale.argtypes = [P, C.c_double, C.c_int, P]
        _orc.orc_row_sums.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]
        _orc.orc_partition.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_void_p]
    return _orc


def ref_available() -> bool:
    return REF_SO.exists()


def ref():
    global _ref
    if _ref is None:
        if not REF_SO.exists():
            raise RuntimeError("Spira reference library not built (needs the Spira source tree)")
        _ref = C.CDLL(str(REF_SO))
        P = C.POINTER(_OrcCsr)
        _ref.ref_last_error.restype = C.c_char_p
        _ref.ref_csr_free.argtypes = [P]
        _ref.ref_lock_epochs.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_uint64, C.c_int, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, P]
        _ref.ref_spmv.argtypes = [C.c_int, C.c_int, P, C.c_void_p, C.c_void_p]
        _ref.ref_spmv_parallel_time.argtypes = [C.c_int, P, C.c_void_p, C.c_void_p, C.c_int]
        _ref.ref_spmv_parallel_time.restype = C.c_double
        _ref.ref_spgemm.argtypes = [C.c_int, C.c_int, P, P, P]
        _ref.ref_transpose.argtypes = [C.c_int, C.c_int, P, P]
        _ref.ref_load_check.argtypes = [P]
        _ref.ref_add.argtypes = [C.c_int, C.c_int, P, P, P]
        _ref.ref_scale.argtypes = [C.c_int, C.c_int, P, C.c_double, P]
        _ref.ref_row_sums.argtypes = [P, C.c_void_p]
        _ref.ref_partition.argtypes = [P, C.c_uint64, C.c_void_p]
    return _ref


# ---------------------------------------------------------------- helpers
def _as_c(A) -> tuple[_OrcCsr, tuple]:
    off = np.ascontiguousarray(A.off, dtype=np.uint64)
    cols = np.ascontiguousarray(A.cols, dtype=np.uint32)
    vals = np.ascontiguousarray(A.vals, dtype=np.float64)
    s = _OrcCsr(A.n_rows, A.n_cols, len(cols), len(cols),
                off.ctypes.data_as(C.POINTER(C.c_uint64)), cols.ctypes.data_as(C.POINTER(C.c_uint32)),
                vals.ctypes.data_as(C.POINTER(C.c_double)))
    return s, (off, cols, vals)  # keep arrays alive


def _take(s: _OrcCsr, free) -> Csr:
    n, nnz = s.n_rows, s.nnz
    off = np.ctypeslib.as_array(s.off, shape=(n + 1,)).copy() if s.off else np.zeros(n + 1, np.uint64)
    cols = np.ctypeslib.as_array(s.cols, shape=(nnz,)).copy() if nnz else np.zeros(0, np.uint32)
    vals = np.ctypeslib.as_array(s.vals, shape=(nnz,)).copy() if nnz else np.zeros(0, np.float64)
    cap = s.capacity
    free(C.byref(s))
    return Csr(n, s.n_cols, off, cols, vals, cap)


def _arr(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


# ---------------------------------------------------------------- oracle API
def lock_epochs(n_rows: int, n_cols: int, epochs) -> Csr:
    """insert/lock/open cycles; epochs = [(rows, cols, vals), ...]."""
    s = _OrcCsr(n_rows, n_cols, 0, 0, None, None, None)
    L = orc()
    for rows, cols, vals in epochs:
        r, c, v = _arr(rows, np.uint32), _arr(cols, np.uint32), _arr(vals, np.float64)
        rc = L.orc_lock(C.byref(s), r.ctypes.data, c.ctypes.data, v.ctypes.data, len(r))
        if rc == 3:
            L.orc_csr_free(C.byref(s))
            raise IndexError("oracle lock: index out of range")
        assert rc == 0, rc
    return _take(s, L.orc_csr_free)


def spmv_scalar(A, x, fused=True):
    y = np.empty(A.n_rows, np.float64)
    off, cols, vals, x = _arr(A.off, np.uint64), _arr(A.cols, np.uint32), _arr(A.vals, np.float64), _arr(x, np.float64)
    orc().orc_spmv_scalar(off.ctypes.data, cols.ctypes.data, vals.ctypes.data, A.n_rows, x.ctypes.data,
                          y.ctypes.data, int(fused))
    return y


def host_dot_shape():
    """(lanes, tail_fused) of Spira's sparse_dot_double on this host: NEON
    (2 lanes, contracted tail) on aarch64, AVX-512 (8 lanes, plain tail) on
    x86-64."""
    import platform
    return (2, 1) if platform.machine() in ("aarch64", "arm64") else (8, 0)


def spmv_blocked(A, x, lanes=None, tail_fused=None):
    if lanes is None:
        lanes, tail_fused = host_dot_shape()
    y = np.empty(A.n_rows, np.float64)
    off, cols, vals, x = _arr(A.off, np.uint64), _arr(A.cols, np.uint32), _arr(A.vals, np.float64), _arr(x, np.float64)
    orc().orc_spmv_blocked(off.ctypes.data, cols.ctypes.data, vals.ctypes.data, A.n_rows, x.ctypes.data,
                           y.ctypes.data, lanes, int(tail_fused))
    return y


def spmv_parallel(A, x, n_threads, lanes=None, tail_fused=None, y=None):
    if lanes is None:
        lanes, tail_fused = host_dot_shape()
    if y is None:
        y = np.empty(A.n_rows, np.float64)
    off, cols, vals, x = _arr(A.off, np.uint64), _arr(A.cols, np.uint32), _arr(A.vals, np.float64), _arr(x, np.float64)
    rc = orc().orc_spmv_parallel(off.ctypes.data, cols.ctypes.data, vals.ctypes.data, A.n_rows, x.ctypes.data,
                                 y.ctypes.data, n_threads, lanes, int(tail_fused))
    assert rc == 0
    return y


def spmv_compensated(A, x):
    """(y, scale): Neumaier-compensated FP64 y and per-row sum |a x|."""
    y = np.empty(A.n_rows, np.float64)
    sc = np.empty(A.n_rows, np.float64)
    off, cols, vals, x = _arr(A.off, np.uint64), _arr(A.cols, np.uint32), _arr(A.vals, np.float64), _arr(x, np.float64)
    orc().orc_spmv_compensated(off.ctypes.data, cols.ctypes.data, vals.ctypes.data, A.n_rows, x.ctypes.data,
                               y.ctypes.data, sc.ctypes.data)
    return y, sc


def spgemm(A, B, fused=False) -> Csr:
    sa, ka = _as_c(A)
    sb, kb = _as_c(B)
    out = _OrcCsr()
    rc = orc().orc_spgemm(C.byref(sa), C.byref(sb), C.byref(out), int(fused))
    assert rc == 0
    return _take(out, orc().orc_csr_free)


def spgemm_parallel(A, B, n_threads: int, fused=False) -> Csr:
    """parallel::algorithms::spgemm on t*n/T row partitions, one thread each."""
    sa, ka = _as_c(A)
    sb, kb = _as_c(B)
    out = _OrcCsr()
    rc = orc().orc_spgemm_parallel(C.byref(sa), C.byref(sb), C.byref(out), int(n_threads), int(fused))
    assert rc == 0
    return _take(out, orc().orc_csr_free)


def transpose_parallel(A, n_threads: int) -> Csr:
    """parallel::algorithms::transpose: each output partition scans all of A."""
    sa, ka = _as_c(A)
    out = _OrcCsr()
    rc = orc().orc_transpose_parallel(C.byref(sa), C.byref(out), int(n_threads))
    assert rc == 0
    return _take(out, orc().orc_csr_free)


def lock_parallel_time(n_rows: int, n_cols: int, epochs, n_threads: int):
    """parallel_matrix::lock of each epoch on n_threads partitions: (wall
    seconds per epoch, stored entries after the last)."""
    keep = [(_arr(r, np.uint32), _arr(c, np.uint32), _arr(v, np.float64)) for r, c, v in epochs]
    n = len(keep)
    rp = (C.c_void_p * n)(*[k[0].ctypes.data for k in keep])
    cp = (C.c_void_p * n)(*[k[1].ctypes.data for k in keep])
    vp = (C.c_void_p * n)(*[k[2].ctypes.data for k in keep])
    ms = np.array([len(k[0]) for k in keep], np.uint64)
    secs = np.zeros(n, np.float64)
    nnz = C.c_uint64()
    rc = orc().orc_lock_parallel_time(n_rows, n_cols, int(n_threads), n, rp, cp, vp, ms.ctypes.data,
                                      secs.ctypes.data, C.byref(nnz))
    if rc == 3:
        raise IndexError("oracle lock: index out of range")
    assert rc == 0, rc
    return secs, nnz.value


def spgemm_products(A, B) -> int:
    sa, ka = _as_c(A)
    sb, kb = _as_c(B)
    return int(orc().orc_spgemm_products(C.byref(sa), C.byref(sb)))


def transpose(A) -> Csr:
    sa, ka = _as_c(A)
    out = _OrcCsr()
    rc = orc().orc_transpose(C.byref(sa), C.byref(out))
    assert rc == 0
    return _take(out, orc().orc_csr_free)


def add(A, B) -> Csr:
    sa, ka = _as_c(A)
    sb, kb = _as_c(B)
    out = _OrcCsr()
    rc = orc().orc_add(C.byref(sa), C.byref(sb), C.byref(out))
    assert rc == 0
    return _take(out, orc().orc_csr_free)


def scale(A, s: float, divide: bool = False) -> Csr:
    sa, ka = _as_c(A)
    out = _OrcCsr()
    rc = orc().orc_scale(C.byref(sa), float(s), int(divide), C.byref(out))
    assert rc == 0
    return _take(out, orc().orc_csr_free)


def row_sums(A) -> np.ndarray:
    off, vals = _arr(A.off, np.uint64), _arr(A.vals, np.float64)
    out = np.empty(A.n_rows, np.float64)
    orc().orc_row_sums(off.ctypes.data, vals.ctypes.data, A.n_rows, out.ctypes.data)
    return out


def partition(A, n_parts: int) -> np.ndarray:
    off = _arr(A.off, np.uint64)
    b = np.empty(n_parts + 1, np.uint64)
    orc().orc_partition(off.ctypes.data, A.n_rows, n_parts, b.ctypes.data)
    return b


# ---------------------------------------------------------------- Spira itself
class RefError(Exception):
    pass


def _ref_rc(rc):
    if rc == 0:
        return
    msg = ref().ref_last_error().decode()
    raise {1: ValueError, 2: RuntimeError, 3: IndexError, 4: ArithmeticError}.get(rc, RefError)(msg)


def ref_lock_epochs(n_rows, n_cols, epochs, layout=1, n_threads=4) -> Csr:
    """Spira's own insert/lock/open (layout 0 AoS matrix, 1 SoA matrix, 2 parallel_matrix)."""
    lens = np.array([len(e[0]) for e in epochs], dtype=np.uint64)
    rows = _arr(np.concatenate([e[0] for e in epochs]) if len(epochs) else [], np.uint32)
    cols = _arr(np.concatenate([e[1] for e in epochs]) if len(epochs) else [], np.uint32)
    vals = _arr(np.concatenate([e[2] for e in epochs]) if len(epochs) else [], np.float64)
    out = _OrcCsr()
    rc = ref().ref_lock_epochs(layout, n_threads, n_rows, n_cols, len(epochs), lens.ctypes.data, rows.ctypes.data,
                               cols.ctypes.data, vals.ctypes.data, C.byref(out))
    _ref_rc(rc)
    return _take(out, ref().ref_csr_free)


def ref_spmv(A, x, mode=0, n_threads=4):
    sa, ka = _as_c(A)
    x = _arr(x, np.float64)
    y = np.empty(A.n_rows, np.float64)
    _ref_rc(ref().ref_spmv(mode, n_threads, C.byref(sa), x.ctypes.data, y.ctypes.data))
    return y


def ref_spmv_parallel_time(A, x, n_threads, reps=10):
    sa, ka = _as_c(A)
    x = _arr(x, np.float64)
    y = np.empty(A.n_rows, np.float64)
    t = ref().ref_spmv_parallel_time(n_threads, C.byref(sa), x.ctypes.data, y.ctypes.data, reps)
    return t, y


def ref_spgemm(A, B, parallel=False, n_threads=4) -> Csr:
    sa, ka = _as_c(A)
    sb, kb = _as_c(B)
    out = _OrcCsr()
    _ref_rc(ref().ref_spgemm(int(parallel), n_threads, C.byref(sa), C.byref(sb), C.byref(out)))
    return _take(out, ref().ref_csr_free)


def ref_transpose(A, parallel=False, n_threads=4) -> Csr:
    sa, ka = _as_c(A)
    out = _OrcCsr()
    _ref_rc(ref().ref_transpose(int(parallel), n_threads, C.byref(sa), C.byref(out)))
    return _take(out, ref().ref_csr_free)


def ref_add(A, B, parallel=False, n_threads=4) -> Csr:
    sa, ka = _as_c(A)
    sb, kb = _as_c(B)
    out = _OrcCsr()
    _ref_rc(ref().ref_add(int(parallel), n_threads, C.byref(sa), C.byref(sb), C.byref(out)))
    return _take(out, ref().ref_csr_free)


def ref_scale(A, s, divide=False, in_place=False) -> Csr:
    sa, ka = _as_c(A)
    out = _OrcCsr()
    _ref_rc(ref().ref_scale(int(in_place), int(divide), C.byref(sa), float(s), C.byref(out)))
    return _take(out, ref().ref_csr_free)


def ref_row_sums(A) -> np.ndarray:
    sa, ka = _as_c(A)
    out = np.empty(A.n_rows, np.float64)
    ref().ref_row_sums(C.byref(sa), out.ctypes.data)
    return out


def ref_partition(A, n_parts: int) -> np.ndarray:
    sa, ka = _as_c(A)
    b = np.empty(n_parts + 1, np.uint64)
    ref().ref_partition(C.byref(sa), n_parts, b.ctypes.data)
    return b


# ---------------------------------------------------------------- host inputs
def gen_draw(seed: int, stream: int, n: int, kind: int, bound: int = 0, counter0: int = 0) -> np.ndarray:
    """spira_gb300.gen's draws computed in C (kind 0 uint32 below(bound),
    1 double in [-1, 1), 2 double in [0, 1))."""
    L = orc()
    L.orc_gen_draw.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64, C.c_int, C.c_uint64, C.c_void_p]
    out = np.empty(n, np.uint32 if kind == 0 else np.float64)
    L.orc_gen_draw(seed, stream, counter0, n, kind, bound, out.ctypes.data)
    return out


def zipf_rows_host(n_rows: int, alpha: float = 1.8, cap: int = 10_000, mean: float = 16.0, seed: int = 42):
    """Equal to spira_gb300.gen.zipf_rows, without large numpy temporaries."""
    from spira_gb300 import gen
    Ls = np.ascontiguousarray(gen.zipf_lengths(n_rows, alpha, cap, mean, seed), dtype=np.int64)
    m = int(Ls.sum())
    rows = np.empty(m, np.uint32)
    L = orc()
    L.orc_gen_expand_rows.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p]
    L.orc_gen_expand_rows(Ls.ctypes.data, n_rows, rows.ctypes.data)
    return rows, gen_draw(seed, 4, m, 0, n_rows), gen_draw(seed, 5, m, 1)


def csr_digest(A) -> str:
    """sha256 over (n_rows, n_cols, offsets, cols, value bits)."""
    import hashlib
    h = hashlib.sha256()
    h.update(np.array([A.n_rows, A.n_cols], np.uint64).tobytes())
    h.update(_arr(A.off, np.uint64).tobytes())
    h.update(_arr(A.cols, np.uint32).tobytes())
    h.update(_arr(A.vals, np.float64).tobytes())
    return h.hexdigest()
