"""spira_gb300 — Python binding of libspg.so, the GB300 engine behind Spira's
sparse hot path (lock / SpMV / transpose / SpGEMM on device-resident CSR).

The engine's public boundary is the C ABI in include/spg.h; the C++23 facade
in include/spira_gb300/ mirrors Spira's own classes over it. This module is a
thin ctypes binding of the same ABI for tests and the benchmark. There is no
CPU fallback: importing works anywhere, but every compute call needs libspg.so
and a GB300, and raises otherwise.
"""
from __future__ import annotations

import ctypes as C
import os
from collections import namedtuple
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libspg.so"

SPMV_AUTO, SPMV_SCALAR, SPMV_VECTOR2, SPMV_VECTOR4, SPMV_VECTOR8, SPMV_VECTOR16, SPMV_VECTOR32, \
    SPMV_STREAM, SPMV_MERGE, SPMV_ADAPTIVE, SPMV_ADAPTIVE16, SPMV_INTERLEAVED = -1, 0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10
SPMV_INTERLEAVED_S4, SPMV_INTERLEAVED_S8, SPMV_ADAPTIVE16_S4, SPMV_ADAPTIVE_S16 = 11, 12, 13, 14
# (variant, tile) candidates: the chunk kernels' tiles (sub-batch depth x
# blocks per SM) compute their base variant's bits
SPMV_VARIANTS = {
    "scalar": 0, "vector2": 1, "vector4": 2, "vector8": 3, "vector16": 4, "vector32": 5,
    "stream": 6, "merge": 7, "adaptive": 8, "adaptive16": 9, "interleaved": 10,
    "interleaved_s4": 11, "interleaved_s8": 12, "adaptive16_s4": 13, "adaptive_s16": 14,
}
SPMV_NAMES = {v: k for k, v in SPMV_VARIANTS.items()}
SPGEMM_AUTO = -1
SPGEMM_VARIANTS = {"rowmerge": 0, "esc": 1, "warpsort_64": 2, "warpsort_128": 3, "warpsort_256": 4}
SPGEMM_NAMES = {v: k for k, v in SPGEMM_VARIANTS.items()}

CsrHost = namedtuple("CsrHost", "n_rows n_cols off cols vals capacity")


class SpgError(RuntimeError):
    code = -1


class InvalidArgument(SpgError, ValueError):
    """std::invalid_argument in Spira."""
    code = 1


class LogicError(SpgError):
    """std::logic_error in Spira."""
    code = 2


class OutOfRange(SpgError, IndexError):
    """std::out_of_range in Spira."""
    code = 3


class NoMemory(SpgError, MemoryError):
    code = 4


class CudaError(SpgError):
    code = 5


class DeviceTimeout(SpgError):
    code = 6


class Unsupported(SpgError):
    code = 7


class DomainError(SpgError, ArithmeticError):
    """std::domain_error in Spira (division by a zero scalar)."""
    code = 8


_ERRORS = {c.code: c for c in (InvalidArgument, LogicError, OutOfRange, NoMemory, CudaError, DeviceTimeout,
                               Unsupported, DomainError)}


class _Info(C.Structure):
    _fields_ = [("n_rows", C.c_uint64), ("n_cols", C.c_uint64), ("nnz", C.c_uint64),
                ("capacity", C.c_uint64), ("built", C.c_int)]


_lib = None

# (name, restype, argtypes) of every symbol include/spg.h declares.
_P = C.c_void_p
_U64, _U32, _I = C.c_uint64, C.c_uint32, C.c_int
_SIGS = [
    ("spg_strerror", C.c_char_p, [_I]),
    ("spg_last_error", C.c_char_p, []),
    ("spg_version", _I, []),
    ("spg_ctx_create", _I, [_I, C.POINTER(_P)]),
    ("spg_ctx_destroy", _I, [_P]),
    ("spg_ctx_stream", _I, [_P, C.POINTER(_P)]),
    ("spg_ctx_sync", _I, [_P]),
    ("spg_ctx_pool_used", _I, [_P, C.POINTER(_U64), C.POINTER(_U64)]),
    ("spg_selftest_wait_timeout", _I, [_P, C.c_longlong, C.POINTER(_I)]),
    ("spg_ctx_timer_start", _I, [_P]),
    ("spg_ctx_timer_stop", _I, [_P, C.POINTER(C.c_double)]),
    ("spg_csr_create", _I, [_P, _U64, _U64, C.POINTER(_P)]),
    ("spg_csr_destroy", _I, [_P]),
    ("spg_csr_info_get", _I, [_P, C.POINTER(_Info)]),
    ("spg_csr_device_arrays", _I, [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)]),
    ("spg_csr_download", _I, [_P, _P, _P, _P, _P]),
    ("spg_csr_load", _I, [_P, _P, _P, _P, _P, _U64]),
    ("spg_csr_copy", _I, [_P, _P, _P]),
    ("spg_csr_get", _I, [_P, _P, _U64, _U32, C.POINTER(C.c_double), C.POINTER(_I)]),
    ("spg_csr_row_range", _I, [_P, _P, _U64, C.POINTER(_U64), C.POINTER(_U64)]),
    ("spg_lock", _I, [_P, _P, _P, _P, _P, _U64]),
    ("spg_lock_device", _I, [_P, _P, _P, _P, _P, _U64]),
    ("spg_spmv", _I, [_P, _P, _P, _P, _I, _P]),
    ("spg_spmv_host", _I, [_P, _P, _P, _U64, _P, _U64, _I]),
    ("spg_spmv_host_async", _I, [_P, _P, _P, _U64, _P, _U64, _I, _P]),
    ("spg_spmv_host_multi", _I, [_P, _U32, _P, _P, _P, _P, _P]),
    ("spg_spmv_noalloc", _I, [_P, _P, _P, _P, _P]),
    ("spg_spmv_noalloc_max", _U64, []),
    ("spg_spmv_selected", _I, [_P, _P, C.POINTER(_I)]),
    ("spg_spmv_launches", _I, [_P, _P, _I, C.POINTER(_I)]),
    ("spg_set_spmv_policy", _I, [_P, _I]),
    ("spg_spmv_features", _I, [_P, _P, _P]),
    ("spg_spmv_autotune", _I, [_P, _P, _I, _P, C.POINTER(_I)]),
    ("spg_probe_gather_rate", _I, [_P, _U64, _U64, C.POINTER(C.c_double)]),
    ("spg_probe_gather_rate_cfg", _I, [_P, _U64, _U64, _I, _I, C.POINTER(C.c_double), C.POINTER(_I)]),
    ("spg_probe_fp64_rate", _I, [_P, C.c_uint32, C.POINTER(C.c_double)]),
    ("spg_selector_load", _I, [_P, _P, _U64, _I]),
    ("spg_mlp_param_count", _U64, [_I]),
    ("spg_selector_predict", _I, [_P, _P, _U32, _P, _P]),
    ("spg_mlp_forward", _I, [_P, _P, _I, _P, _U32, _P, _P, _P]),
    ("spg_mlp_backward", _I, [_P, _P, _I, _P, _U32, _P, _P, _P, _P]),
    ("spg_mlp_mse", _I, [_P, _P, _P, _U64, _P, _P, _P]),
    ("spg_mlp_adam", _I, [_P, _P, _P, _P, _P, _U64, C.c_float, C.c_float, C.c_float, C.c_float, _U32, _P]),
    ("spg_mlp_argmin", _I, [_P, _P, _U32, _I, _P, _P]),
    ("spg_batch_create", _I, [_P, _U32, _P, _P, _P, _P, _I, C.POINTER(_P)]),
    ("spg_batch_config", _I, [_P, C.POINTER(_I), C.POINTER(_U32)]),
    ("spg_batch_run", _I, [_P, _P, _P]),
    ("spg_batch_run_plain", _I, [_P, _P, _P]),
    ("spg_batch_destroy", _I, [_P]),
    ("spg_csr_add", _I, [_P, _P, _P, _P]),
    ("spg_csr_scale", _I, [_P, _P, _P, C.c_double, _I]),
    ("spg_csr_row_sums", _I, [_P, _P, _P, _P]),
    ("spg_csr_row_sums_host", _I, [_P, _P, _U64, _U64, _P]),
    ("spg_csr_lookup", _I, [_P, _P, _U64, _P, _P, _P, _P, _P]),
    ("spg_csr_partition", _I, [_P, _P, _U64, _P]),
    ("spg_csr_save", _I, [_P, _P, C.c_char_p]),
    ("spg_csr_load_file", _I, [_P, _P, C.c_char_p]),
    ("spg_csr_file_info", _I, [C.c_char_p, C.POINTER(_U64), C.POINTER(_U64), C.POINTER(_U64)]),
    ("spg_transpose", _I, [_P, _P, _P]),
    ("spg_spgemm", _I, [_P, _P, _P, _P]),
    ("spg_spgemm_variant", _I, [_P, _P, _P, _P, _I]),
    ("spg_spgemm_selected", _I, [_P, _P, _P, C.POINTER(_I)]),
    ("spg_spgemm_features", _I, [_P, _P, _P, _P]),
    ("spg_spgemm_autotune", _I, [_P, _P, _P, _I, _P, C.POINTER(_I)]),
    ("spg_spgemm_selector_load", _I, [_P, _P, _U64, _I]),
    ("spg_spgemm_selector_predict", _I, [_P, _P, _U32, _P, _P]),
    ("spg_set_spgemm_policy", _I, [_P, _I]),
    # spg_gen.h
    ("spg_gen_draw", _I, [_P, _U64, _U64, _U64, _U64, _I, _U64, _P]),
    ("spg_gen_expand_rows", _I, [_P, _P, _U64, _P, C.POINTER(_U64)]),
    ("spg_gen_family", _I, [_P, _I, _U64, _U64, C.c_double, _P, _U64, _P, _P, _P, C.POINTER(_U64)]),
]

N_FEATURES, N_HIDDEN = 40, 64
POLICY_SELECTOR, POLICY_AUTOTUNE, POLICY_FIXED = 0, 1, 2
FAM_BANDED, FAM_BLOCKDIAG, FAM_POWERLAW, FAM_UNIFORM, FAM_STENCIL2D, FAM_STENCIL3D, FAM_POISSON = range(7)


def exported_symbols() -> list[str]:
    return [s[0] for s in _SIGS]


def lib():
    """Load libspg.so (raises if it was not built: no fallback exists)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in _SIGS:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(status: int):
    if status != 0:
        msg = lib().spg_last_error().decode(errors="replace")
        raise _ERRORS.get(status, SpgError)(f"[{lib().spg_strerror(status).decode()}] {msg}")


def _ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch tensors


class Context:
    """One device, one stream, the device memory pool (spg_ctx)."""

    def __init__(self, device: int = 0):
        h = _P()
        _check(lib().spg_ctx_create(device, C.byref(h)))
        self.h = h
        self.device = device

    def close(self):
        if self.h:
            lib().spg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        s = _P()
        _check(lib().spg_ctx_stream(self.h, C.byref(s)))
        return s.value or 0

    def sync(self):
        _check(lib().spg_ctx_sync(self.h))

    def device_ms(self, fn) -> float:
        """Runs fn() and returns the device time of the work it put on the
        context stream, host round trips at the operations' internal
        synchronisations excluded (spg_ctx_timer_start / _stop)."""
        _check(lib().spg_ctx_timer_start(self.h))
        try:
            fn()
        finally:
            ms = C.c_double()
            st = lib().spg_ctx_timer_stop(self.h, C.byref(ms))
        _check(st)
        return ms.value

    def pool_used(self):
        """(bytes live buffers hold, bytes the pool holds) of the context's
        device memory pool."""
        u, r = C.c_uint64(), C.c_uint64()
        _check(lib().spg_ctx_pool_used(self.h, C.byref(u), C.byref(r)))
        return u.value, r.value

    def set_spmv_policy(self, policy: int):
        _check(lib().spg_set_spmv_policy(self.h, policy))

    def set_spgemm_policy(self, policy: int):
        _check(lib().spg_set_spgemm_policy(self.h, policy))

    def load_spgemm_selector(self, blob, n_outputs: int):
        """Install an SpGEMM selector blob (numpy float32); None removes it."""
        if blob is None:
            _check(lib().spg_spgemm_selector_load(self.h, None, 0, 0))
            return
        blob = np.ascontiguousarray(blob, dtype=np.float32)
        _check(lib().spg_spgemm_selector_load(self.h, _ptr(blob), len(blob), n_outputs))

    def load_selector(self, blob, n_outputs: int):
        """Install a selector blob (numpy float32) for SPMV_AUTO; None removes it."""
        if blob is None:
            _check(lib().spg_selector_load(self.h, None, 0, 0))
            return
        blob = np.ascontiguousarray(blob, dtype=np.float32)
        _check(lib().spg_selector_load(self.h, _ptr(blob), len(blob), n_outputs))

    def probe_gather_rate(self, n_x: int = 1 << 22, n_gathers: int = 1 << 26) -> float:
        """Random 8-byte gathers per second from an n_x-entry vector: the
        ceiling of SpMV on matrices with randomly spread columns."""
        r = C.c_double()
        _check(lib().spg_probe_gather_rate(self.h, n_x, n_gathers, C.byref(r)))
        return r.value

    def probe_gather_rate_cfg(self, per_thread: int, blocks_per_sm: int, n_x: int = 1 << 22,
                              n_gathers: int = 1 << 26):
        """(gathers per second, resident blocks per SM) of the random-read
        probe with per_thread reads in flight per thread and blocks_per_sm
        blocks of 256 threads per SM."""
        r, b = C.c_double(), C.c_int()
        _check(lib().spg_probe_gather_rate_cfg(self.h, n_x, n_gathers, per_thread, blocks_per_sm, C.byref(r),
                                               C.byref(b)))
        return r.value, b.value

    def gather_ceiling_sweep(self, n_x: int = 1 << 22, n_gathers: int = 1 << 26):
        """The random-read probe over reads in flight per thread (2..64) and
        blocks per SM (2..16): every point and the maximum."""
        pts = []
        for per in (2, 4, 8, 16, 32, 64):
            for bps in (2, 4, 8, 16):
                rate, res = self.probe_gather_rate_cfg(per, bps, n_x, n_gathers)
                pts.append({"per_thread": per, "blocks_per_sm": bps, "resident_blocks_per_sm": res,
                            "gathers_per_s": rate})
        best = max(pts, key=lambda p: p["gathers_per_s"])
        return best, pts

    def probe_fp64_rate(self, iters: int = 4096) -> float:
        """FP64 fused multiply-adds per second over every SM: the ceiling of
        the batched multi-RHS SpMV (one FMA per nonzero and right-hand side)."""
        r = C.c_double()
        _check(lib().spg_probe_fp64_rate(self.h, iters, C.byref(r)))
        return r.value


class Csr:
    """A device-resident CSR matrix handle (spg_csr)."""

    def __init__(self, ctx: Context, n_rows: int, n_cols: int):
        self.ctx = ctx
        h = _P()
        _check(lib().spg_csr_create(ctx.h, n_rows, n_cols, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().spg_csr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> dict:
        i = _Info()
        _check(lib().spg_csr_info_get(self.h, C.byref(i)))
        return {"n_rows": i.n_rows, "n_cols": i.n_cols, "nnz": i.nnz, "capacity": i.capacity,
                "built": bool(i.built)}

    @property
    def n_rows(self):
        return self.info()["n_rows"]

    @property
    def n_cols(self):
        return self.info()["n_cols"]

    @property
    def nnz(self):
        return self.info()["nnz"]

    def lock(self, rows, cols, vals):
        """Merge one epoch of host-staged inserts (insertion order)."""
        rows = np.ascontiguousarray(rows, dtype=np.uint32)
        cols = np.ascontiguousarray(cols, dtype=np.uint32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        if not (len(rows) == len(cols) == len(vals)):
            raise InvalidArgument("rows/cols/vals length mismatch")
        _check(lib().spg_lock(self.ctx.h, self.h, _ptr(rows), _ptr(cols), _ptr(vals), len(rows)))

    def lock_device(self, d_rows, d_cols, d_vals, n: int):
        _check(lib().spg_lock_device(self.ctx.h, self.h, _ptr(d_rows), _ptr(d_cols), _ptr(d_vals), n))

    def load(self, off, cols, vals):
        off = np.ascontiguousarray(off, dtype=np.uint64)
        cols = np.ascontiguousarray(cols, dtype=np.uint32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        _check(lib().spg_csr_load(self.ctx.h, self.h, _ptr(off), _ptr(cols), _ptr(vals), len(cols)))

    def download(self) -> CsrHost:
        i = self.info()
        off = np.empty(i["n_rows"] + 1, np.uint64)
        cols = np.empty(i["nnz"], np.uint32)
        vals = np.empty(i["nnz"], np.float64)
        _check(lib().spg_csr_download(self.ctx.h, self.h, _ptr(off), _ptr(cols), _ptr(vals)))
        return CsrHost(i["n_rows"], i["n_cols"], off, cols, vals, i["capacity"])

    def device_arrays(self):
        o, c, v = _P(), _P(), _P()
        _check(lib().spg_csr_device_arrays(self.h, C.byref(o), C.byref(c), C.byref(v)))
        return o.value, c.value, v.value

    def copy_from(self, other: "Csr"):
        _check(lib().spg_csr_copy(self.ctx.h, other.h, self.h))

    def get(self, row: int, col: int):
        v, f = C.c_double(), C.c_int()
        _check(lib().spg_csr_get(self.ctx.h, self.h, row, col, C.byref(v), C.byref(f)))
        return (v.value if f.value else None)

    def row_range(self, row: int):
        b, e = C.c_uint64(), C.c_uint64()
        _check(lib().spg_csr_row_range(self.ctx.h, self.h, row, C.byref(b), C.byref(e)))
        return b.value, e.value

    def spmv(self, d_x, d_y, variant: int = SPMV_AUTO, stream: int | None = None):
        """Asynchronous y = A x on device pointers (ints or torch tensors)."""
        _check(lib().spg_spmv(self.ctx.h, self.h, _ptr(d_x), _ptr(d_y), variant, stream))

    def spmv_host(self, x, y=None, variant: int = SPMV_AUTO):
        x = np.ascontiguousarray(x, dtype=np.float64)
        if y is None:
            y = np.empty(self.n_rows, np.float64)
        _check(lib().spg_spmv_host(self.ctx.h, self.h, _ptr(x), len(x), _ptr(y), len(y), variant))
        return y

    def spmv_host_async(self, x, y, variant: int = SPMV_AUTO, stream=None):
        """y = A x from pinned host buffers (numpy views of pinned torch
        tensors), enqueued on `stream`; y is ready once the stream is."""
        _check(lib().spg_spmv_host_async(self.ctx.h, self.h, _ptr(x), len(x), _ptr(y), len(y), variant, stream))
        return y

    def selected_spmv(self) -> int:
        v = C.c_int()
        _check(lib().spg_spmv_selected(self.ctx.h, self.h, C.byref(v)))
        return v.value

    def spmv_launches(self, variant: int = SPMV_AUTO) -> int:
        n = C.c_int()
        _check(lib().spg_spmv_launches(self.ctx.h, self.h, variant, C.byref(n)))
        return n.value

    def features(self) -> np.ndarray:
        f = np.empty(N_FEATURES, np.float32)
        _check(lib().spg_spmv_features(self.ctx.h, self.h, _ptr(f)))
        return f

    def autotune(self, reps: int = 5):
        """(times_ms per variant, fastest variant)."""
        t = np.empty(len(SPMV_VARIANTS), np.float32)
        b = C.c_int()
        _check(lib().spg_spmv_autotune(self.ctx.h, self.h, reps, _ptr(t), C.byref(b)))
        return t, b.value

    def transpose(self) -> "Csr":
        """A new device matrix holding A^T."""
        T = Csr(self.ctx, 0, 0)
        _check(lib().spg_transpose(self.ctx.h, self.h, T.h))
        return T

    def spgemm(self, B: "Csr", variant: int = SPGEMM_AUTO) -> "Csr":
        """A new device matrix holding self * B (SPGEMM_AUTO: the context's
        policy picks the kernel path; every path gives the same C)."""
        Cm = Csr(self.ctx, 0, 0)
        if variant == SPGEMM_AUTO:
            _check(lib().spg_spgemm(self.ctx.h, self.h, B.h, Cm.h))
        else:
            _check(lib().spg_spgemm_variant(self.ctx.h, self.h, B.h, Cm.h, variant))
        return Cm

    def spgemm_selected(self, B: "Csr") -> int:
        v = C.c_int()
        _check(lib().spg_spgemm_selected(self.ctx.h, self.h, B.h, C.byref(v)))
        return v.value

    def spgemm_features(self, B: "Csr") -> np.ndarray:
        f = np.empty(N_FEATURES, np.float32)
        _check(lib().spg_spgemm_features(self.ctx.h, self.h, B.h, _ptr(f)))
        return f

    def spgemm_autotune(self, B: "Csr", reps: int = 3):
        """(times_ms per SpGEMM variant, fastest variant)."""
        t = np.empty(len(SPGEMM_VARIANTS), np.float32)
        b = C.c_int()
        _check(lib().spg_spgemm_autotune(self.ctx.h, self.h, B.h, reps, _ptr(t), C.byref(b)))
        return t, b.value

    def add(self, B: "Csr") -> "Csr":
        """A new device matrix holding self + B (MatrixAddition)."""
        Cm = Csr(self.ctx, 0, 0)
        _check(lib().spg_csr_add(self.ctx.h, self.h, B.h, Cm.h))
        return Cm

    def scaled(self, s: float, divide: bool = False) -> "Csr":
        """A new device matrix holding self * s (or self / s)."""
        Cm = Csr(self.ctx, 0, 0)
        _check(lib().spg_csr_scale(self.ctx.h, self.h, Cm.h, float(s), int(divide)))
        return Cm

    def scale_(self, s: float, divide: bool = False) -> "Csr":
        """In place: self *= s (or self /= s)."""
        _check(lib().spg_csr_scale(self.ctx.h, self.h, self.h, float(s), int(divide)))
        return self

    def row_sums(self, d_out=None, stream=None):
        """Row sums in CSR order (a locked row's accumulate()); a torch CUDA
        tensor, or written into d_out asynchronously."""
        if d_out is None:
            import torch
            out = torch.empty(self.n_rows, dtype=torch.float64, device="cuda")
            _check(lib().spg_csr_row_sums(self.ctx.h, self.h, _ptr(out), None))
            self.ctx.sync()
            return out
        _check(lib().spg_csr_row_sums(self.ctx.h, self.h, _ptr(d_out), stream))
        return d_out

    def row_sums_host(self, row0: int = 0, n: int | None = None) -> np.ndarray:
        n = self.n_rows - row0 if n is None else n
        out = np.empty(n, np.float64)
        _check(lib().spg_csr_row_sums_host(self.ctx.h, self.h, row0, n, _ptr(out)))
        return out

    def save(self, path) -> None:
        """Writes the CSR to a binary file (spg_csr_save)."""
        _check(lib().spg_csr_save(self.ctx.h, self.h, str(path).encode()))

    def load_file(self, path) -> "Csr":
        """Replaces this matrix with a saved file's CSR (checked)."""
        _check(lib().spg_csr_load_file(self.ctx.h, self.h, str(path).encode()))
        return self

    def lookup(self, d_rows, d_cols, d_vals=None, d_found=None, stream=None):
        """Batched point lookups on device arrays (uint64 rows, uint32 cols):
        writes the stored value (or 0.0) and a found flag (uint8) per query."""
        n = int(d_rows.numel()) if hasattr(d_rows, "numel") else len(d_rows)
        _check(lib().spg_csr_lookup(self.ctx.h, self.h, n, _ptr(d_rows), _ptr(d_cols), _ptr(d_vals), _ptr(d_found),
                                    stream))

    def partition(self, n_parts: int) -> np.ndarray:
        """nnz-balanced row boundaries (n_parts + 1 entries)."""
        b = np.empty(n_parts + 1, np.uint64)
        _check(lib().spg_csr_partition(self.ctx.h, self.h, n_parts, _ptr(b)))
        return b


# ---------------------------------------------------------------- device draws
GEN_BELOW_U32, GEN_SYM_F64, GEN_UNIT_F64 = 0, 1, 2


def spmv_host_multi(ctx: Context, mats, xs, ys, variants=None, stream=None):
    """SpMVs of several matrices from pinned host buffers (numpy views of
    pinned torch tensors) in one call, enqueued on `stream`."""
    n = len(mats)
    hm = (C.c_void_p * n)(*[A.h for A in mats])
    hx = (C.c_void_p * n)(*[_ptr(x) for x in xs])
    hy = (C.c_void_p * n)(*[_ptr(y) for y in ys])
    hv = (C.c_int * n)(*variants) if variants is not None else None
    _check(lib().spg_spmv_host_multi(ctx.h, n, hm, hx, hy, hv, stream))


def csr_file_info(path):
    """(n_rows, n_cols, nnz) from a CSR file's header; needs no device."""
    r, c, z = C.c_uint64(), C.c_uint64(), C.c_uint64()
    _check(lib().spg_csr_file_info(str(path).encode(), C.byref(r), C.byref(c), C.byref(z)))
    return r.value, c.value, z.value


def gen_draw(ctx: Context, seed: int, stream: int, n: int, kind: int, bound: int, d_out, counter0: int = 0):
    """Seeded draws on the device, equal to spira_gb300.gen on the host."""
    _check(lib().spg_gen_draw(ctx.h, seed, stream, counter0, n, kind, bound, _ptr(d_out)))


def gen_expand_rows(ctx: Context, d_lengths, n_rows: int, d_rows=None) -> int:
    tot = C.c_uint64()
    _check(lib().spg_gen_expand_rows(ctx.h, _ptr(d_lengths), n_rows, _ptr(d_rows), C.byref(tot)))
    return tot.value


def gen_family(ctx: Context, family: int, n_rows: int, p: int, ls: float = 0.0, d_cdf=None, seed: int = 0,
               d_rows=None, d_cols=None, d_vals=None) -> int:
    m = C.c_uint64()
    _check(lib().spg_gen_family(ctx.h, family, n_rows, p, ls, _ptr(d_cdf), seed, _ptr(d_rows), _ptr(d_cols),
                                _ptr(d_vals), C.byref(m)))
    return m.value


class Batch:
    """Persistent multi-RHS batch (spg_batch). mats: Csr list; X, Y: device
    buffers (torch tensors / pointers), row-major n x k; k: powers of two."""

    def __init__(self, ctx: Context, mats, Xs, Ys, ks, config: int = -1):
        n = len(mats)
        self.ctx, self._keep = ctx, (mats, Xs, Ys)
        ph = (C.c_void_p * n)(*[m.h.value for m in mats])
        px = (C.c_void_p * n)(*[_ptr(x) for x in Xs])
        py = (C.c_void_p * n)(*[_ptr(y) for y in Ys])
        kk = (C.c_uint32 * n)(*ks)
        h = _P()
        _check(lib().spg_batch_create(ctx.h, n, ph, px, py, kk, config, C.byref(h)))
        self.h = h

    def config(self):
        c, n = C.c_int(), C.c_uint32()
        _check(lib().spg_batch_config(self.h, C.byref(c), C.byref(n)))
        return c.value, n.value

    def run(self, stream=None):
        _check(lib().spg_batch_run(self.ctx.h, self.h, stream))

    def run_plain(self, stream=None):
        _check(lib().spg_batch_run_plain(self.ctx.h, self.h, stream))

    def close(self):
        if self.h:
            lib().spg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Mlp:
    """Device-side FP32 MLP 40 -> 64 -> 64 -> K through libspg's kernels
    (buffers are torch CUDA tensors)."""

    def __init__(self, ctx: Context, n_outputs: int):
        self.ctx, self.K = ctx, n_outputs
        self.n_params = int(lib().spg_mlp_param_count(n_outputs))

    def forward(self, params, X, act, out, B: int):
        _check(lib().spg_mlp_forward(self.ctx.h, _ptr(params), self.K, _ptr(X), B, _ptr(act), _ptr(out), None))

    def backward(self, params, X, act, dout, grad, B: int):
        _check(lib().spg_mlp_backward(self.ctx.h, _ptr(params), self.K, _ptr(X), B, _ptr(act), _ptr(dout),
                                      _ptr(grad), None))

    def mse(self, pred, target, n: int, dpred, loss=None):
        _check(lib().spg_mlp_mse(self.ctx.h, _ptr(pred), _ptr(target), n, _ptr(dpred), _ptr(loss), None))

    def adam(self, params, grad, m, v, lr, step, beta1=0.9, beta2=0.999, eps=1e-8):
        _check(lib().spg_mlp_adam(self.ctx.h, _ptr(params), _ptr(grad), _ptr(m), _ptr(v), self.n_params, lr, beta1,
                                  beta2, eps, step, None))

    def argmin(self, pred, B: int, best):
        _check(lib().spg_mlp_argmin(self.ctx.h, _ptr(pred), B, self.K, _ptr(best), None))
