"""The C ABI surface without compute calls: libspg.so loads, exports every
entry point include/spg.h declares, and reports errors as status codes."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import pytest

import spira_gb300 as sg

ROOT = Path(__file__).resolve().parent.parent


def declared(header: Path) -> list[str]:
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(spg_[a-z0-9_]+)\s*\(", text)))


def test_header_declarations_match_binding():
    names = sorted({n for h in (ROOT / "include").glob("*.h") for n in declared(h)})
    assert "spg_spmv" in names and "spg_lock" in names
    assert sorted(sg.exported_symbols()) == names


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(sg.LIB_PATH))
    for h in sorted((ROOT / "include").glob("*.h")):
        for name in declared(h):
            assert hasattr(lib, name), f"{name} declared in {h.name} but not exported"


def test_strerror_and_version_need_no_gpu():
    L = sg.lib()
    assert L.spg_strerror(0) == b"ok"
    assert L.spg_strerror(3) == b"index out of range"
    assert L.spg_version() >= 10000


def test_null_arguments_are_status_codes():
    L = sg.lib()
    assert L.spg_ctx_create(0, None) == 1
    assert L.spg_csr_info_get(None, None) == 1
    assert L.spg_spmv(None, None, None, None, 0, None) == 1
    assert L.spg_csr_add(None, None, None, None) == 1
    assert L.spg_csr_scale(None, None, None, 2.0, 0) == 1
    assert L.spg_csr_row_sums(None, None, None, None) == 1
    assert L.spg_csr_lookup(None, None, 0, None, None, None, None, None) == 1
    assert L.spg_csr_partition(None, None, 4, None) == 1
    assert L.spg_csr_save(None, None, b"x") == 1
    assert L.spg_csr_load_file(None, None, b"x") == 1
    assert L.spg_csr_file_info(None, None, None, None) == 1
    assert L.spg_strerror(8) == b"domain error"


def test_no_gpu_is_an_error_not_a_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(sg.SpgError):
        sg.Context(0)
