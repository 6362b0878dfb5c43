"""The binary CSR file header, read without a device: sizes come back, and
files that do not match their header are refused."""
from __future__ import annotations

import numpy as np
import pytest

import spira_gb300 as sg
import csr_file


def _small():
    off = np.array([0, 2, 2, 5], np.uint64)
    cols = np.array([1, 4, 0, 2, 3], np.uint32)
    vals = np.array([1.0, -2.0, 0.5, 3.0, 4.0])
    return off, cols, vals


def test_header_sizes(tmp_path):
    p = tmp_path / "a.spgcsr"
    off, cols, vals = _small()
    csr_file.write(p, 3, 5, off, cols, vals)
    assert sg.csr_file_info(p) == (3, 5, 5)
    assert p.stat().st_size == 64 + 4 * 8 + 24 + 5 * 8


def test_header_rejections(tmp_path):
    off, cols, vals = _small()
    p = tmp_path / "bad.spgcsr"
    csr_file.write(p, 3, 5, off, cols, vals)
    raw = p.read_bytes()
    p.write_bytes(b"XPGCSR\x00\x00" + raw[8:])
    with pytest.raises(sg.InvalidArgument):
        sg.csr_file_info(p)
    p.write_bytes(raw[:-8])  # truncated
    with pytest.raises(sg.InvalidArgument):
        sg.csr_file_info(p)
    csr_file.write(p, 3, 5, off, cols, vals, version=2)
    with pytest.raises(sg.Unsupported):
        sg.csr_file_info(p)
    csr_file.write(p, 4, 5, off, cols, vals)  # header claims a row the file lacks
    with pytest.raises(sg.InvalidArgument):
        sg.csr_file_info(p)
    with pytest.raises(sg.InvalidArgument):
        sg.csr_file_info(tmp_path / "missing.spgcsr")
