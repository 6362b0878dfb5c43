"""A numpy writer for the binary CSR file format of spg_csr_save (header,
8-byte aligned sections, order-independent word checksum), used by the tests
to craft files independently of the library."""
from __future__ import annotations

import struct

import numpy as np

MAGIC = b"SPGCSR\x00\x00"
GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def _mix64(z: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def payload(off, cols, vals) -> bytes:
    c = np.asarray(cols, "<u4").tobytes()
    c += b"\x00" * ((-len(c)) % 8)
    return np.asarray(off, "<u8").tobytes() + c + np.asarray(vals, "<f8").tobytes()


def checksum(body: bytes) -> int:
    w = np.frombuffer(body, dtype="<u8")
    with np.errstate(over="ignore"):
        z = w ^ (np.arange(len(w), dtype=np.uint64) * GOLDEN)
        return int(_mix64(z).sum(dtype=np.uint64))


def write(path, n_rows, n_cols, off, cols, vals, flags=0, version=1, checksum_override=None):
    body = payload(off, cols, vals)
    cs = checksum(body) if checksum_override is None else checksum_override
    head = MAGIC + struct.pack("<7Q", version, n_rows, n_cols, len(cols), flags, cs, 0)
    with open(path, "wb") as f:
        f.write(head + body)
