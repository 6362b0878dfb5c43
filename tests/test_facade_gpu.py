"""Runs the C++ facade test program: Spira's own test scenarios, spelled as
Spira spells them, against include/spira_gb300/spira.hpp + libspg.so."""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "cpp"))


def test_facade_compiles():
    import build_facade_tests
    assert build_facade_tests.build().exists()


@pytest.mark.gpu
def test_facade_program_passes():
    import build_facade_tests
    exe = build_facade_tests.build()
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 failed" in r.stdout
