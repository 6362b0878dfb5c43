"""Compile the C++ facade test program (tests/cpp/test_facade.cpp) against
include/spira_gb300/spira.hpp and libspg.so into tests/cpp/_build/."""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
OUT = HERE / "_build" / "test_facade"


def build() -> Path:
    OUT.parent.mkdir(exist_ok=True)
    src = HERE / "test_facade.cpp"
    deps = [src, ROOT / "include" / "spira_gb300" / "spira.hpp", ROOT / "include" / "spg.h",
            ROOT / "spira_gb300" / "libspg.so"]
    if OUT.exists() and OUT.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return OUT
    cmd = ["g++", "-std=c++23", "-O2", "-Wall", "-Wextra", "-I", str(ROOT / "include"), str(src), "-o", str(OUT),
           "-L", str(ROOT / "spira_gb300"), "-lspg", f"-Wl,-rpath,{ROOT / 'spira_gb300'}", "-lpthread"]
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    print(build())
