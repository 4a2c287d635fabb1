"""Build recipe of the CPU oracle (test infrastructure).

Compiles ``oracle.cpp`` into ``oracle/_build/liboracle.so`` with
``-O2 -ffp-contract=off -fno-fast-math`` so that every f32 operation is the
IEEE operation the reference crate's Rust source performs, in its order.
The reference itself is Rust and cannot be built here (no rustc), so there
is no ``oracle/_ref`` build.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
SOURCES = [HERE / "oracle.cpp"]
HEADERS = [HERE / "oracle.h", HERE.parent / "include" / "pbrt_gpu.h"]


def build(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    deps = SOURCES + HEADERS + [Path(__file__)]
    if not force and LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    cxx = os.environ.get("CXX", "g++")
    tmp = BUILD / "liboracle.so.tmp"
    cmd = [cxx, "-O2", "-ffp-contract=off", "-fno-fast-math", "-std=c++17", "-fPIC", "-shared",
           "-pthread", *map(str, SOURCES), "-o", str(tmp)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
