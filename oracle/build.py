"""Builds the oracle — test infrastructure only — into ``oracle/_build``.

The oracle is a C++ restatement of the reference's CPU numeric phase
(``oracle_numeric.cpp``) and of its values-refresh operations and
Jacobi-preconditioned CG (``oracle_values.cpp``).  It is compiled without floating-point
contraction (``-ffp-contract=off``) so its element arithmetic is the
reference's mul-then-add on every host architecture.  The reference itself
is C# and cannot be built in this environment (no .NET SDK), so there is no
``oracle/_ref`` build.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRCS = [HERE / "oracle_numeric.cpp", HERE / "oracle_values.cpp"]
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "liboracle.so"


def build(verbose: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    if LIB.exists() and all(LIB.stat().st_mtime >= s.stat().st_mtime for s in SRCS):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", *map(str, SRCS), "-o",
           str(LIB), "-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{proc.stdout}\n{proc.stderr}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
