"""Build recipe for the CPU oracle shared library (test infrastructure only).

Compiles ``oracle/fsi_oracle.cpp`` with g++ into ``oracle/_build/libfsi_oracle.so``.
``-ffp-contract=off`` keeps every multiply and add separately rounded, as the
restatement requires; OpenMP provides the multi-threaded CPU baseline.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "fsi_oracle.cpp"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "libfsi_oracle.so"


def build(force: bool = False, verbose: bool = False) -> Path:
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    if LIB.exists() and not force and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cmd = [
        os.environ.get("CXX", "g++"),
        "-O2",
        "-std=c++17",
        "-fPIC",
        "-shared",
        "-fopenmp",
        "-ffp-contract=off",
        "-fno-fast-math",
        str(SRC),
        "-o",
        str(LIB) + ".tmp",
    ]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(str(LIB) + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
