"""Builds the CPU oracle (test infrastructure) into oracle/_build/libp3oracle.so.

g++ with OpenMP over columns.  Floating-point contraction is disabled so the
oracle gives the same results on x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libp3oracle.so"
SRC = HERE / "p3_oracle.cpp"
HDR = HERE / "p3_oracle.h"


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    newest = max(SRC.stat().st_mtime, HDR.stat().st_mtime, Path(__file__).stat().st_mtime)
    if LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", str(SRC), "-o", str(LIB)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
