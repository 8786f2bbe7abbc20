"""Builds the CPU oracle (test infrastructure) into oracle/_build/libpsm_oracle.so.

g++ -O3 -ffp-contract=off keeps every multiply and add separately rounded, so
the voxelization arithmetic is the IEEE double sequence of the reference.
OpenMP is used when the compiler supports it (threads parallelize the x-slabs;
with one thread the sweep order is the reference's x, y, z order).
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "libpsm_oracle.so"
SRC = HERE / "psm_oracle.cpp"


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(SRC.stat().st_mtime, Path(__file__).stat().st_mtime):
        return LIB
    OUT.mkdir(exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    base = [cxx, "-O3", "-ffp-contract=off", "-std=c++17", "-shared", "-fPIC", str(SRC)]
    tmp = LIB.with_suffix(".so.tmp")
    r = subprocess.run(base + ["-fopenmp", "-o", str(tmp)], capture_output=True, text=True)
    if r.returncode != 0:
        r = subprocess.run(base + ["-o", str(tmp)], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
