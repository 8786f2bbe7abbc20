"""Builds the reference harness (test infrastructure) into oracle/_ref/.

The harness compiles the LBDEMcoupling reference's PSM headers where they lie
(``<reference>/src``, plus ``<reference>`` for ``fix_lb_coupling_onetoone.h``)
against the minimal Palabos/LIGGGHTS stand-ins of ``oracle/ref_harness/include``.
Nothing of the reference is copied into this repository.  Without the
reference tree (e.g. on a machine that only has this repository) the harness
is simply not built.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libref_harness.so"
SRC = HERE / "ref_harness" / "ref_harness.cpp"
INC = HERE / "ref_harness" / "include"
REFERENCE = Path(os.environ.get("LBDEM_REFERENCE", "/root/reference"))


def reference_present() -> bool:
    return (REFERENCE / "src" / "ibCompositeDynamics3D.hh").exists()


def build(force: bool = False) -> Path | None:
    if not reference_present():
        return None
    deps = [SRC] + list(INC.rglob("*")) + [Path(__file__)]
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return LIB
    OUT.mkdir(exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cxx, "-O2", "-ffp-contract=off", "-std=c++11", "-shared", "-fPIC", "-w",
           f"-I{INC}", f"-I{REFERENCE / 'src'}", f"-I{REFERENCE}", str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference harness build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
