"""The C++ shim on the GPU: the excludeType filter of setSpheresOnLattice
(src/ibDataExchangeWrappers3D.hh:62-73) through the reference's call
setSpheresOnLattice(lattice, wrapper, units, excludeType, initVel) and
getForcesFromLattice(lattice, wrapper, units) -- tests/exclude_type_check.cpp,
built against the library and the LIGGGHTS stand-in of the example programs."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "lbdemcoupling-public_gb300"


def _build(tmp_path):
    import build as pkg_build
    lib = pkg_build.build()
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "exclude_type_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-Wall", f"-I{ROOT / 'include'}", f"-I{PKG / 'plb'}",
                    f"-I{PKG / 'examples'}", str(ROOT / "tests" / "exclude_type_check.cpp"), f"-L{lib.parent}",
                    "-llbdem_gb300", f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    return exe


def test_exclude_type_builds_and_needs_a_gpu(lbdem_lib, tmp_path):
    torch = pytest.importorskip("torch")
    exe = _build(tmp_path)
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert subprocess.run([str(exe)], capture_output=True, text=True).returncode == 77


@pytest.mark.gpu
def test_exclude_type(gpu, tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
