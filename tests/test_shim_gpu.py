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


@pytest.mark.gpu
def test_set_omega_and_periodicity_after_creation(gpu, oracle):
    """lbdem_set_omega / lbdem_set_periodic (defineDynamics and
    lattice.periodicity().toggle of the reference's drivers): a handle created
    with other values steps exactly as the oracle built with the new ones."""
    import numpy as np
    import workloads as W
    from helpers import rel_err, small_suspension
    shape, per, omega = (20, 16, 24), (1, 0, 1), 1 / 0.6
    rng = np.random.default_rng(8)
    f0 = rng.standard_normal((19, *shape)) * 1e-3
    p = small_suspension(shape, 3, 2.0, 3.5, seed=9, periodic=per)
    ol = oracle.OracleLattice(*shape, omega, periodic=per)
    ol.set_populations(f0)
    with gpu.Lattice(*shape, 1.0, periodic=(1, 1, 1), max_particles=32, max_tag=16, max_radius=6) as L:
        L.set_omega(omega)
        L.set_periodic(per)
        L.set_populations(f0)
        for _ in range(3):
            g = W.with_ghosts(p, shape, per)
            L.set_particles(g.x, g.v, g.w, g.r, g.tag)
            ol.set_particles(g.x, g.v, g.w, g.r, g.tag)
            L.collide_and_stream()
            ol.collide_and_stream()
            Fg, _ = L.get_forces()
            Fo, _ = ol.get_forces()
            p = W.advance(p, shape, per)
        assert rel_err(L.get_populations(), ol.get_populations()) <= 1e-12
        assert rel_err(Fg, Fo) <= 1e-10 and np.abs(Fo).max() > 0
        with pytest.raises(gpu.LbdemError):
            L.set_omega(2.5)
        L.set_pressure_drop(0, [0, 0, 1, 14, 1, 22], [19, 19, 1, 14, 1, 22], 1.0, 0.999)
        with pytest.raises(gpu.LbdemError):
            L.set_periodic((1, 1, 1))
