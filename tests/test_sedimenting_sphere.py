"""The C++ host shim (plb/lbdem_plb.h) driving the C ABI, with the LIGGGHTS
stand-in of examples/dem_standin.h: the sedimenting-sphere case, and the
multisphere branch of setSpheresOnLattice (examples/multisphere_check.cpp).

* CPU: the example program compiles and links against the library; without a GPU it
  exits with status 77.
* GPU: the first 20 coupling cycles agree with the oracle driven by the same
  integrator (trace z, vz, fz within 1e-9 relative), and a longer run shows a
  sphere settling: falling, drag opposing the motion and staying below the
  buoyant weight while the sphere still accelerates.
"""
import math
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "lbdemcoupling-public_gb300"
EXE = PKG / "_build" / "sedimenting_sphere"


def build_example(name="sedimenting_sphere"):
    import build as pkg_build
    lib = pkg_build.build()
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = PKG / "_build" / name
    src = PKG / "examples" / f"{name}.cpp"
    deps = [src, PKG / "examples" / "dem_standin.h", PKG / "plb" / "lbdem_plb.h", PKG / "plb" / "physunits_gpu.h",
            ROOT / "include" / "lbdem_gpu.h", lib]
    if not exe.exists() or exe.stat().st_mtime < max(p.stat().st_mtime for p in deps):
        cmd = [cxx, "-O2", "-std=c++17", "-Wall", f"-I{ROOT / 'include'}", f"-I{PKG / 'plb'}",
               f"-I{PKG / 'examples'}", str(src), f"-L{lib.parent}", "-llbdem_gb300",
               f"-Wl,-rpath,{lib.parent}", "-o", str(exe)]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def run_example(steps, prec, trace, every):
    exe = build_example()
    return subprocess.run([str(exe), str(steps), prec, str(trace), str(every)], capture_output=True, text=True)


def test_example_builds_and_needs_a_gpu(lbdem_lib, tmp_path):
    torch = pytest.importorskip("torch")
    exe = build_example()
    assert exe.exists()
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = run_example(2, "fp64", tmp_path / "c.txt", 1)
    assert r.returncode == 77, r.stderr


def test_multisphere_check_builds_and_needs_a_gpu(lbdem_lib):
    torch = pytest.importorskip("torch")
    exe = build_example("multisphere_check")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert subprocess.run([str(exe)], capture_output=True, text=True).returncode == 77


@pytest.mark.gpu
def test_multisphere_members_use_translation_only(gpu):
    exe = build_example("multisphere_check")
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_channel_example_builds_and_needs_a_gpu(lbdem_lib):
    torch = pytest.importorskip("torch")
    exe = build_example("channel")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert subprocess.run([str(exe), "3"], capture_output=True, text=True).returncode == 77


@pytest.mark.gpu
def test_channel_example_fused_equals_explicit(gpu, oracle):
    """The reference's per-step computeAverageDensity + Zhang functional calls and the
    fused pressure drop give the same channel (box sums differ only in summation order).
    The shim's field export (solid fraction, owner tag, surface velocity) covers
    exactly the cells the oracle's voxelization of the held sphere covers."""
    import json
    exe = build_example("channel")
    out = {}
    for mode in ("explicit", "fused"):
        r = subprocess.run([str(exe), "300", mode], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out[mode] = json.loads(r.stdout)
    assert out["fused"]["mean_ux"] > 1e-4
    assert out["fused"]["fx"] > 0                       # drag on the held sphere points downstream
    # the held sphere: physical centre (32.5, 12.5, 12.5) = lattice (32, 12, 12), radius 4, tag 1
    ol = oracle.OracleLattice(64, 24, 24, 1 / 0.6, periodic=(1, 0, 0))
    ol.set_particles(np.array([[32.0, 12.0, 12.0]]), np.zeros((1, 3)), np.zeros((1, 3)), np.array([4.0]),
                     np.array([1], dtype=np.int32))
    covered = int(np.count_nonzero(ol.state()["sf"] > 0))
    assert covered > 400
    for mode in out:
        assert out[mode]["solid_cells"] == covered
        assert out[mode]["owned_cells"] == covered
        assert out[mode]["max_up"] == 0.0
    for k in ("mean_ux", "fx"):
        assert abs(out["fused"][k] - out["explicit"][k]) <= 1e-10 * abs(out["explicit"][k])


def oracle_trace(oracle, steps):
    """The example program's loop on the CPU oracle: same sphere, same integrator."""
    nx, ny, nz, tau, radius, rho_s, g = 60, 60, 180, 0.6, 5.0, 1.5, 1e-5
    ol = oracle.OracleLattice(nx, ny, nz, 1.0 / tau, periodic=(0, 0, 0), threads=os.cpu_count() or 1)
    x = [30.5, 30.5, 150.5]
    v = [0.0, 0.0, 0.0]
    w = [0.0, 0.0, 0.0]
    m = rho_s * 4.0 / 3.0 * math.pi * radius * radius * radius
    inertia = 0.4 * m * radius * radius
    grav = [0.0, 0.0, -g * (rho_s - 1.0) / rho_s]
    dt = 1.0 / 10
    out = []
    for it in range(steps):
        ol.set_particles(np.array([[x[0] - 0.5, x[1] - 0.5, x[2] - 0.5]]), np.array([v]), np.array([w]),
                         np.array([radius]), np.array([1], dtype=np.int32))
        ol.collide_and_stream()
        F, T = ol.get_forces()
        f, t = F[0], T[0]
        for _ in range(10):
            for d in range(3):
                a = f[d] / m + grav[d]
                x[d] += v[d] * dt + 0.5 * a * dt * dt
                v[d] += a * dt
                w[d] += t[d] / inertia * dt
        out.append((it, x[2] - 0.5, v[2], f[2]))
    return np.array(out)


@pytest.mark.gpu
def test_example_matches_oracle_first_cycles(gpu, oracle, tmp_path):
    trace = tmp_path / "coords.txt"
    r = run_example(20, "fp64", trace, 1)
    assert r.returncode == 0, r.stderr
    got = np.loadtxt(trace)
    want = oracle_trace(oracle, 20)
    assert got.shape == want.shape
    for col, name in ((1, "z"), (2, "vz"), (3, "fz")):
        scale = np.max(np.abs(want[:, col]))
        assert np.max(np.abs(got[:, col] - want[:, col])) <= 1e-9 * scale, name


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_sphere_settles(gpu, tmp_path, prec):
    trace = tmp_path / "coords.txt"
    r = run_example(2000, prec, trace, 10)
    assert r.returncode == 0, r.stderr
    t, z, vz, fz = np.loadtxt(trace).T
    m = 1.5 * 4.0 / 3.0 * math.pi * 125.0
    weight = m * 1e-5 * 0.5 / 1.5               # buoyant weight the drag must approach
    assert z[-1] < z[0] - 0.5                    # it falls
    assert np.all(vz[1:] < 0)
    assert np.all(fz[1:] > 0)                    # drag opposes the motion
    assert 0.5 * weight < fz[-1] < 1.05 * weight
    assert abs(vz[-1]) > abs(vz[len(vz) // 2])   # still accelerating towards terminal velocity
