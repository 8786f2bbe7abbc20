"""Generates tests/golden/ref_psm_*.npz and ref_pressure.npz from the reference harness.

The harness runs the LBDEMcoupling reference's own SetSingleSphere3D,
IBcompositeDynamics::collide, SumForceTorque3D, ZhangPeriodicPressureFunctional3D
and the PressureGradient / PoiseuilleProfileAndPressureGradient functors
(compiled from the reference tree against Palabos/LIGGGHTS stand-ins,
oracle/ref_harness).  The ref_psm fixtures record, for a seeded case, the
particle lists and the reference's outputs after every coupling cycle; the
ref_pressure fixture the populations after a sequence of plane rescales and
the initial states of both functors along each axis.  Needs the reference
tree; run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT), str(ROOT / "lbdemcoupling-public_gb300"), str(ROOT / "tests")]

from oracle import ref_harness  # noqa: E402
import workloads as W  # noqa: E402
from helpers import small_suspension  # noqa: E402

CASES = {
    # name: shape, omega, n spheres, rmin, rmax, seed, steps, init_vel steps
    "ref_psm_overlap": ((12, 10, 14), 1 / 0.6, 5, 1.5, 3.5, 21, 4, (0, 3)),
    "ref_psm_dense": ((10, 12, 9), 1 / 0.55, 8, 0.7, 2.6, 5, 3, (1,)),
}


def make(name, shape, omega, n, rmin, rmax, seed, steps, init_steps):
    rng = np.random.default_rng(seed)
    f0 = rng.standard_normal((19, *shape)) * 1e-3
    ref = ref_harness.RefLattice(*shape, omega)
    ref.set_populations(f0)
    p = small_suspension(shape, n, rmin, rmax, seed, overlap=True, v_std=0.3, w_std=0.05)
    out = {"shape": np.array(shape), "omega": np.array(omega), "seed": np.array(seed), "f0": f0,
           "init_steps": np.array(init_steps, dtype=np.int32)}
    for s in range(steps):
        g = W.with_ghosts(p, shape)
        ref.set_particles(g.x, g.v, g.w, g.r, g.tag, init_vel=s in init_steps)
        st = ref.state()
        out[f"x{s}"], out[f"v{s}"], out[f"w{s}"], out[f"r{s}"], out[f"tag{s}"] = g.x, g.v, g.w, g.r, g.tag
        out[f"n{s}"] = np.rint(st["sf"] * 125).astype(np.uint8)
        out[f"id{s}"] = st["id"]
        out[f"up{s}"] = st["up"]
        ref.collide_and_stream()
        F, T = ref.get_forces()
        st = ref.state()
        out[f"cf{s}"], out[f"F{s}"], out[f"T{s}"] = st["cf"], F, T
        p = W.advance(p, shape)
    out["steps"] = np.array(steps)
    out["f_final"] = ref.get_populations()
    path = Path(__file__).resolve().parent / f"{name}.npz"
    np.savez_compressed(path, **out)
    print(path, path.stat().st_size)


def make_pressure(name="ref_pressure", shape=(6, 5, 7), seed=41):
    """The Zhang rescale (ZhangPeriodicPressureFunctional3D::process) on planes
    along each axis in both directions, applied in sequence to seeded
    populations, and the PressureGradient / PoiseuilleProfileAndPressureGradient
    initial states for each flow axis."""
    rng = np.random.default_rng(seed)
    f0 = rng.standard_normal((19, *shape)) * 1e-3
    ref = ref_harness.RefLattice(*shape, 1 / 0.6)
    ref.set_populations(f0)
    boxes, ops = [], []
    for k in range(12):
        dim, direction = k % 3, (1 if (k // 3) % 2 == 0 else -1)
        plane = int(rng.integers(0, shape[dim]))
        box = []
        for a in range(3):
            if a == dim:
                box += [plane, plane]
            else:
                lo = int(rng.integers(0, shape[a]))
                box += [lo, int(rng.integers(lo, shape[a]))]
        rho_target, rho_avg = 1 + rng.uniform(-0.01, 0.01), 1 + rng.uniform(-0.01, 0.01)
        ref.zhang_rescale(box, dim, direction, rho_target, rho_avg)
        boxes.append(box)
        ops.append((dim, direction, rho_target, rho_avg))
    out = {"shape": np.array(shape), "f0": f0, "boxes": np.array(boxes, dtype=np.int32),
           "ops": np.array(ops, dtype=np.float64), "f_rescaled": ref.get_populations()}
    profiles = []
    for kind in (0, 1):
        for dim in range(3):
            n = list(shape)
            n[dim] -= (kind + dim) % 2            # grid sizes as given (the channel case passes nx - 1)
            p_hi, p_lo, u_max = 1 + rng.uniform(0, 0.01), 1 - rng.uniform(0, 0.01), rng.uniform(0, 0.05)
            ref.init_profile(kind, p_hi, p_lo, u_max, n, dim)
            profiles.append([kind, dim, p_hi, p_lo, u_max, *n])
            out[f"profile{len(profiles) - 1}"] = ref.get_populations()
    out["profiles"] = np.array(profiles, dtype=np.float64)
    path = Path(__file__).resolve().parent / f"{name}.npz"
    np.savez_compressed(path, **out)
    print(path, path.stat().st_size)


if __name__ == "__main__":
    for name, args in CASES.items():
        make(name, *args)
    make_pressure()
