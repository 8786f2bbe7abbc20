"""The oracle pinned to the reference's own PSM code.

tests/golden/ref_psm_*.npz and ref_pressure.npz were produced by the reference
harness (the reference's SetSingleSphere3D, IBcompositeDynamics::collide,
SumForceTorque3D, ZhangPeriodicPressureFunctional3D and the PressureGradient /
PoiseuilleProfileAndPressureGradient functors compiled against Palabos/LIGGGHTS
stand-ins, tests/golden/make_golden.py).  The oracle must reproduce them bit
for bit.  Where the reference tree is present the harness is also run live on
further random cases.
"""
from pathlib import Path

import numpy as np
import pytest

import workloads as W
from helpers import small_suspension

GOLDEN = sorted((Path(__file__).resolve().parent / "golden").glob("ref_psm_*.npz"))


def replay_oracle(oracle, d):
    shape = tuple(int(s) for s in d["shape"])
    ol = oracle.OracleLattice(*shape, float(d["omega"]))
    ol.set_populations(d["f0"])
    init = set(int(s) for s in d["init_steps"])
    for s in range(int(d["steps"])):
        ol.set_particles(d[f"x{s}"], d[f"v{s}"], d[f"w{s}"], d[f"r{s}"], d[f"tag{s}"], init_vel=s in init)
        st = ol.state()
        yield s, "n", st["n"], d[f"n{s}"]
        yield s, "id", st["id"], d[f"id{s}"]
        yield s, "up", st["up"], d[f"up{s}"]
        ol.collide_and_stream()
        F, T = ol.get_forces()
        yield s, "cf", ol.state()["cf"], d[f"cf{s}"]
        yield s, "F", F, d[f"F{s}"]
        yield s, "T", T, d[f"T{s}"]
    yield -1, "f_final", ol.get_populations(), d["f_final"]


@pytest.mark.parametrize("path", GOLDEN, ids=[p.stem for p in GOLDEN])
def test_oracle_reproduces_reference_fixture_bitwise(oracle, path):
    d = np.load(path)
    for step, what, got, want in replay_oracle(oracle, d):
        assert np.array_equal(got, want), f"{path.stem} step {step}: {what} differs"


def test_fixtures_exist():
    assert len(GOLDEN) >= 2


@pytest.mark.parametrize("seed", [101, 202, 303])
def test_oracle_matches_reference_harness_live(oracle, seed):
    from oracle import ref_harness
    if not ref_harness.available():
        pytest.skip("reference tree not present")
    rng = np.random.default_rng(seed)
    shape = tuple(int(v) for v in rng.integers(6, 15, 3))
    omega = float(rng.uniform(0.8, 1.9))
    f0 = rng.standard_normal((19, *shape)) * 1e-3
    ref = ref_harness.RefLattice(*shape, omega)
    ol = oracle.OracleLattice(*shape, omega)
    ref.set_populations(f0)
    ol.set_populations(f0)
    p = small_suspension(shape, int(rng.integers(2, 9)), 0.6, 3.0, seed, overlap=True, v_std=0.4, w_std=0.1)
    for s in range(4):
        g = W.with_ghosts(p, shape)
        iv = bool(rng.integers(0, 2))
        ref.set_particles(g.x, g.v, g.w, g.r, g.tag, init_vel=iv)
        ol.set_particles(g.x, g.v, g.w, g.r, g.tag, init_vel=iv)
        a, b = ref.state(), ol.state()
        for k in ("sf", "id", "up"):
            assert np.array_equal(a[k], b[k]), f"step {s}: {k}"
        ref.collide_and_stream()
        ol.collide_and_stream()
        Fa, Ta = ref.get_forces()
        Fb, Tb = ol.get_forces()
        assert np.array_equal(ref.get_populations(), ol.get_populations()), f"step {s}: populations"
        assert np.array_equal(ref.state()["cf"], ol.state()["cf"]), f"step {s}: cell force"
        assert np.array_equal(Fa, Fb) and np.array_equal(Ta, Tb), f"step {s}: force/torque"
        p = W.advance(p, shape)


PRESSURE = Path(__file__).resolve().parent / "golden" / "ref_pressure.npz"


def test_oracle_reproduces_reference_pressure_fixture_bitwise(oracle):
    """Plane rescales of src/periodicPressureFunctionals3D.hh:137-159 on every axis
    and direction, and the initial states of :238-298 along every axis."""
    d = np.load(PRESSURE)
    shape = tuple(int(s) for s in d["shape"])
    ol = oracle.OracleLattice(*shape, 1 / 0.6)
    ol.set_populations(d["f0"])
    for box, (dim, direction, rho_target, rho_avg) in zip(d["boxes"], d["ops"]):
        ol.zhang_rescale(box, int(dim), int(direction), rho_target, rho_avg)
    got = ol.get_populations()
    assert np.array_equal(got, d["f_rescaled"])
    assert np.count_nonzero(got != d["f0"]) > 100
    for k, (kind, dim, p_hi, p_lo, u_max, n0, n1, n2) in enumerate(d["profiles"]):
        ol.init_profile(int(kind), p_hi, p_lo, u_max, (int(n0), int(n1), int(n2)), int(dim))
        assert np.array_equal(ol.get_populations(), d[f"profile{k}"]), f"profile {k}"


@pytest.mark.parametrize("seed", [7, 8])
def test_pressure_functionals_match_reference_harness_live(oracle, seed):
    from oracle import ref_harness
    if not ref_harness.available():
        pytest.skip("reference tree not present")
    rng = np.random.default_rng(seed)
    shape = tuple(int(v) for v in rng.integers(4, 13, 3))
    ref = ref_harness.RefLattice(*shape, 1 / 0.6)
    ol = oracle.OracleLattice(*shape, 1 / 0.6)
    f0 = rng.standard_normal((19, *shape)) * 1e-3
    ref.set_populations(f0)
    ol.set_populations(f0)
    for k in range(18):
        dim, direction = k % 3, int(rng.choice([-1, 1]))
        box = []
        for a in range(3):
            lo = int(rng.integers(0, shape[a]))
            hi = lo if a == dim else int(rng.integers(lo, shape[a]))
            box += [lo, hi]
        rho_target, rho_avg = 1 + rng.uniform(-0.02, 0.02), 1 + rng.uniform(-0.02, 0.02)
        ref.zhang_rescale(box, dim, direction, rho_target, rho_avg)
        ol.zhang_rescale(box, dim, direction, rho_target, rho_avg)
    assert np.array_equal(ref.get_populations(), ol.get_populations())
    for kind in (0, 1):
        for dim in range(3):
            n = [s - int(rng.integers(0, 2)) for s in shape]
            args = (kind, 1 + rng.uniform(0, 0.02), 1 - rng.uniform(0, 0.02), rng.uniform(0, 0.08), n, dim)
            ref.init_profile(*args)
            ol.init_profile(*args)
            assert np.array_equal(ref.get_populations(), ol.get_populations()), (kind, dim)
