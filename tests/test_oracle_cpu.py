"""The CPU oracle against an independent pure-Python restatement of the
reference (tests/pyref.py) and against physical invariants."""
import math

import numpy as np
import pytest

import pyref
from helpers import rel_err


def test_subcell_constants():
    # -0.5 + (i + 0.5) * (1./5.) in double, src/ibProcessors3D.hh:141-147
    d = [-0.5 + (i + 0.5) * (1.0 / 5.0) for i in range(5)]
    assert d == [-0.4, -0.19999999999999996, 0.0, 0.20000000000000007, 0.4]
    assert math.sqrt(3.1) / 2.0 == 0.8803408430829505
    assert (1.0 / 125.0) * 125.0 == 1.0   # so "return 1" and n = 125 are the same solid fraction


@pytest.mark.parametrize("seed", range(4))
def test_solid_count_matches_pyref(oracle, seed):
    rng = np.random.default_rng(seed)
    for _ in range(400):
        r = rng.uniform(0.5, 9.0)
        d = rng.uniform(-r - 2, r + 2, 3)
        n = oracle.solid_count(*d, r)
        assert pyref.calc_solid_fraction(*d, r) == (1.0 / 125.0) * n


def test_solid_count_known_answers(oracle):
    assert oracle.solid_count(0, 0, 0, 3.0) == 125
    assert oracle.solid_count(10.0, 0, 0, 3.0) == 0
    # cell centre on the sphere surface: the plane x = 3 splits the 5 x-slices 3:2 minus the curvature
    assert oracle.solid_count(3.0, 0.0, 0.0, 3.0) == 50
    # exactly symmetric offsets give symmetric counts
    assert oracle.solid_count(2.5, 0, 0, 3.0) == oracle.solid_count(-2.5, 0, 0, 3.0)


def _tiny_particles(seed, shape, n=4):
    rng = np.random.default_rng(seed)
    L = np.asarray(shape, float)
    x = rng.uniform(-2, 1, (n, 3)) * 0 + rng.uniform(0, 1, (n, 3)) * L
    v = rng.normal(0, 0.3, (n, 3))
    w = rng.normal(0, 0.05, (n, 3))
    r = rng.uniform(0.8, 3.2, n)
    tag = rng.permutation(np.arange(1, n + 1)).astype(np.int32)
    tag[-1] = tag[0]  # an image sharing its owner's tag
    x[-1] = x[0] + np.array([L[0], 0, 0]) * (1 if x[0, 0] < L[0] / 2 else -1)
    return x, v, w, r, tag


@pytest.mark.parametrize("seed", range(3))
def test_voxelization_matches_pyref_bitwise(oracle, seed):
    shape = (9, 7, 8)
    ol = oracle.OracleLattice(*shape, 1.2)
    st = {"sf": np.zeros(shape), "id": np.zeros(shape, np.int32), "up": np.zeros((3, *shape))}
    x, v, w, r, tag = _tiny_particles(seed, shape)
    for step in range(4):
        ol.set_particles(x, v, w, r, tag)
        pyref.set_spheres(st, shape, x, v, w, r, tag)
        o = ol.state()
        assert np.array_equal(o["sf"], st["sf"])
        assert np.array_equal(o["id"], st["id"])
        assert np.array_equal(o["up"], st["up"])
        x = x + v


@pytest.mark.parametrize("omega", [1.0 / 0.6, 1.0 / 0.55, 1.9])
def test_collide_and_force_sum_match_pyref(oracle, omega):
    shape = (6, 5, 7)
    rng = np.random.default_rng(11)
    f0 = rng.standard_normal((19, *shape)) * 1e-3
    ol = oracle.OracleLattice(*shape, omega)
    ol.set_populations(f0)
    x = np.array([[2.6, 2.1, 3.3], [4.4, 2.2, 1.0]])
    v = rng.normal(0, 0.02, (2, 3))
    w = rng.normal(0, 0.01, (2, 3))
    r = np.array([1.7, 1.3])
    tag = np.array([1, 2], dtype=np.int32)
    ol.set_particles(x, v, w, r, tag)
    st = ol.state()
    ol.collide_and_stream()
    F, T = ol.get_forces()
    # pure-Python collide of every cell, then push streaming (periodic)
    post = np.empty_like(f0)
    cf = np.zeros((3, *shape))
    for idx in np.ndindex(shape):
        fc, Fc = pyref.psm_collide(f0[(slice(None), *idx)], st["sf"][idx], st["up"][(slice(None), *idx)], omega)
        post[(slice(None), *idx)] = fc
        cf[(slice(None), *idx)] = Fc
    ref = np.empty_like(post)
    for i, c in enumerate(pyref.C):
        ref[i] = np.roll(post[i], shift=c, axis=(0, 1, 2))
    assert rel_err(ol.get_populations(), ref) <= 1e-14
    assert rel_err(ol.state()["cf"], cf) <= 1e-13
    Fp, Tp = pyref.sum_force_torque(shape, st["id"], cf, x, tag)
    assert np.allclose(F, Fp, rtol=1e-12, atol=1e-16)
    assert np.allclose(T, Tp, rtol=1e-12, atol=1e-16)
    assert np.abs(F).max() > 0


def test_mass_conservation_periodic(oracle):
    shape = (10, 12, 9)
    rng = np.random.default_rng(5)
    ol = oracle.OracleLattice(*shape, 1.4)
    f0 = rng.standard_normal((19, *shape)) * 1e-3
    ol.set_populations(f0)
    m0 = ol.mass()
    for _ in range(6):
        ol.collide_and_stream()
    assert abs(ol.mass() - m0) <= 1e-12 * m0


def _momentum(f):
    c = np.array(pyref.C, dtype=np.float64)
    return c.T @ np.asarray(f).reshape(19, -1).sum(axis=1)


def test_momentum_balance_periodic(oracle):
    """Periodic box without walls or body force: with no particles the fluid
    momentum is conserved; with moving spheres, each step changes it by minus
    the sum of the particle forces (the momentum exchange of the PSM collision,
    src/ibCompositeDynamics3D.hh:160-200), to rounding."""
    import workloads as W
    shape = (14, 12, 16)
    rng = np.random.default_rng(17)
    f0 = rng.standard_normal((19, *shape)) * 1e-3
    ol = oracle.OracleLattice(*shape, 1 / 0.6)
    ol.set_populations(f0)
    p0 = _momentum(ol.get_populations())
    for _ in range(5):
        ol.collide_and_stream()
    assert np.abs(_momentum(ol.get_populations()) - p0).max() <= 1e-14 * np.abs(f0).sum()

    ol = oracle.OracleLattice(*shape, 1 / 0.6)
    ol.set_populations(f0)
    p = W.suspension(shape, n_max=4, rmin=2.0, rmax=3.5, seed=5, v_std=0.05, w_std=0.01)
    total = 0.0
    for s in range(5):
        g = W.with_ghosts(p, shape)
        ol.set_particles(g.x, g.v, g.w, g.r, g.tag, init_vel=(s == 0))
        before = _momentum(ol.get_populations())
        ol.collide_and_stream()
        F, _ = ol.get_forces()
        gain = _momentum(ol.get_populations()) - before
        total += np.abs(F.sum(axis=0)).max()
        assert np.abs(gain + F.sum(axis=0)).max() <= 1e-12 * np.abs(F).sum(), s
        p = W.advance(p, shape)
    assert total > 1e-6                       # the spheres do exchange momentum


def test_mass_conservation_bounce_back_with_sphere(oracle):
    """Walls and a resting sphere in fluid at rest: mass is conserved, and a
    particle at rest in a fluid at rest feels no force."""
    shape = (12, 12, 14)
    ol = oracle.OracleLattice(*shape, 1.6, periodic=(0, 0, 0))
    x = np.array([[5.7, 6.2, 7.1]]); z = np.zeros((1, 3))
    ol.set_particles(x, z, z, np.array([3.3]), np.array([1], dtype=np.int32))
    m0 = ol.mass()
    for _ in range(4):
        ol.collide_and_stream()
    F, T = ol.get_forces()
    assert np.all(F == 0) and np.all(T == 0)
    assert abs(ol.mass() - m0) <= 1e-12 * m0


def test_sphere_on_axis_has_no_transverse_force(oracle):
    """A sphere on the symmetry axis of a closed box, moving along the axis."""
    shape = (15, 15, 30)
    ol = oracle.OracleLattice(*shape, 1.5, periodic=(0, 0, 0))
    x = np.array([[7.0, 7.0, 15.0]]); v = np.array([[0.0, 0.0, -0.02]]); z = np.zeros((1, 3))
    for _ in range(5):
        ol.set_particles(x, v, z, np.array([4.0]), np.array([1], dtype=np.int32))
        ol.collide_and_stream()
        F, T = ol.get_forces()
        assert F[0, 2] > 0  # drag opposes the motion
        assert abs(F[0, 0]) <= 1e-13 * abs(F[0, 2]) and abs(F[0, 1]) <= 1e-13 * abs(F[0, 2])
        assert np.abs(T).max() <= 1e-12 * abs(F[0, 2])


def test_equilibrium_is_a_fixed_point(oracle):
    ol = oracle.OracleLattice(8, 8, 8, 1.2)
    ol.init_equilibrium(0.02, (0.01, -0.02, 0.03))
    f0 = ol.get_populations()
    ol.collide_and_stream()
    assert rel_err(ol.get_populations(), f0) <= 1e-14


def test_fp32_oracle_tracks_fp64(oracle):
    shape = (12, 10, 14)
    rng = np.random.default_rng(2)
    f0 = rng.standard_normal((19, *shape)) * 1e-3
    x = np.array([[5.5, 4.9, 7.2]]); v = np.array([[0.01, 0.0, -0.02]]); w = np.array([[0.0, 0.01, 0.0]])
    res = []
    for prec in (0, 1):
        ol = oracle.OracleLattice(*shape, 1.5, precision=prec)
        ol.set_populations(f0)
        for _ in range(5):
            ol.set_particles(x, v, w, np.array([3.5]), np.array([1], dtype=np.int32))
            ol.collide_and_stream()
        res.append((ol.get_populations(), ol.get_forces()[0]))
    assert rel_err(res[1][0], res[0][0]) <= 1e-5
    assert rel_err(res[1][1], res[0][1]) <= 1e-4


def test_threads_do_not_change_results(oracle):
    if not oracle.has_openmp():
        pytest.skip("oracle built without OpenMP")
    shape = (16, 12, 10)
    rng = np.random.default_rng(9)
    f0 = rng.standard_normal((19, *shape)) * 1e-3
    x = np.array([[7.5, 5.5, 4.5], [2.0, 2.0, 2.0]]); v = rng.normal(0, 0.02, (2, 3)); w = np.zeros((2, 3))
    out = []
    for th in (1, 4):
        ol = oracle.OracleLattice(*shape, 1.3, threads=th)
        ol.set_populations(f0)
        for _ in range(3):
            ol.set_particles(x, v, w, np.array([3.0, 2.5]), np.array([1, 2], dtype=np.int32))
            ol.collide_and_stream()
        out.append((ol.get_populations(), ol.state()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1]["id"], out[1][1]["id"])
