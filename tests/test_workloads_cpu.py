"""Seeded synthetic workloads (workloads.py): the prescribed kinematics and the
two storage orientations of the batched channels."""
import numpy as np

import workloads as W


def test_shuttle_is_x_plus_v_with_reversals():
    shape = (40, 36, 44)
    p = W.suspension(shape, n_max=12, radius=3.0, seed=5)
    h = 7
    q = W.shuttle(p, shape, 0, h)
    assert np.array_equal(q.x, p.x) and np.array_equal(q.v, p.v) and np.array_equal(q.w, p.w)
    for s in range(1, 5 * h + 3):
        nxt = W.shuttle(p, shape, s, h)
        step = np.mod(q.x + q.v, np.asarray(shape, dtype=np.float64))   # x += v with the previous step's v
        d = np.abs(nxt.x - step)
        d = np.minimum(d, np.asarray(shape) - d)
        assert d.max() < 1e-9, s
        sign = 1.0 if (s // h) % 2 == 0 else -1.0
        assert np.array_equal(nxt.v, sign * p.v) and np.array_equal(nxt.w, sign * p.w)
        # displacement stays within one half period of travel
        disp = np.abs(nxt.x - p.x)
        disp = np.minimum(disp, np.asarray(shape) - disp)
        assert np.all(disp <= h * np.abs(p.v) + 1e-9)
        q = nxt


def test_channels_two_orientations_are_mirror_images():
    a = W.channels(n_domains=6, seed=11, flow_axis=0)
    b = W.channels(n_domains=6, seed=11, flow_axis=2)
    perm = [2, 1, 0]
    for (da, pa), (db, pb) in zip(a, b):
        assert db["shape"] == tuple(da["shape"][k] for k in perm)
        assert db["periodic"] == (0, 0, 1) and da["periodic"] == (1, 0, 0)
        assert db["drop"]["dimension"] == 2 and da["drop"]["dimension"] == 0
        # inlet / outlet boxes: [x0, x1, y0, y1, z0, z1] with x and z swapped
        for key in ("inlet", "outlet"):
            ba, bb = da["drop"][key], db["drop"][key]
            assert bb == [ba[4], ba[5], ba[2], ba[3], ba[0], ba[1]]
        assert np.array_equal(pb.x, pa.x[:, perm]) and np.array_equal(pb.v, pa.v[:, perm])
        assert np.array_equal(pb.w, -pa.w[:, perm])            # axial vector under a reflection
        assert np.array_equal(pb.r, pa.r) and np.array_equal(pb.tag, pa.tag)


def _min_image_dist(a, b, L, periodic):
    d = a - b
    for k in range(3):
        if periodic[k]:
            d[..., k] -= L[k] * np.round(d[..., k] / L[k])
    return np.sqrt((d * d).sum(-1))


def test_suspension_places_non_overlapping_spheres():
    """Random sequential addition: no two spheres overlap (minimum image on periodic
    axes), walls are kept at a radius plus two cells, the solid fraction target
    stops the insertion, and a seed reproduces the same list."""
    shape = (48, 40, 56)
    L = np.asarray(shape, dtype=np.float64)
    for periodic in ((1, 1, 1), (1, 0, 0), (0, 0, 1)):
        p = W.suspension(shape, rmin=2.0, rmax=5.0, phi_target=0.2, seed=9, periodic=periodic)
        assert p.n > 20
        for i in range(p.n):
            d = _min_image_dist(p.x[i][None, :], p.x, L, periodic)
            d[i] = np.inf
            assert np.all(d >= p.r[i] + p.r - 1e-9), i
        for k in range(3):
            if not periodic[k]:
                assert np.all(p.x[:, k] >= p.r + 2.0) and np.all(p.x[:, k] <= L[k] - p.r - 3.0)
        phi = (4.0 / 3.0 * np.pi * p.r ** 3).sum() / L.prod()
        assert 0.2 <= phi < 0.2 + 4.0 / 3.0 * np.pi * 5.0 ** 3 / L.prod()
        assert np.all((p.r >= 2.0) & (p.r <= 5.0))
        assert np.array_equal(p.tag, np.arange(1, p.n + 1))
        q = W.suspension(shape, rmin=2.0, rmax=5.0, phi_target=0.2, seed=9, periodic=periodic)
        assert np.array_equal(p.x, q.x) and np.array_equal(p.r, q.r) and np.array_equal(p.v, q.v)


def test_with_ghosts_covers_the_periodic_faces():
    """Locals come first, in order; every image is a local shifted by whole lattice
    lengths along periodic axes, carries its owner's tag, velocity, angular
    velocity and radius, and reaches the lattice (its box x +- (r + 2), truncated toward
    zero as src/ibProcessors3D.h:43-45 does, overlaps the cells 0 .. L - 1); a sphere
    whose box crosses a periodic face has an image on the other side."""
    shape = (32, 24, 40)
    L = np.asarray(shape, dtype=np.float64)
    for periodic in ((1, 1, 1), (0, 1, 0)):
        p = W.suspension(shape, n_max=30, rmin=2.0, rmax=4.5, seed=4, periodic=periodic)
        g = W.with_ghosts(p, shape, periodic)
        assert np.array_equal(g.x[:p.n], p.x) and np.array_equal(g.tag[:p.n], p.tag)
        owner = {int(t): i for i, t in enumerate(p.tag)}
        for k in range(p.n, g.n):
            i = owner[int(g.tag[k])]
            shift = (g.x[k] - p.x[i]) / L
            assert np.allclose(shift, np.round(shift), atol=1e-12)
            for a in range(3):
                assert periodic[a] or shift[a] == 0.0
            assert g.r[k] == p.r[i] and np.array_equal(g.v[k], p.v[i]) and np.array_equal(g.w[k], p.w[i])
            lo, hi = np.trunc(g.x[k] - g.r[k] - 2.0), np.trunc(g.x[k] + g.r[k] + 2.0)
            assert np.all(hi >= 0.0) and np.all(lo <= L - 1.0)
        for i in range(p.n):
            for a in range(3):
                if not periodic[a]:
                    continue
                crosses = p.x[i, a] - p.r[i] - 2.0 < 0.0 or p.x[i, a] + p.r[i] + 2.0 > L[a] - 1.0
                if crosses:
                    img = (g.tag == p.tag[i]) & (np.arange(g.n) >= p.n)
                    assert np.any(np.abs(g.x[img, a] - p.x[i, a]) == L[a]), (i, a)
