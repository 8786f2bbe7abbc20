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
