"""The float fast path of the voxelization (lbdemcoupling-public_gb300/csrc/k_voxel.cu)
decides the reference's double comparisons exactly.

The kernel evaluates, in float, the cell distance dx^2 + (dy^2 + dz^2) (two
fused multiply-adds) and the 125 sub-cell sums (xs_i + ys_j) + zs_k from the
centre split x = xh + xl, and
falls back to the reference's double sequence (src/ibProcessors3D.hh:128-155)
only when a float value lies within M = 2^-19 (r + 4)^2 of its threshold.  This
emulates that float arithmetic in IEEE single precision on the CPU (numpy, one
rounding per operation; with and without the fused multiply-adds the compiler
may form) and checks, over random spheres up to r = 32 with centres anywhere in
[0, 2^23) (the kernel takes |x| < 2^24):
  * |dist_f - dist_d| <= 22 u (r + 3.2)^2 and |t_f - t_d| <= 27 u (r + 3.5)^2,
    u = 2^-24, the bounds the kernel's comment states;
  * M exceeds each bound plus the rounding of the threshold to float;
  * every comparison the float path treats as decided agrees with the double one.
"""
import numpy as np
import pytest

U = 2.0 ** -24
MARGIN_EXP = -19   # M = 2^MARGIN_EXP (r + 4)^2, SphereFast::margin in the kernel
SQRT3HALF = 0.8803408430829505
SUB_D = np.array([-0.4, -0.19999999999999996, 0.0, 0.20000000000000007, 0.4])   # double sub-cell offsets
SUB_F = np.array([-0.4, -0.2, 0.0, 0.2, 0.4], dtype=np.float32)                   # the kernel's float ones
f32 = np.float32


def _fma(a, b, c):
    """float fma(a, b, c): the exact product of two floats fits a double; one more
    rounding to float (a double rounding in rare ties, far below the bounds)."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def _dist_f(dxf, dyf, dzf, form):
    if form == "kernel":   # k_voxel.cu: __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)))
        return _fma(dxf, dxf, _fma(dyf, dyf, dzf * dzf))
    if form == "plain":
        return (dxf * dxf + dyf * dyf) + dzf * dzf
    return _fma(dzf, dzf, _fma(dyf, dyf, dxf * dxf))


def _split(x):
    xh = x.astype(np.float32)
    xl = (x - xh.astype(np.float64)).astype(np.float32)
    return xh, xl


def _spheres(seed, n):
    rng = np.random.default_rng(seed)
    r = np.concatenate([rng.uniform(0.5, 8.0, n // 2), rng.uniform(8.0, 32.0, n - n // 2)])
    scale = rng.choice([16.0, 4096.0, 2.0 ** 20, 2.0 ** 23], n)
    x = rng.uniform(0.0, 1.0, (n, 3)) * scale[:, None]
    return x, r


@pytest.mark.parametrize("form", ["kernel", "plain", "fused"])
def test_distance_band_decides_like_double(form):
    x, r = _spheres(3, 40)
    worst = 0.0
    for c, rad in zip(x, r):
        lo = np.trunc(c - rad - 2.0).astype(np.int64)
        hi = np.trunc(c + rad + 2.0).astype(np.int64)
        X, Y, Z = np.meshgrid(*[np.arange(lo[d], hi[d] + 1) for d in range(3)], indexing="ij")
        P = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
        dd = P.astype(np.float64) - c                                        # reference: X - x in double
        dist_d = (dd[:, 0] * dd[:, 0] + dd[:, 1] * dd[:, 1]) + dd[:, 2] * dd[:, 2]
        xh, xl = _split(c)
        df = (P.astype(np.float32) - xh) - xl                                # ((float)X - xh) - xl
        dist_f = _dist_f(df[:, 0], df[:, 1], df[:, 2], form).astype(np.float64)
        bound = 22 * U * (rad + 3.2) ** 2
        err = np.abs(dist_f - dist_d).max()
        worst = max(worst, err / bound)
        assert err <= bound
        Mf = np.ldexp(f32((f32(rad) + f32(4.0)) * (f32(rad) + f32(4.0))), MARGIN_EXP)
        M = float(Mf)
        rp = rad + SQRT3HALF
        rm = rad - SQRT3HALF
        dist_f32 = dist_f.astype(np.float32)
        for thr_d in (rp * rp, rm * rm):
            thr_f = f32(thr_d)
            assert M > bound + abs(float(thr_f) - thr_d)
            sure = np.abs(dist_f32 - thr_f) > Mf                          # fabsf(distf - thr) <= M: exact path
            assert np.array_equal((dist_f32 > thr_f)[sure], (dist_d > thr_d)[sure])
            assert np.array_equal((dist_f32 < thr_f)[sure], (dist_d < thr_d)[sure])
    assert worst > 0.0


@pytest.mark.parametrize("fused", [False, True])
def test_subcell_band_decides_like_double(fused):
    x, r = _spheres(4, 24)
    checked = 0
    for c, rad in zip(x, r):
        lo = np.trunc(c - rad - 2.0).astype(np.int64)
        hi = np.trunc(c + rad + 2.0).astype(np.int64)
        X, Y, Z = np.meshgrid(*[np.arange(lo[d], hi[d] + 1) for d in range(3)], indexing="ij")
        P = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
        dd = P.astype(np.float64) - c
        dist_d = (dd[:, 0] * dd[:, 0] + dd[:, 1] * dd[:, 1]) + dd[:, 2] * dd[:, 2]
        rp, rm = rad + SQRT3HALF, rad - SQRT3HALF
        shell = (dist_d <= rp * rp) & (dist_d >= rm * rm)                     # the cells that are counted
        P, dd = P[shell], dd[shell]
        if len(P) == 0:
            continue
        xh, xl = _split(c)
        df = (P.astype(np.float32) - xh) - xl
        # per axis, the five offsets: double reference and float kernel
        ad = dd[:, :, None] + SUB_D[None, None, :]                            # [cells, 3, 5]
        sq_d = ad * ad
        af = df[:, :, None] + SUB_F[None, None, :]
        t_d = (sq_d[:, 0, :, None, None] + sq_d[:, 1, None, :, None]) + sq_d[:, 2, None, None, :]
        if fused:
            xs = af[:, 0] * af[:, 0]
            a = _fma(af[:, 1, None, :], af[:, 1, None, :], xs[:, :, None])   # xs_i + ay_j^2
            t_f = _fma(af[:, 2, None, None, :], af[:, 2, None, None, :], a[:, :, :, None])
        else:
            sq_f = af * af
            t_f = (sq_f[:, 0, :, None, None] + sq_f[:, 1, None, :, None]) + sq_f[:, 2, None, None, :]
        t_f = t_f.astype(np.float64)
        bound = 27 * U * (rad + 3.5) ** 2
        assert np.abs(t_f - t_d).max() <= bound
        rsq_d = rad * rad
        rsq_f = f32(rsq_d)
        Mf = np.ldexp(f32((f32(rad) + f32(4.0)) * (f32(rad) + f32(4.0))), MARGIN_EXP)
        lo, hi = rsq_f - Mf, rsq_f + Mf                                  # float, as the kernel forms them
        assert float(rsq_f) - float(lo) > bound + abs(float(rsq_f) - rsq_d)
        assert float(hi) - float(rsq_f) > bound + abs(float(rsq_f) - rsq_d)
        t32 = t_f.astype(np.float32)
        # the resolve routine's rule: t < lo counted, t >= hi not, in between in double
        inside, outside = t32 < lo, ~(t32 < hi)
        assert np.all(t_d[inside] < rsq_d) and not np.any(t_d[outside] < rsq_d)
        # the fast count's rule: d = t - r^2 in float (exact near r^2); a slice is
        # decided when every |d| > M, and a sample is inside when d < 0
        d32 = (t32 - rsq_f).astype(np.float32)
        sure = np.abs(d32) > Mf
        assert np.array_equal((d32 < 0)[sure], (t_d < rsq_d)[sure])
        near = (t32 >= f32(0.5) * rsq_f) & (t32 <= f32(2.0) * rsq_f)          # Sterbenz: d exact
        assert np.array_equal(d32[near].astype(np.float64), t32[near].astype(np.float64) - float(rsq_f))
        checked += int(inside.sum() + outside.sum())
    assert checked > 10 ** 6


def test_box_distance_bounds_every_cell():
    """k_voxel.cu skips the per-cell classification of a (tile, sphere) pair when the
    float squared distance from the centre to the box of the sphere's cells in the
    tile exceeds (r + sqrt(3.1)/2)^2 + 2 M: the box distance is formed from the box
    corners' float offsets with the cells' operation order, so it is at most every
    cell's float distance (each rounding is monotone in non-negative terms), and
    every cell is then outside without the double-precision test."""
    x, r = _spheres(5, 40)
    rng = np.random.default_rng(6)
    checked = 0
    for c, rad in zip(x, r):
        xh, xl = _split(c)
        lo = np.trunc(c - rad - 2.0).astype(np.int64)
        for _ in range(40):
            a = lo + rng.integers(0, int(2 * rad + 4), 3)
            b = a + rng.integers(0, 8, 3)
            X, Y, Z = np.meshgrid(*[np.arange(a[d], b[d] + 1) for d in range(3)], indexing="ij")
            P = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
            df = (P.astype(np.float32) - xh) - xl
            cell = _dist_f(df[:, 0], df[:, 1], df[:, 2], "kernel")
            lo_f = (a.astype(np.float32) - xh) - xl
            hi_f = (b.astype(np.float32) - xh) - xl
            e = np.maximum(f32(0), np.maximum(lo_f, -hi_f)).astype(np.float32)
            box = _dist_f(e[None, 0], e[None, 1], e[None, 2], "kernel")[0]
            assert box <= cell.min()
            checked += len(P)
    assert checked > 10 ** 5
