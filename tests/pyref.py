"""Pure-Python restatement of the reference's voxelization, PSM collision and
force sum, used only to cross-check the C oracle on tiny lattices.

Python floats are IEEE doubles and Python never fuses a multiply-add, so the
voxelization here is the same double sequence as the reference's
(src/ibProcessors3D.hh:53-184) and must agree bit for bit with the oracle.
"""
from __future__ import annotations

import math

import numpy as np

SOLFRAC_MIN = 0.001
SOLFRAC_MAX = 0.999
C = [(0, 0, 0), (-1, 0, 0), (0, -1, 0), (0, 0, -1), (-1, -1, 0), (-1, 1, 0), (-1, 0, -1), (-1, 0, 1),
     (0, -1, -1), (0, -1, 1), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, -1, 0), (1, 0, 1), (1, 0, -1),
     (0, 1, 1), (0, 1, -1)]
W = [1 / 3] + [1 / 18] * 3 + [1 / 36] * 6 + [1 / 18] * 3 + [1 / 36] * 6


def calc_solid_fraction(dx_, dy_, dz_, r_):
    """src/ibProcessors3D.hh:117-158, returns sf."""
    slices = 5
    slice_width = 1.0 / slices
    fraction = 1.0 / (slices * slices * slices)
    sqrt3half = math.sqrt(3.1) / 2.0
    dist = dx_ * dx_ + dy_ * dy_ + dz_ * dz_
    r_p = r_ + sqrt3half
    if dist > r_p * r_p:
        return 0.0
    r_m = r_ - sqrt3half
    if dist < r_m * r_m:
        return 1.0
    r_sq = r_ * r_
    xs, ys, zs = [], [], []
    for i in range(slices):
        delta = -0.5 + (float(i) + 0.5) * slice_width
        dx = dx_ + delta
        xs.append(dx * dx)
        dy = dy_ + delta
        ys.append(dy * dy)
        dz = dz_ + delta
        zs.append(dz * dz)
    n = 0
    for i in range(slices):
        for j in range(slices):
            for k in range(slices):
                n += (xs[i] + ys[j] + zs[k] < r_sq)
    return fraction * float(n)


def trunc(v: float) -> int:
    return int(v)  # Python int() truncates toward zero, like double -> plint


def set_spheres(state, shape, x, v, w, r, tag):
    """SetSingleSphere3D::process for every sphere in order; state = dict(sf, id, up)."""
    sf_a, id_a, up_a = state["sf"], state["id"], state["up"]
    for s in range(len(r)):
        xs, vs, ws, rs, t = x[s], v[s], w[s], float(r[s]), int(tag[s])
        lo = [max(trunc(xs[d] - rs - 2), 0) for d in range(3)]
        hi = [min(trunc(xs[d] + rs + 2), shape[d] - 1) for d in range(3)]
        if any(lo[d] > hi[d] for d in range(3)):
            continue
        for iX in range(lo[0], hi[0] + 1):
            for iY in range(lo[1], hi[1] + 1):
                for iZ in range(lo[2], hi[2] + 1):
                    dx = float(iX) - xs[0]
                    dy = float(iY) - xs[1]
                    dz = float(iZ) - xs[2]
                    sf = calc_solid_fraction(dx, dy, dz, rs)
                    sf_old = sf_a[iX, iY, iZ]
                    id_old = id_a[iX, iY, iZ]
                    dec = int(sf > SOLFRAC_MIN) + 2 * int(sf_old > SOLFRAC_MIN)
                    setv = zero = False
                    if dec == 0:
                        zero = True
                    elif dec == 1:
                        setv = True
                    elif dec == 2:
                        zero = id_old == t
                    else:
                        setv = sf > sf_old or id_old == t
                    if zero:
                        sf_a[iX, iY, iZ] = 0.0
                        id_a[iX, iY, iZ] = 0
                        up_a[:, iX, iY, iZ] = 0.0
                    if setv:
                        up_a[0, iX, iY, iZ] = vs[0] + (ws[1] * dz - ws[2] * dy)
                        up_a[1, iX, iY, iZ] = vs[1] + (-ws[0] * dz + ws[2] * dx)
                        up_a[2, iX, iY, iZ] = vs[2] + (ws[0] * dy - ws[1] * dx)
                        sf_a[iX, iY, iZ] = sf
                        id_a[iX, iY, iZ] = t


def feq(i, rho_bar, inv_rho, j, j_sqr):
    cj = C[i][0] * j[0] + C[i][1] * j[1] + C[i][2] * j[2]
    return W[i] * (rho_bar + 3.0 * cj + inv_rho * (4.5 * cj * cj - 1.5 * j_sqr))


def psm_collide(f, sf, up, omega):
    """src/ibCompositeDynamics3D.hh:130-203 for one cell (list of 19); returns (f, F)."""
    f = list(f)
    f_pre = list(f) if sf > SOLFRAC_MIN else None
    F = [0.0, 0.0, 0.0]
    if sf <= SOLFRAC_MAX:
        rb = sum(f)
        j = [sum(C[i][d] * f[i] for i in range(19)) for d in range(3)]
        inv = 1.0 / (1.0 + rb)
        js = j[0] ** 2 + j[1] ** 2 + j[2] ** 2
        f = [f[i] * (1 - omega) + omega * feq(i, rb, inv, j, js) for i in range(19)]
    if sf < SOLFRAC_MIN:
        return f, F
    rb = sum(f)
    j = [sum(C[i][d] * f[i] for i in range(19)) for d in range(3)]
    inv = 1.0 / (1.0 + rb)
    js = j[0] ** 2 + j[1] ** 2 + j[2] ** 2
    fe = [feq(i, rb, inv, j, js) for i in range(19)]
    u = [up[d] * (1.0 + rb) for d in range(3)]
    us = u[0] ** 2 + u[1] ** 2 + u[2] ** 2
    fs = [feq(i, rb, inv, u, us) for i in range(19)]
    if sf > SOLFRAC_MAX:
        B, omB = 1.0, 0.0
    else:
        ooo = 1.0 / omega - 0.5
        B = sf * ooo / ((1.0 - sf) + ooo)
        omB = 1.0 - B
    f[0] = f_pre[0] + omB * (f[0] - f_pre[0]) + B * (fe[0] - fs[0])
    for i in range(1, 10):
        o = i + 9
        bb = B * ((f_pre[o] - fe[o]) - (f_pre[i] - fs[i]))
        bbo = B * ((f_pre[i] - fe[i]) - (f_pre[o] - fs[o]))
        f[i] = f_pre[i] + omB * (f[i] - f_pre[i]) + bb
        f[o] = f_pre[o] + omB * (f[o] - f_pre[o]) + bbo
        for d in range(3):
            F[d] -= C[i][d] * (bb - bbo)
    return f, F


def sum_force_torque(shape, ids, cf, x, tag):
    """src/ibProcessors3D.hh:203-263 with LAMMPS atom->map (lowest index per tag)."""
    n = len(tag)
    F = np.zeros((n, 3))
    T = np.zeros((n, 3))
    first = {}
    for i in range(n - 1, -1, -1):
        first[int(tag[i])] = i
    nx, ny, nz = shape
    for iX in range(nx):
        for iY in range(ny):
            for iZ in range(nz):
                t = int(ids[iX, iY, iZ])
                if t < 1 or t not in first:
                    continue
                k = first[t]
                d = [float(iX) - x[k][0], float(iY) - x[k][1], float(iZ) - x[k][2]]
                for a, L in enumerate(shape):
                    h = int(L / 2)
                    if d[a] > h:
                        d[a] -= L
                    elif d[a] < -h:
                        d[a] += L
                fx, fy, fz = (float(cf[q, iX, iY, iZ]) for q in range(3))
                F[k] += (fx, fy, fz)
                T[k] += (d[1] * fz - d[2] * fy, -d[0] * fz + d[2] * fx, d[0] * fy - d[1] * fx)
    return F, T
