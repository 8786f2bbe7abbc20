"""Synthetic particle workloads for the PSM step (seeded, host side).

A LIGGGHTS run hands the coupling its local atoms followed by ghost images
(periodic copies carrying the owner's tag; src/ibDataExchangeWrappers3D.hh:48,62).
Without LIGGGHTS, this module produces the same kind of list:

* ``suspension``: non-overlapping spheres at uniform random centres by random
  sequential addition (monodisperse or radius ~ U[rmin, rmax]), velocities
  N(0, v_std) per component and angular velocities N(0, w_std);
* ``with_ghosts``: appends the periodic images whose bounding box reaches the
  lattice, axis by axis (x, then y, then z, images of earlier images included),
  the order in which LAMMPS builds ghost atoms;
* ``advance``: prescribed kinematics, x += v per step with periodic wrap;
* ``channels``: many pressure-driven rectangular channels of uneven size, the
  domains of a batch.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Particles:
    x: np.ndarray      # [n, 3] lattice units
    v: np.ndarray      # [n, 3] lattice units per step
    w: np.ndarray      # [n, 3] rad per step
    r: np.ndarray      # [n]
    tag: np.ndarray    # [n] int32, LIGGGHTS tags (1-based)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    def copy(self) -> "Particles":
        return Particles(self.x.copy(), self.v.copy(), self.w.copy(), self.r.copy(), self.tag.copy())


def _min_image(d: np.ndarray, L: np.ndarray, periodic) -> np.ndarray:
    d = d.copy()
    for k in range(3):
        if periodic[k]:
            d[..., k] -= L[k] * np.round(d[..., k] / L[k])
    return d


def suspension(shape, n_max: int | None = None, radius=8.0, rmin=None, rmax=None, phi_target=None,
               seed: int = 0, v_std=0.01, w_std=1e-3, periodic=(1, 1, 1), gap=0.0,
               max_trials: int = 2_000_000) -> Particles:
    """Random sequential addition of non-overlapping spheres.

    Monodisperse with ``radius`` unless ``rmin``/``rmax`` are given (radius
    U[rmin, rmax]).  Stops at ``n_max`` spheres or at solid volume fraction
    ``phi_target``.  Non-periodic axes keep spheres one radius plus two cells
    away from the walls.
    """
    rng = np.random.default_rng(seed)
    L = np.asarray(shape, dtype=np.float64)
    vol = float(np.prod(L))
    poly = rmin is not None and rmax is not None
    rbig = float(rmax if poly else radius)
    # uniform grid of buckets for the overlap test
    cell = 2.0 * rbig + gap
    nb = np.maximum((L // cell).astype(int), 1)
    buckets: dict[tuple, list[int]] = {}
    xs: list[np.ndarray] = []
    rs: list[float] = []
    phi = 0.0
    trials = 0
    while trials < max_trials:
        if n_max is not None and len(xs) >= n_max:
            break
        if phi_target is not None and phi >= phi_target:
            break
        trials += 1
        r = float(rng.uniform(rmin, rmax)) if poly else float(radius)
        p = rng.uniform(0.0, 1.0, 3) * L
        ok = True
        for k in range(3):
            if not periodic[k] and (p[k] < r + 2.0 or p[k] > L[k] - r - 3.0):
                ok = False
        if not ok:
            continue
        b = tuple((p // (L / nb)).astype(int) % nb)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    key = ((b[0] + dx) % nb[0], (b[1] + dy) % nb[1], (b[2] + dz) % nb[2])
                    for j in buckets.get(key, ()):
                        d = _min_image(p - xs[j], L, periodic)
                        if np.dot(d, d) < (r + rs[j] + gap) ** 2:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if not ok:
            continue
        buckets.setdefault(b, []).append(len(xs))
        xs.append(p)
        rs.append(r)
        phi += 4.0 / 3.0 * np.pi * r ** 3 / vol
    n = len(xs)
    x = np.array(xs).reshape(n, 3)
    v = rng.normal(0.0, v_std, (n, 3))
    w = rng.normal(0.0, w_std, (n, 3))
    return Particles(x, v, w, np.array(rs, dtype=np.float64), np.arange(1, n + 1, dtype=np.int32))


def with_ghosts(p: Particles, shape, periodic=(1, 1, 1)) -> Particles:
    """Locals followed by periodic images whose bounding box reaches the lattice."""
    x, v, w, r, tag = [a.copy() for a in (p.x, p.v, p.w, p.r, p.tag)]
    for k in range(3):
        if not periodic[k]:
            continue
        L = float(shape[k])
        lo = x[:, k] - r - 2.0
        hi = x[:, k] + r + 2.0
        plus = np.nonzero(lo < 0.0)[0]          # image at x + L covers the far side
        minus = np.nonzero(hi > L - 1.0)[0]     # image at x - L covers the near side
        idx = np.concatenate([plus, minus])
        shift = np.concatenate([np.full(plus.size, L), np.full(minus.size, -L)])
        xi = x[idx].copy()
        xi[:, k] += shift
        x = np.concatenate([x, xi])
        v = np.concatenate([v, v[idx]])
        w = np.concatenate([w, w[idx]])
        r = np.concatenate([r, r[idx]])
        tag = np.concatenate([tag, tag[idx]])
    return Particles(np.ascontiguousarray(x), np.ascontiguousarray(v), np.ascontiguousarray(w),
                     np.ascontiguousarray(r), np.ascontiguousarray(tag, dtype=np.int32))


def advance(p: Particles, shape, periodic=(1, 1, 1), steps: int = 1) -> Particles:
    """Prescribed kinematics: x += v per step, wrapped into [0, L) on periodic axes."""
    q = p.copy()
    L = np.asarray(shape, dtype=np.float64)
    for _ in range(steps):
        q.x = q.x + q.v
        for k in range(3):
            if periodic[k]:
                q.x[:, k] = np.mod(q.x[:, k], L[k])
    return q


def shuttle(p0: Particles, shape, step: int, half_period: int, periodic=(1, 1, 1)) -> Particles:
    """Prescribed kinematics that stay near the seeded placement: every particle
    moves with its seeded velocity v (and angular velocity w) for half_period
    steps, then with -v (-w) for half_period steps, and so on, so |v| and |w|
    keep their seeded distributions at every step while the displacement stays
    within half_period |v|.  Returns the particles at the given step: positions
    after `step` steps, and the velocities of the step that starts there."""
    h = int(half_period)
    k, t = divmod(int(step), 2 * h)
    disp = t if t <= h else 2 * h - t          # net steps of +v after `step` steps
    sign = 1.0 if t < h else -1.0
    L = np.asarray(shape, dtype=np.float64)
    x = p0.x + disp * p0.v
    for a in range(3):
        if periodic[a]:
            x[:, a] = np.mod(x[:, a], L[a])
    return Particles(x, sign * p0.v, sign * p0.w, p0.r.copy(), p0.tag.copy())


def monodisperse_256(seed: int = 2024) -> tuple[tuple[int, int, int], Particles]:
    """Periodic 256^3, 2000 spheres r = 8, v ~ N(0, 0.01), omega ~ N(0, 1e-3)."""
    shape = (256, 256, 256)
    return shape, suspension(shape, n_max=2000, radius=8.0, seed=seed)


def polydisperse_512(seed: int = 2025) -> tuple[tuple[int, int, int], Particles]:
    """Periodic 512x256x256, r ~ U[4, 10] until solid fraction 0.30."""
    shape = (512, 256, 256)
    return shape, suspension(shape, rmin=4.0, rmax=10.0, phi_target=0.30, seed=seed)


def channels(n_domains: int = 512, seed: int = 2026, tau: float = 0.6, rho_in: float = 1.0,
             rho_out: float = 0.999, flow_axis: int = 2) -> list[tuple[dict, Particles]]:
    """Independent channels: length U{64..160} along the flow, square cross-section
    U{24..48}, walls on the four sides, periodic along the flow and driven by the
    Zhang pressure drop between the first and last plane (interior rows, as
    examples/showcaseRectChannel); 1..40 spheres of radius U[3, 6] per channel
    (fewer where random sequential addition does not fit them), v ~ N(0, 0.01),
    omega ~ N(0, 1e-3).  flow_axis 2 (default) stores the flow along z, the
    fastest-varying axis of the layout (long rows for the collide-stream
    segments); flow_axis 0 keeps it along x.  The same seed gives mirror images
    of the same channels in either orientation.  Returns (domain, locals)
    pairs; a domain's max_particles leaves room for the periodic images."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_domains):
        lx = int(rng.integers(64, 161))
        l = int(rng.integers(24, 49))
        shape_x = (lx, l, l)
        want = int(rng.integers(1, 41))
        p = suspension(shape_x, n_max=want, rmin=3.0, rmax=6.0, seed=seed * 100003 + k, periodic=(1, 0, 0),
                       max_trials=20000)
        if flow_axis == 2:   # swap x and z: a reflection, so the angular velocity also changes sign
            shape = (l, l, lx)
            perm = [2, 1, 0]
            p = Particles(np.ascontiguousarray(p.x[:, perm]), np.ascontiguousarray(p.v[:, perm]),
                          np.ascontiguousarray(-p.w[:, perm]), p.r, p.tag)
            periodic = (0, 0, 1)
            inlet = [1, l - 2, 1, l - 2, 0, 0]
            outlet = [1, l - 2, 1, l - 2, lx - 1, lx - 1]
        else:
            shape = shape_x
            periodic = (1, 0, 0)
            inlet = [0, 0, 1, l - 2, 1, l - 2]
            outlet = [lx - 1, lx - 1, 1, l - 2, 1, l - 2]
        dom = {"shape": shape, "periodic": periodic, "omega": 1.0 / tau, "max_particles": 2 * max(p.n, 1),
               "drop": {"dimension": flow_axis, "inlet": inlet, "outlet": outlet, "rho_in": rho_in,
                        "rho_out": rho_out}}
        out.append((dom, p))
    return out
