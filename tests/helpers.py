"""Shared helpers for the parity tests: workloads and tolerance checks."""
from __future__ import annotations

import numpy as np


def rel_err(a, b) -> float:
    """max |a - b| / max |b| (norm-wise relative error of a field)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = float(np.max(np.abs(b))) if b.size else 0.0
    if scale == 0.0:
        return float(np.max(np.abs(a))) if a.size else 0.0
    return float(np.max(np.abs(a - b))) / scale


def small_suspension(shape, n, rmin, rmax, seed, periodic=(1, 1, 1), overlap=False, v_std=0.01, w_std=1e-3):
    """A few spheres, optionally overlapping (exercises the owner state machine)."""
    import workloads as W
    if overlap:
        rng = np.random.default_rng(seed)
        L = np.asarray(shape, dtype=np.float64)
        r = rng.uniform(rmin, rmax, n)
        x = rng.uniform(0, 1, (n, 3)) * L
        for k in range(3):
            if not periodic[k]:
                x[:, k] = np.clip(x[:, k], r + 2, L[k] - r - 3)
        v = rng.normal(0, v_std, (n, 3))
        w = rng.normal(0, w_std, (n, 3))
        return W.Particles(x, v, w, r, np.arange(1, n + 1, dtype=np.int32))
    return W.suspension(shape, n_max=n, rmin=rmin, rmax=rmax, seed=seed, periodic=periodic, v_std=v_std,
                        w_std=w_std)
