"""GPU parity at the benchmarked configuration and at a dense polydisperse one.

* ``test_headline_workload``: the exact workload the benchmark times (periodic
  256^3, tau 0.55, 2000 spheres of radius 8 seeded as in bench.py, ghost images
  appended, prescribed kinematics), three coupling cycles against the CPU
  oracle on the same inputs:
    - sub-cell counts n and owner tags bit-identical in every cycle, in both
      forms;
    - FP64 form: particle surface velocity bit-identical, populations within
      1e-12 of max |f̄|, per-particle force and torque within
      1e-12 * sum_{cells of p} |f_cell| (torque: times the lattice extent);
    - FP32 deviation form: per-particle forces and torques within 1e-4 of
      max |F| of the FP64 oracle.
* ``test_dense_polydisperse``: radii U[4, 10] (the polydisperse workload's
  range) overlapping at high number density plus a cluster of small spheres:
  up to 170 spheres reach one 8^3 tile (mean about 16, eight tiles past the
  64-entry bin), so the tile-bin ordering and the bin-overflow path run at
  scale.  Same bars.
* ``test_dense_polydisperse_large_tags``: the same spheres with tags spread up to
  about 6000: the collide-stream kernel then looks owners up in the global
  tag -> slot map instead of its shared-memory copy (which holds tags below 2047).

Reference: src/ibProcessors3D.hh:53-184 (voxelization), :203-263 (force sum),
src/ibCompositeDynamics3D.hh:130-203 (collision).
"""
import os

import numpy as np
import pytest

import workloads as W
from helpers import rel_err

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

THREADS = os.cpu_count() or 1


def _scale(ost, tag, n):
    """sum_{cells owned by tag} |f_cell| at the first list entry of each tag."""
    ids = ost["id"].ravel()
    cf = np.abs(ost["cf"].astype(np.float64)).reshape(3, -1).sum(axis=0)
    sums = np.bincount(ids, weights=cf, minlength=int(tag.max()) + 1)
    _, first = np.unique(tag, return_index=True)
    s = np.zeros(n)
    s[first] = sums[tag[first]]
    return s


def _tile_load(g, shape, tile=8):
    """Spheres whose bounding box reaches each 8^3 tile (src/ibProcessors3D.h:43-45)."""
    nt = [(s + tile - 1) // tile for s in shape]
    cnt = np.zeros(nt, dtype=np.int64)
    for x, r in zip(g.x, g.r):
        lo = [max(int(x[d] - r - 2.0), 0) for d in range(3)]
        hi = [min(int(x[d] + r + 2.0), shape[d] - 1) for d in range(3)]
        if any(lo[d] > hi[d] for d in range(3)):
            continue
        cnt[lo[0] // tile:hi[0] // tile + 1, lo[1] // tile:hi[1] // tile + 1, lo[2] // tile:hi[2] // tile + 1] += 1
    return cnt


def _compare(gpu, oracle, shape, tau, tables, check_pops_every=True):
    n_max = max(g.n for g in tables)
    max_tag = int(max(g.tag.max() for g in tables)) + 1
    ol = oracle.OracleLattice(*shape, 1.0 / tau, threads=THREADS)
    fp64_forces = []
    with gpu.Lattice(*shape, 1.0 / tau, precision=gpu.PREC_FP64, max_particles=n_max, max_tag=max_tag,
                     max_radius=10.0) as L:
        for s, g in enumerate(tables):
            L.set_particles(g.x, g.v, g.w, g.r, g.tag)
            ol.set_particles(g.x, g.v, g.w, g.r, g.tag)
            ost = ol.state()
            assert np.array_equal(L.get_field(gpu.FIELD_SUBCELL_COUNT), ost["n"]), f"cycle {s}: counts"
            assert np.array_equal(L.get_field(gpu.FIELD_PARTICLE_ID), ost["id"]), f"cycle {s}: owner tags"
            assert np.array_equal(L.get_field(gpu.FIELD_PARTICLE_VELOCITY), ost["up"]), f"cycle {s}: uPart"
            del ost
            L.collide_and_stream()
            ol.collide_and_stream()
            Fg, Tg = L.get_forces()
            Fo, To = ol.get_forces()
            ost = ol.state()
            scale = _scale(ost, g.tag, g.n)
            del ost
            assert np.all(np.abs(Fg - Fo) <= 1e-12 * scale[:, None] + 1e-300), f"cycle {s}: FP64 forces"
            assert np.all(np.abs(Tg - To) <= 1e-12 * max(shape) * scale[:, None] + 1e-300), f"cycle {s}: torques"
            if check_pops_every or s == len(tables) - 1:
                e = rel_err(L.get_populations(), ol.get_populations())
                assert e <= 1e-12, f"cycle {s}: FP64 populations {e:.3e}"
            fp64_forces.append((Fo, To))
        assert L.device_errors() == 0
    assert max(np.abs(F).max() for F, _ in fp64_forces) > 0, "no force was exercised"

    # FP32 deviation form against the FP64 oracle's forces on the same inputs
    ol32 = oracle.OracleLattice(*shape, 1.0 / tau, threads=THREADS)
    with gpu.Lattice(*shape, 1.0 / tau, precision=gpu.PREC_FP32_DEV, max_particles=n_max, max_tag=max_tag,
                     max_radius=10.0) as L:
        for s, g in enumerate(tables):
            L.set_particles(g.x, g.v, g.w, g.r, g.tag)
            ol32.set_particles(g.x, g.v, g.w, g.r, g.tag)
            ost = ol32.state()
            assert np.array_equal(L.get_field(gpu.FIELD_SUBCELL_COUNT), ost["n"]), f"cycle {s}: FP32 counts"
            assert np.array_equal(L.get_field(gpu.FIELD_PARTICLE_ID), ost["id"]), f"cycle {s}: FP32 tags"
            del ost
            L.collide_and_stream()
            F32, T32 = L.get_forces()
            F64, T64 = fp64_forces[s]
            assert rel_err(F32, F64) <= 1e-4, f"cycle {s}: FP32 force error {rel_err(F32, F64):.3e}"
            assert rel_err(T32, T64) <= 1e-4, f"cycle {s}: FP32 torque error {rel_err(T32, T64):.3e}"
        assert L.device_errors() == 0


def test_headline_workload(gpu, oracle):
    """bench.py's 256^3 workload (workloads.monodisperse_256(2024), 2547 spheres
    with ghost images), three cycles."""
    shape, p = W.monodisperse_256(2024)
    assert p.n == 2000
    tables = []
    for _ in range(3):
        tables.append(W.with_ghosts(p, shape))
        p = W.advance(p, shape)
    assert tables[0].n > 2500 and np.all(tables[0].r == 8.0)
    _compare(gpu, oracle, shape, 0.55, tables, check_pops_every=False)


def _dense_polydisperse(tag_of):
    rng = np.random.default_rng(11)
    shape = (96, 96, 96)
    n_big, n_small = 700, 150
    x = np.concatenate([rng.uniform(0, 96, (n_big, 3)), 40.0 + rng.uniform(-2, 2, (n_small, 3))])
    r = np.concatenate([rng.uniform(4.0, 10.0, n_big), rng.uniform(0.6, 1.5, n_small)])
    n = n_big + n_small
    p = W.Particles(x, rng.normal(0, 0.01, (n, 3)), rng.normal(0, 1e-3, (n, 3)), r,
                    tag_of(np.arange(n)).astype(np.int32))
    tables = []
    for _ in range(3):
        tables.append(W.with_ghosts(p, shape))
        p = W.advance(p, shape)
    load = _tile_load(tables[0], shape)
    assert load.max() > 64 and (load >= 20).sum() >= 100 and r.max() > 9.5
    return shape, tables


def test_dense_polydisperse(gpu, oracle):
    shape, tables = _dense_polydisperse(lambda i: i + 1)
    _compare(gpu, oracle, shape, 0.6, tables)


def test_dense_polydisperse_large_tags(gpu, oracle):
    shape, tables = _dense_polydisperse(lambda i: 7 * i + 13)
    assert max(int(g.tag.max()) for g in tables) > 4000
    _compare(gpu, oracle, shape, 0.6, tables)
