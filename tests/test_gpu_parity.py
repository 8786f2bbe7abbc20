"""GPU parity against the CPU oracle, through the C ABI.

Bars (stated per assertion below):
* voxelization: sub-cell count n, owner tag and particle surface velocity are
  bit-identical to the oracle (IEEE double with no fused multiply-add);
* FP64 populations: max |Δf̄| <= 1e-12 max |f̄|;
* FP64 forces/torques: |ΔF_p| <= 1e-12 Σ_{cells of p} |f_cell| (summation order differs);
* FP32 deviation form against the FP32 oracle: populations within 2e-5 of
  max |f̄|; per-particle forces against the FP64 oracle within 1e-4 of max |F|.
"""
import numpy as np
import pytest

import workloads as W
from helpers import rel_err, small_suspension

pytestmark = pytest.mark.gpu

CASES = {
    # shape, periodic, omega, n, rmin, rmax, overlap, body_force
    "periodic_overlap": ((24, 20, 28), (1, 1, 1), 1 / 0.6, 7, 3.0, 5.5, True, (0.0, 0.0, 0.0)),
    "channel_force": ((20, 24, 18), (1, 0, 1), 1 / 0.55, 4, 2.5, 4.5, False, (1e-5, 0.0, 2e-6)),
    "closed_box": ((16, 18, 40), (0, 0, 0), 1 / 0.6, 2, 4.0, 5.0, False, (0.0, 0.0, 0.0)),
    "tiny_radius": ((13, 11, 9), (1, 1, 1), 1.7, 5, 0.6, 1.6, True, (0.0, 0.0, 0.0)),
    # z-rows longer than one 64-cell staged segment, last segment partial
    "long_z_walls": ((6, 7, 200), (0, 1, 0), 1 / 0.6, 6, 1.5, 2.5, True, (0.0, 0.0, 1e-5)),
    "long_z_periodic": ((5, 6, 264), (1, 1, 1), 1 / 0.55, 6, 1.5, 2.4, True, (0.0, 0.0, 0.0)),
    # rows not 16-byte aligned (nz % 4 != 0): z walls, and rows of several segments
    "odd_z_walls": ((12, 10, 37), (1, 1, 0), 1 / 0.6, 4, 2.0, 3.5, True, (0.0, 0.0, 0.0)),
    "odd_long_z": ((5, 6, 133), (0, 1, 1), 1 / 0.55, 6, 1.5, 2.4, True, (2e-6, 0.0, 0.0)),
    # one-cell-thick lattices: rows of one cell; a single periodic x plane with z walls
    "flat_z": ((17, 13, 1), (1, 1, 1), 1 / 0.6, 3, 1.5, 3.0, True, (0.0, 0.0, 0.0)),
    "flat_x": ((1, 12, 20), (1, 1, 0), 1 / 0.6, 2, 1.2, 2.5, True, (0.0, 1e-6, 0.0)),
}


def _per_particle_scale(ostate, tag, n):
    """Σ_{cells owned by tag} |f_cell| per list entry (zero for ghost entries)."""
    ids = ostate["id"].ravel()
    cf = np.abs(ostate["cf"].astype(np.float64)).reshape(3, -1).sum(axis=0)
    sums = np.bincount(ids, weights=cf, minlength=int(tag.max()) + 1)
    first = {}
    for i, t in enumerate(tag):
        first.setdefault(int(t), i)
    s = np.zeros(n)
    for t, i in first.items():
        s[i] = sums[t]
    return s


def _run(lbdem, oracle, case, precision, steps, init_steps=(0, 3), seed=7):
    shape, periodic, omega, n, rmin, rmax, overlap, bf = CASES[case]
    rng = np.random.default_rng(seed)
    dt = np.float64 if precision == lbdem.PREC_FP64 else np.float32
    f0 = (rng.standard_normal((19, *shape)) * 1e-3).astype(dt)
    gl = lbdem.Lattice(*shape, omega, periodic=periodic, precision=precision, body_force=bf,
                       max_particles=256, max_tag=64, max_radius=8.0, flags=lbdem.FLAG_CELL_FORCE)
    ol = oracle.OracleLattice(*shape, omega, periodic=periodic, precision=0 if dt == np.float64 else 1,
                              body_force=bf)
    gl.set_populations(f0)
    ol.set_populations(f0)
    assert np.array_equal(gl.get_populations(), f0)
    p = small_suspension(shape, n, rmin, rmax, seed, periodic=periodic, overlap=overlap, v_std=0.3,
                         w_std=0.05)
    out = []
    for s in range(steps):
        g = W.with_ghosts(p, shape, periodic)
        iv = s in init_steps
        gl.set_particles(g.x, g.v, g.w, g.r, g.tag, init_vel=iv)
        ol.set_particles(g.x, g.v, g.w, g.r, g.tag, init_vel=iv)
        ost = ol.state()
        assert np.array_equal(gl.get_field(lbdem.FIELD_SUBCELL_COUNT), ost["n"]), f"step {s}: counts differ"
        assert np.array_equal(gl.get_field(lbdem.FIELD_PARTICLE_ID), ost["id"]), f"step {s}: owner tags differ"
        assert np.array_equal(gl.get_field(lbdem.FIELD_SOLID_FRACTION), ost["sf"]), f"step {s}: sf differs"
        upg = gl.get_field(lbdem.FIELD_PARTICLE_VELOCITY)
        if dt == np.float64:   # FP64 form: the reference's double sequence, bit for bit
            assert np.array_equal(upg, ost["up"]), f"step {s}: uPart differs"
        else:                  # FP32 form: evaluated in float
            assert rel_err(upg, ost["up"]) <= 1e-6, f"step {s}: uPart {rel_err(upg, ost['up']):.3e}"
        if iv:
            assert np.array_equal(gl.get_populations(), ol.get_populations()) or \
                rel_err(gl.get_populations(), ol.get_populations()) <= (1e-14 if dt == np.float64 else 2e-5)
        gl.collide_and_stream()
        ol.collide_and_stream()
        Fg, Tg = gl.get_forces()
        Fo, To = ol.get_forces()
        ost = ol.state()
        out.append((gl.get_populations(), ol.get_populations(), Fg, Fo, Tg, To, ost, g,
                    gl.get_field(lbdem.FIELD_HYDRO_FORCE)))
        p = W.advance(p, shape, periodic)
    assert gl.device_errors() == 0
    return out


@pytest.mark.parametrize("case", list(CASES))
def test_fp64_parity(gpu, oracle, case):
    res = _run(gpu, oracle, case, gpu.PREC_FP64, steps=6)
    for s, (fg, fo, Fg, Fo, Tg, To, ost, g, cfg) in enumerate(res):
        assert rel_err(fg, fo) <= 1e-12, f"step {s}: populations {rel_err(fg, fo):.3e}"
        assert rel_err(cfg, ost["cf"]) <= 1e-12, f"step {s}: cell force field"
        scale = _per_particle_scale(ost, g.tag, g.n)
        span = max(fg.shape[1:])
        assert np.all(np.abs(Fg - Fo) <= 1e-12 * scale[:, None] + 1e-300), f"step {s}: forces"
        assert np.all(np.abs(Tg - To) <= 1e-12 * span * scale[:, None] + 1e-300), f"step {s}: torques"
        ghost = np.ones(g.n, bool)
        _, first = np.unique(g.tag, return_index=True)
        ghost[first] = False
        assert np.all(Fg[ghost] == 0) and np.all(Tg[ghost] == 0)
    assert any(np.abs(r[2]).max() > 0 for r in res), "no force was exercised"


@pytest.mark.parametrize("case", ["periodic_overlap", "channel_force", "closed_box", "long_z_walls", "long_z_periodic",
                                  "odd_long_z"])
def test_fp32_dev_parity(gpu, oracle, case):
    res = _run(gpu, oracle, case, gpu.PREC_FP32_DEV, steps=6)
    for s, (fg, fo, Fg, Fo, Tg, To, ost, g, cfg) in enumerate(res):
        assert rel_err(fg, fo) <= 2e-5, f"step {s}: populations {rel_err(fg, fo):.3e}"
    # FP32 form against the FP64 oracle on the same inputs: per-particle force and
    # torque (the FP32 form takes torque arms per run of cells of one particle)
    res64 = _run(gpu, oracle, case, gpu.PREC_FP64, steps=6)
    for s in range(len(res)):
        F32, F64 = res[s][2], res64[s][3]
        T32, T64 = res[s][4], res64[s][5]
        assert rel_err(F32, F64) <= 1e-4, f"step {s}: FP32 force error {rel_err(F32, F64):.3e}"
        assert rel_err(T32, T64) <= 1e-4, f"step {s}: FP32 torque error {rel_err(T32, T64):.3e}"


def test_mass_and_fields(gpu, oracle):
    shape = (20, 16, 24)
    rng = np.random.default_rng(3)
    f0 = rng.standard_normal((19, *shape)) * 1e-3
    gl = gpu.Lattice(*shape, 1.3, periodic=(1, 1, 1))
    gl.set_populations(f0)
    m0 = gl.mass()
    assert abs(m0 - (f0.sum() + np.prod(shape))) <= 1e-9
    for _ in range(5):
        gl.collide_and_stream()
    assert abs(gl.mass() - m0) <= 1e-10 * m0
    f = gl.get_populations()
    c = np.array([[0, 0, 0], [-1, 0, 0], [0, -1, 0], [0, 0, -1], [-1, -1, 0], [-1, 1, 0], [-1, 0, -1],
                  [-1, 0, 1], [0, -1, -1], [0, -1, 1], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0],
                  [1, -1, 0], [1, 0, 1], [1, 0, -1], [0, 1, 1], [0, 1, -1]], dtype=np.float64)
    rho = 1 + f.sum(axis=0)
    j = np.einsum("qd,qxyz->dxyz", c, f)
    assert rel_err(gl.get_field(gpu.FIELD_DENSITY), rho) <= 1e-14
    assert rel_err(gl.get_field(gpu.FIELD_VELOCITY), j / rho) <= 1e-12


def test_equilibrium_fixed_point(gpu):
    gl = gpu.Lattice(12, 12, 12, 1.1)
    gl.init_equilibrium(0.01, (0.02, -0.01, 0.005))
    f0 = gl.get_populations()
    for _ in range(3):
        gl.collide_and_stream()
    assert rel_err(gl.get_populations(), f0) <= 1e-13


def test_unmapped_tag_is_reported(gpu, oracle):
    """Cells keep a particle's state when it leaves the list (the reference
    does too); the force sum then names a tag with no particle."""
    shape = (16, 16, 16)
    gl = gpu.Lattice(*shape, 1.2, max_particles=8, max_tag=8)
    ol = oracle.OracleLattice(*shape, 1.2)
    x = np.array([[8.0, 8.0, 8.0]]); v = np.zeros((1, 3)); w = np.zeros((1, 3)); r = np.array([3.0])
    t = np.array([1], dtype=np.int32)
    gl.set_particles(x, v, w, r, t)
    ol.set_particles(x, v, w, r, t)
    gl.collide_and_stream(); gl.get_forces()
    e = np.zeros((0, 3))
    gl.set_particles(e, e, e, np.zeros(0), np.zeros(0, np.int32))
    ol.set_particles(e, e, e, np.zeros(0), np.zeros(0, np.int32))
    gl.collide_and_stream()
    ol.collide_and_stream()
    ol.get_forces(e, np.zeros(0, np.int32))
    with pytest.raises(gpu.LbdemError) as ei:
        gl.get_forces()
    assert ei.value.status == 5
    assert gl.device_errors() & gpu.DEVERR_UNMAPPED_TAG
    assert np.array_equal(gl.get_field(gpu.FIELD_PARTICLE_ID), ol.state()["id"])


def test_bad_particles_rejected(gpu):
    gl = gpu.Lattice(16, 16, 16, 1.2, max_particles=4, max_tag=10, max_radius=5.0)
    x = np.full((1, 3), 8.0); z = np.zeros((1, 3))
    with pytest.raises(gpu.LbdemError):
        gl.set_particles(np.zeros((5, 3)), np.zeros((5, 3)), np.zeros((5, 3)), np.ones(5), np.arange(1, 6))
    gl.set_particles(x, z, z, np.array([6.0]), np.array([1]))  # radius above max_radius
    gl.collide_and_stream()
    with pytest.raises(gpu.LbdemError):
        gl.get_forces()
    assert gl.device_errors() & gpu.DEVERR_RADIUS
    gl.set_particles(x, z, z, np.array([3.0]), np.array([11]))  # tag above max_tag
    gl.collide_and_stream()
    with pytest.raises(gpu.LbdemError):
        gl.get_forces()
    assert gl.device_errors() & gpu.DEVERR_TAG_RANGE
    assert gl.device_errors() == 0


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("steps", [0, 1, 2])
def test_init_equilibrium_in_either_phase(gpu, prec, steps):
    """A uniform moving equilibrium written after an even or odd number of steps
    (the in-place layout differs) reads back as that density and velocity in
    every cell, next to walls too."""
    shape = (10, 9, 12)
    rb, u = 0.003, (0.02, -0.01, 0.015)
    with gpu.Lattice(*shape, 1 / 0.6, periodic=(1, 0, 0), precision=prec, max_particles=4, max_tag=4,
                     max_radius=4) as L:
        for _ in range(steps):
            L.collide_and_stream()
        L.init_equilibrium(rb, u)
        rho, vel = L.get_field(gpu.FIELD_DENSITY), L.get_field(gpu.FIELD_VELOCITY)
        tol = 1e-14 if prec == 0 else 2e-6
        assert np.max(np.abs(rho - (1 + rb))) <= tol
        for a in range(3):
            assert np.max(np.abs(vel[a] - u[a])) <= tol * 10, a


@pytest.mark.parametrize("prec", [0, 1])
def test_device_table_equals_host_buffers(gpu, prec):
    """Particle tables handed over in device memory -- a slice of a larger table,
    overwritten by the caller right after each call (the handle keeps its own
    copy) -- give the populations of the host-buffer path bit for bit, and its
    forces up to the order of the double atomic sums (read back through the
    device-pointer variant); forces read between a voxelization and its step
    are zero."""
    import torch
    shape = (24, 20, 28)
    p = small_suspension(shape, 5, 2.5, 4.0, seed=31, overlap=True)
    n = len(p.r)
    res = []
    for on_device in (False, True):
        x = p.x.copy()
        with gpu.Lattice(*shape, 1 / 0.6, precision=prec, max_particles=8, max_tag=16, max_radius=6) as L, \
                torch.cuda.stream(torch.cuda.Stream(device=0)):
            # the handle and the caller's tensors on one stream
            L.set_stream(torch.cuda.current_stream(0).cuda_stream)
            big = torch.zeros((n + 3) * 12, dtype=torch.float64, device="cuda:0")
            ft = torch.zeros(6 * n, dtype=torch.float64, device="cuda:0")
            for it in range(4):
                if on_device:
                    rec = gpu.pack_records(x, p.v, p.w, p.r, p.tag)
                    big[36:36 + 12 * n] = torch.from_numpy(rec.ravel()).to("cuda:0")
                    L.set_particles_device(n, big.data_ptr() + 36 * 8, init_vel=(it == 0))
                    big.fill_(float("nan"))            # queued after the handle's copy
                else:
                    L.set_particles(x, p.v, p.w, p.r, p.tag, init_vel=(it == 0))
                if it == 2:
                    F0, T0 = L.get_forces()
                    assert not F0.any() and not T0.any()
                L.collide_and_stream()
                if on_device:
                    L.get_forces_device(ft.data_ptr())
                    F = ft[:3 * n].cpu().numpy().reshape(n, 3)
                    T = ft[3 * n:].cpu().numpy().reshape(n, 3)
                else:
                    F, T = L.get_forces()
                x = np.mod(x + p.v, shape)
            L.set_stream(None)
            res.append((L.get_populations(), F, T))
    (fh, Fh, Th), (fd, Fd, Td) = res
    assert np.array_equal(fh, fd)
    assert rel_err(Fd, Fh) <= 1e-12 and rel_err(Td, Th) <= 1e-12
    assert np.abs(Fh).max() > 0


@pytest.mark.parametrize("kind", ["bin_overflow", "queue_overflow"])
def test_voxelization_overflow_paths(gpu, oracle, kind):
    """Clusters of spheres that overflow a tile's sphere bin (more than 64 spheres
    reach one 8^3 tile: the tile re-collects its spheres from every box) or a
    chunk's shell queue (more than 2048 shell pairs in one tile: the pairs past
    the queue are counted directly).  Counts and owners bit-exact, FP64 surface
    velocity bit-exact, FP32 within float rounding, populations after a step."""
    rng = np.random.default_rng(41 if kind == "bin_overflow" else 42)
    shape = (24, 24, 24)
    if kind == "bin_overflow":
        n, r = 90, rng.uniform(0.6, 1.2, 90)
    else:
        n, r = 40, rng.uniform(2.5, 3.5, 40)
    x = 12.0 + rng.uniform(-2.0, 2.0, (n, 3))
    v = rng.normal(0, 0.01, (n, 3))
    w = rng.normal(0, 1e-3, (n, 3))
    tag = np.arange(1, n + 1, dtype=np.int32)
    for prec in (0, 1):
        with gpu.Lattice(*shape, 1 / 0.6, precision=prec, max_particles=128, max_tag=128, max_radius=4) as L:
            ol = oracle.OracleLattice(*shape, 1 / 0.6, threads=4)
            L.set_particles(x, v, w, r, tag)
            ol.set_particles(x, v, w, r, tag)
            st = ol.state()
            assert np.array_equal(L.get_field(gpu.FIELD_SUBCELL_COUNT), st["n"])
            assert np.array_equal(L.get_field(gpu.FIELD_PARTICLE_ID), st["id"])
            up = L.get_field(gpu.FIELD_PARTICLE_VELOCITY)
            if prec == 0:
                assert np.array_equal(up, st["up"])
            else:
                assert rel_err(up, st["up"]) <= 1e-6
            L.collide_and_stream()
            ol.collide_and_stream()
            assert rel_err(L.get_populations(), ol.get_populations()) <= (1e-12 if prec == 0 else 2e-5)
            assert L.device_errors() == 0
