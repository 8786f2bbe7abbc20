"""Periodic pressure drop (Zhang & Kwok rescale, src/periodicPressureFunctionals3D.hh:121-159),
Palabos computeAverageDensity, and the equilibrium initial profiles
(PressureGradient, PoiseuilleProfileAndPressureGradient, :242-298).

The channel case follows examples/showcaseRectChannel/showcaseRectChannel.cpp:253-273:
x periodic, walls in y and z, inlet box at x = 0 and outlet box at x = nx - 1
without the wall rows, averages taken before collideAndStream, the rescale after it.
"""
import numpy as np
import pytest

from helpers import rel_err, small_suspension

SHAPE = (40, 20, 24)
PER = (1, 0, 0)
TAU = 0.6
RHO_HI, RHO_LO = 1.0, 0.998


def boxes(shape):
    nx, ny, nz = shape
    return [0, 0, 1, ny - 2, 1, nz - 2], [nx - 1, nx - 1, 1, ny - 2, 1, nz - 2]


# ---- CPU: the oracle's restatement --------------------------------------------------------------

def test_oracle_zhang_rescales_only_incoming_populations(oracle):
    ol = oracle.OracleLattice(*SHAPE, 1 / TAU, periodic=PER)
    ol.init_profile(1, RHO_HI, RHO_LO, 0.01, SHAPE, 0)
    f0 = ol.get_populations().astype(np.float64)
    inlet, _ = boxes(SHAPE)
    ol.zhang_rescale(inlet, 0, 1, 1.0, 0.999)
    f1 = ol.get_populations().astype(np.float64)
    W = np.array([1 / 3] + [1 / 18] * 3 + [1 / 36] * 6 + [1 / 18] * 3 + [1 / 36] * 6)
    cxs = np.array([0, -1, 0, 0, -1, -1, -1, -1, 0, 0, 1, 0, 0, 1, 1, 1, 1, 0, 0])
    changed = np.any(f1 != f0, axis=(1, 2, 3))
    assert set(np.nonzero(changed)[0]) == set(np.nonzero(cxs == 1)[0])
    k = 1.0 / 0.999
    sl = (slice(0, 1), slice(1, SHAPE[1] - 1), slice(1, SHAPE[2] - 1))
    for i in np.nonzero(cxs == 1)[0]:
        np.testing.assert_allclose(f1[i][sl] + W[i], (f0[i][sl] + W[i]) * k, rtol=1e-15)
        outside = np.ones(SHAPE, bool)
        outside[sl] = False
        assert np.array_equal(f1[i][outside], f0[i][outside])


def test_oracle_profile_density_and_velocity(oracle):
    nx, ny, nz = SHAPE
    ol = oracle.OracleLattice(*SHAPE, 1 / TAU, periodic=PER)
    ol.init_profile(1, RHO_HI, RHO_LO, 0.02, (nx, ny, nz), 0)
    f = ol.get_populations()
    rho = 1 + f.sum(axis=0)
    assert abs(rho[0].mean() - RHO_HI) < 1e-14 and abs(rho[-1].mean() - RHO_LO) < 1e-14
    cxs = np.array([0, -1, 0, 0, -1, -1, -1, -1, 0, 0, 1, 0, 0, 1, 1, 1, 1, 0, 0])
    ux = np.tensordot(cxs, f, axes=(0, 0)) / rho
    y = (np.arange(ny) - ny / 2) / (ny / 2)
    z = (np.arange(nz) - nz / 2) / (nz / 2)
    want = 0.02 * np.outer(1 - y * y, 1 - z * z)
    np.testing.assert_allclose(ux[5], want, atol=1e-15)
    assert abs(ol.average_density([0, 0, 0, ny - 1, 0, nz - 1]) - RHO_HI) < 1e-14


# ---- GPU parity ---------------------------------------------------------------------------------

def _gpu_lattice(lb, prec, shape=SHAPE, per=PER):
    return lb.Lattice(*shape, 1 / TAU, periodic=per, precision=prec, max_particles=64, max_tag=64, max_radius=8)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("kind,dim", [(0, 0), (1, 0), (1, 1), (1, 2), (0, 2)])
@pytest.mark.parametrize("pre_steps", [0, 1])
def test_init_profile_bit_exact(gpu, oracle, prec, kind, dim, pre_steps):
    n = (SHAPE[0] - 1, SHAPE[1], SHAPE[2] + 1)          # functor sizes need not equal the lattice's
    ol = oracle.OracleLattice(*SHAPE, 1 / TAU, periodic=PER, precision=prec)
    ol.init_profile(kind, RHO_HI, RHO_LO, 0.03, n, dim)
    with _gpu_lattice(gpu, prec) as L:
        for _ in range(pre_steps):                      # odd in-place phase
            L.collide_and_stream()
        L.init_profile(kind, RHO_HI, RHO_LO, 0.03, n, dim)
        assert np.array_equal(L.get_populations(), ol.get_populations())


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("pre_steps", [0, 1, 2])
def test_average_density_and_rescale(gpu, oracle, prec, pre_steps):
    sp = small_suspension(SHAPE, 4, 3.0, 5.0, seed=3, periodic=PER)
    ol = oracle.OracleLattice(*SHAPE, 1 / TAU, periodic=PER, precision=prec)
    ol.init_profile(1, RHO_HI, RHO_LO, 0.02, SHAPE, 0)
    with _gpu_lattice(gpu, prec) as L:
        L.init_profile(1, RHO_HI, RHO_LO, 0.02, SHAPE, 0)
        for _ in range(pre_steps):
            for lat in (L, ol):
                lat.set_particles(sp.x, sp.v, sp.w, sp.r, sp.tag)
                lat.collide_and_stream()
        inlet, outlet = boxes(SHAPE)
        for box in (inlet, outlet, [3, 9, 2, 7, 0, 23]):
            a, b = L.average_density(box), ol.average_density(box)
            # the float form sums a cell's populations in float (the oracle in double), and
            # float populations after a step differ from the float oracle's at the float level
            assert abs(a - b) <= (1e-13 if prec == 0 else 1e-8) * abs(b)
        L.zhang_rescale(inlet, 0, 1, RHO_HI, 0.9991)
        ol.zhang_rescale(inlet, 0, 1, RHO_HI, 0.9991)
        L.zhang_rescale(outlet, 0, -1, RHO_LO, 1.0003)
        ol.zhang_rescale(outlet, 0, -1, RHO_LO, 1.0003)
        g, o = L.get_populations(), ol.get_populations()
        if pre_steps == 0:
            assert np.array_equal(g, o)                 # same inputs, same rounded sequence
        else:
            assert rel_err(g, o) < (1e-12 if prec == 0 else 5e-6)


def _channel_pair(gpu, oracle, prec, steps, sp, fused=True):
    inlet, outlet = boxes(SHAPE)
    ol = oracle.OracleLattice(*SHAPE, 1 / TAU, periodic=PER, precision=prec, threads=4)
    ol.init_profile(1, RHO_HI, RHO_LO, 0.01, (SHAPE[0] - 1, SHAPE[1], SHAPE[2]), 0)
    L = _gpu_lattice(gpu, prec)
    L.init_profile(1, RHO_HI, RHO_LO, 0.01, (SHAPE[0] - 1, SHAPE[1], SHAPE[2]), 0)
    if fused:
        L.set_pressure_drop(0, inlet, outlet, RHO_HI, RHO_LO)
    Fg = Fo = None
    for it in range(steps):
        init_vel = it == 0
        # oracle: the reference's loop order
        ol.set_particles(sp.x, sp.v, sp.w, sp.r, sp.tag, init_vel=init_vel)
        a_in, a_out = ol.average_density(inlet), ol.average_density(outlet)
        ol.collide_and_stream()
        ol.zhang_rescale(inlet, 0, 1, RHO_HI, a_out)
        ol.zhang_rescale(outlet, 0, -1, RHO_LO, a_in)
        Fo, To = ol.get_forces()
        L.set_particles(sp.x, sp.v, sp.w, sp.r, sp.tag, init_vel=init_vel)
        if not fused:
            g_in, g_out = L.average_density(inlet), L.average_density(outlet)
        L.collide_and_stream()
        if not fused:
            L.zhang_rescale(inlet, 0, 1, RHO_HI, g_out)
            L.zhang_rescale(outlet, 0, -1, RHO_LO, g_in)
        Fg, Tg = L.get_forces()
        sp.x[:] = sp.x + sp.v
        sp.x[:, 0] %= SHAPE[0]
    return L, ol, Fg, Fo


@pytest.mark.gpu
@pytest.mark.parametrize("fused", [True, False])
def test_channel_fp64_matches_oracle(gpu, oracle, fused):
    sp = small_suspension(SHAPE, 5, 3.0, 4.5, seed=11, periodic=PER)
    L, ol, Fg, Fo = _channel_pair(gpu, oracle, 0, 30, sp, fused)
    with L:
        assert rel_err(L.get_populations(), ol.get_populations()) <= 1e-12
        assert rel_err(Fg, Fo) <= 1e-10
        assert L.step_count() == 30


@pytest.mark.gpu
def test_channel_fp32_matches_fp64_oracle(gpu, oracle):
    sp = small_suspension(SHAPE, 5, 3.0, 4.5, seed=11, periodic=PER)
    L32, _, F32, _ = _channel_pair(gpu, oracle, 1, 30, sp, True)
    sp = small_suspension(SHAPE, 5, 3.0, 4.5, seed=11, periodic=PER)
    L64, ol64, _, F64_oracle = _channel_pair(gpu, oracle, 0, 30, sp, True)
    with L32, L64:
        assert rel_err(F32, F64_oracle) <= 1e-4
        f = ol64.get_populations()
        rho = 1 + f.sum(axis=0)
        cxs = np.array([0, -1, 0, 0, -1, -1, -1, -1, 0, 0, 1, 0, 0, 1, 1, 1, 1, 0, 0])
        ux = np.tensordot(cxs, f, axes=(0, 0)) / rho
        assert rel_err(L32.get_field(gpu.FIELD_VELOCITY)[0], ux) <= 1e-4


@pytest.mark.gpu
def test_pressure_drop_drives_the_channel(gpu):
    """Fluid at rest with the pressure drop only: a flow towards +x builds up and the
    inlet/outlet averages settle near the targets."""
    inlet, outlet = boxes(SHAPE)
    with _gpu_lattice(gpu, 1) as L:
        L.set_pressure_drop(0, inlet, outlet, 1.0 + 1e-3, 1.0 - 1e-3)
        for _ in range(400):
            L.collide_and_stream()
        u = L.get_field(gpu.FIELD_VELOCITY)
        ux = u[0][:, 1:-1, 1:-1]
        assert ux.mean() > 1e-5
        assert ux[:, SHAPE[1] // 2, SHAPE[2] // 2].mean() > ux[:, 1, 1].mean()   # faster on the axis
        assert L.average_density(inlet) > L.average_density(outlet)


@pytest.mark.gpu
def test_pressure_drop_rejects_bad_boxes(gpu):
    inlet, outlet = boxes(SHAPE)
    with _gpu_lattice(gpu, 0) as L:
        with pytest.raises(gpu.LbdemError):
            L.set_pressure_drop(0, inlet, inlet, 1.0, 0.99)                     # overlapping
        with pytest.raises(gpu.LbdemError):
            L.set_pressure_drop(0, [0, 0, 0, 99, 0, 5], outlet, 1.0, 0.99)      # outside
        with pytest.raises(gpu.LbdemError):
            L.set_pressure_drop(3, inlet, outlet, 1.0, 0.99)
        with pytest.raises(gpu.LbdemError):
            L.zhang_rescale(inlet, 0, 2, 1.0, 1.0)
        with pytest.raises(gpu.LbdemError):
            L.init_profile(0, 1.0, 0.9, 0.0, (1, 1, 1), 0)
        L.set_pressure_drop(None)
