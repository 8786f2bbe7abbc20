"""Checkpoint / resume (lbdem_save_state / lbdem_load_state), VTK field export, and
determinism of the GPU step (the same inputs give the same bytes).

The checkpoint holds what IBcompositeDynamics::serialize writes per cell
(src/ibCompositeDynamics3D.hh:77-107) plus populations and the step count; a run
resumed from it continues bit for bit.
"""
import re
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from helpers import small_suspension


def read_vti(path):
    """Minimal reader of the appended-raw VTK ImageData this library writes."""
    raw = open(path, "rb").read()
    head, _, rest = raw.partition(b'<AppendedData encoding="raw">\n_')
    root = ET.fromstring(head.decode() + "</VTKFile>")
    img = root.find("ImageData")
    ext = [int(v) for v in img.get("WholeExtent").split()]
    nx, ny, nz = ext[1] + 1, ext[3] + 1, ext[5] + 1
    out = {}
    types = {"Float64": "<f8", "Float32": "<f4", "Int32": "<i4", "UInt8": "u1"}
    for da in img.iter("DataArray"):
        off = int(da.get("offset"))
        n = int(np.frombuffer(rest[off:off + 8], "<u8")[0])
        a = np.frombuffer(rest[off + 8:off + 8 + n], types[da.get("type")])
        comps = int(da.get("NumberOfComponents"))
        a = a.reshape(nz, ny, nx, comps) if comps > 1 else a.reshape(nz, ny, nx)
        out[da.get("Name")] = np.moveaxis(a, -1, 0).transpose(0, 3, 2, 1) if comps > 1 else a.transpose(2, 1, 0)
    return (nx, ny, nz), out


def test_vtk_writer_round_trip(lbdem_lib, tmp_path):
    rng = np.random.default_rng(1)
    rho = rng.random((5, 4, 3))
    u = rng.random((3, 5, 4, 3)).astype(np.float32)
    ids = rng.integers(0, 9, (5, 4, 3)).astype(np.int32)
    p = tmp_path / "f.vti"
    lbdem_lib.write_vtk(p, {"density": rho, "velocity": u, "particle_id": ids})
    shape, got = read_vti(p)
    assert shape == (5, 4, 3)
    assert np.array_equal(got["density"], rho)
    assert np.array_equal(got["velocity"], u)
    assert np.array_equal(got["particle_id"], ids)
    assert re.search(rb'WholeExtent="0 4 0 3 0 2"', open(p, "rb").read())


def _lattice(lb, prec, shape=(24, 20, 28)):
    return lb.Lattice(*shape, 1 / 0.6, periodic=(1, 0, 1), precision=prec, body_force=(1e-5, 0, 0),
                      max_particles=64, max_tag=64, max_radius=8)


def _drive(L, sp, shape, steps, start=0):
    import workloads as W
    p = sp
    for s in range(start):
        p = W.advance(p, shape, (1, 0, 1))
    for s in range(steps):
        g = W.with_ghosts(p, shape, (1, 0, 1))
        L.set_particles(g.x, g.v, g.w, g.r, g.tag, init_vel=(start + s == 0))
        L.collide_and_stream()
        F, T = L.get_forces()
        p = W.advance(p, shape, (1, 0, 1))
    return F, T


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("split", [4, 5])        # resume at an even and at an odd step
def test_resume_is_bit_exact(gpu, tmp_path, prec, split):
    shape = (24, 20, 28)
    sp = small_suspension(shape, 5, 2.5, 4.0, seed=31, periodic=(1, 0, 1), overlap=True)
    ck = tmp_path / "state.ckpt"
    with _lattice(gpu, prec) as A:
        _drive(A, sp, shape, split)
        A.save_state(ck)
        FA, TA = _drive(A, sp, shape, 6, start=split)
        fa = A.get_populations()
        va = A.get_field(gpu.FIELD_SUBCELL_COUNT)
    with _lattice(gpu, prec) as B:
        B.load_state(ck)
        assert B.step_count() == split
        FB, TB = _drive(B, sp, shape, 6, start=split)
        assert np.array_equal(B.get_populations(), fa)
        assert np.array_equal(B.get_field(gpu.FIELD_SUBCELL_COUNT), va)
        assert np.allclose(FB, FA, rtol=1e-12, atol=0) and np.allclose(TB, TA, rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_load_state_rejects_a_different_lattice(gpu, tmp_path):
    ck = tmp_path / "s.ckpt"
    with _lattice(gpu, 0) as A:
        A.save_state(ck)
    with _lattice(gpu, 1) as B, pytest.raises(gpu.LbdemError):
        B.load_state(ck)
    with _lattice(gpu, 0, shape=(24, 20, 24)) as C, pytest.raises(gpu.LbdemError):
        C.load_state(ck)
    (tmp_path / "junk").write_bytes(b"not a checkpoint")
    with _lattice(gpu, 0) as D, pytest.raises(gpu.LbdemError):
        D.load_state(tmp_path / "junk")


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
def test_step_is_deterministic(gpu, prec):
    """Two lattices fed the same calls hold the same bytes (voxel state, surface
    velocity, populations); only the force sums' last bits may differ (double atomics)."""
    shape = (24, 20, 28)
    sp = small_suspension(shape, 6, 2.5, 4.0, seed=32, periodic=(1, 0, 1), overlap=True)
    out = []
    for _ in range(2):
        with _lattice(gpu, prec) as L:
            F, _ = _drive(L, sp, shape, 7)
            out.append((L.get_populations(), L.get_field(gpu.FIELD_SUBCELL_COUNT), L.get_field(gpu.FIELD_PARTICLE_ID),
                        L.get_field(gpu.FIELD_PARTICLE_VELOCITY), F))
    for a, b in zip(out[0][:4], out[1][:4]):
        assert np.array_equal(a, b)
    assert np.allclose(out[0][4], out[1][4], rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_lattice_vtk_export(gpu, tmp_path):
    shape = (24, 20, 28)
    sp = small_suspension(shape, 3, 2.5, 4.0, seed=33, periodic=(1, 0, 1))
    with _lattice(gpu, 1) as L:
        _drive(L, sp, shape, 3)
        L.write_vtk(tmp_path / "l.vti")
        grid, got = read_vti(tmp_path / "l.vti")
        assert grid == shape
        assert np.array_equal(got["density"], L.get_field(gpu.FIELD_DENSITY))
        assert np.array_equal(got["solid_fraction"], L.get_field(gpu.FIELD_SOLID_FRACTION))
