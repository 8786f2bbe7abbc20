"""GPU against the fixtures produced by the reference's own PSM code
(tests/golden/ref_psm_*.npz), through the C ABI, FP64 form.

Bars: sub-cell counts, owner tags and surface velocities bit-identical;
populations within 1e-12 of max |f̄|; per-cell force within 1e-12 of max
|f_cell|; per-particle F/T within 1e-12 of the sum of |f_cell| over the
particle's cells."""
from pathlib import Path

import numpy as np
import pytest

from helpers import rel_err

pytestmark = pytest.mark.gpu
GOLDEN = sorted((Path(__file__).resolve().parent / "golden").glob("ref_psm_*.npz"))


@pytest.mark.parametrize("path", GOLDEN, ids=[p.stem for p in GOLDEN])
def test_gpu_reproduces_reference_fixture(gpu, path):
    lbdem = gpu
    d = np.load(path)
    shape = tuple(int(s) for s in d["shape"])
    gl = lbdem.Lattice(*shape, float(d["omega"]), max_particles=256, max_tag=64, max_radius=8.0,
                       flags=lbdem.FLAG_CELL_FORCE)
    gl.set_populations(d["f0"])
    init = set(int(s) for s in d["init_steps"])
    for s in range(int(d["steps"])):
        gl.set_particles(d[f"x{s}"], d[f"v{s}"], d[f"w{s}"], d[f"r{s}"], d[f"tag{s}"], init_vel=s in init)
        assert np.array_equal(gl.get_field(lbdem.FIELD_SUBCELL_COUNT), d[f"n{s}"]), f"step {s}: counts"
        assert np.array_equal(gl.get_field(lbdem.FIELD_PARTICLE_ID), d[f"id{s}"]), f"step {s}: tags"
        assert np.array_equal(gl.get_field(lbdem.FIELD_PARTICLE_VELOCITY), d[f"up{s}"]), f"step {s}: uPart"
        gl.collide_and_stream()
        F, T = gl.get_forces()
        cf = gl.get_field(lbdem.FIELD_HYDRO_FORCE)
        assert rel_err(cf, d[f"cf{s}"]) <= 1e-12, f"step {s}: cell force"
        tag = d[f"tag{s}"]
        ids = d[f"id{s}"].ravel()
        w = np.abs(d[f"cf{s}"]).reshape(3, -1).sum(axis=0)
        sums = np.bincount(ids, weights=w, minlength=int(tag.max()) + 1)
        scale = np.zeros(len(tag))
        seen = set()
        for i, t in enumerate(tag):
            if int(t) not in seen:
                scale[i] = sums[int(t)]
                seen.add(int(t))
        span = max(shape)
        assert np.all(np.abs(F - d[f"F{s}"]) <= 1e-12 * scale[:, None] + 1e-300), f"step {s}: forces"
        assert np.all(np.abs(T - d[f"T{s}"]) <= 1e-12 * span * scale[:, None] + 1e-300), f"step {s}: torques"
    assert rel_err(gl.get_populations(), d["f_final"]) <= 1e-12
    assert gl.device_errors() == 0
