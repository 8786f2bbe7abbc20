"""lbdem_voxelize_static: the voxelization entry point that allocates nothing.

It serves callers that cannot let a library allocate device memory (an
application whose pool allocator owns the GPU, or a coupling loop that must not
pay cudaMalloc's device-wide synchronisation).  Its result must equal the
handle-based lbdem_set_particles on the same particle lists: sub-cell counts,
owner tags and particle surface velocities bit-identical (FP64: the values
setValues stores; FP32: the velocity the FP32 collision recomputes from the
owner particle, the same kernel on the same inputs), over two calls in a row
that share the static scratch, on a stream of the caller's, and without any
change in the device's free memory after the first call.

This file is collected last so that a failure here comes after every other test.
"""
import numpy as np
import pytest

import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_static_voxelization_matches_handle(gpu, precision):
    torch = pytest.importorskip("torch")
    lbdem = gpu
    shape = (40, 36, 48)
    dt = np.float64 if precision == lbdem.PREC_FP64 else np.float32
    tdt = torch.float64 if precision == lbdem.PREC_FP64 else torch.float32
    p = W.suspension(shape, n_max=12, rmin=3.0, rmax=6.0, seed=11, v_std=0.4, w_std=0.05)
    lat = lbdem.Lattice(*shape, 1.2, precision=precision, max_particles=512, max_tag=64, max_radius=8.0)
    N = int(np.prod(shape))
    dev = torch.device("cuda:0")
    vox = torch.zeros(N, dtype=torch.int32, device=dev)
    up = torch.zeros(3 * N, dtype=tdt, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    tables = []
    for call in range(2):
        g = W.with_ghosts(p, shape)
        tables.append((g, torch.from_numpy(lbdem.pack_records(g.x, g.v, g.w, g.r, g.tag)).to(dev)))
        p = W.advance(p, shape, steps=3)
    torch.cuda.synchronize()
    for call, (g, rec) in enumerate(tables):
        free_before = torch.cuda.mem_get_info(dev)[0]
        st = lbdem.voxelize_static(shape, precision, g.n, rec.data_ptr(), vox.data_ptr(), up.data_ptr(),
                                   err.data_ptr(), stream.cuda_stream)
        assert st == 0, lbdem.STATUS.get(st, st)
        stream.synchronize()
        if call > 0:   # past the first call on the device, a call allocates nothing
            free_after = torch.cuda.mem_get_info(dev)[0]
            assert free_after == free_before, f"free device memory changed by {free_after - free_before} bytes"
        lat.set_particles(g.x, g.v, g.w, g.r, g.tag)
        words = vox.cpu().numpy().view(np.uint32).reshape(shape)
        assert np.array_equal(words & 127, lat.get_field(lbdem.FIELD_SUBCELL_COUNT)), f"call {call}: counts"
        assert np.array_equal((words >> 7).astype(np.int32), lat.get_field(lbdem.FIELD_PARTICLE_ID)), \
            f"call {call}: owner tags"
        u_static = up.cpu().numpy().reshape(3, *shape)
        u_handle = lat.get_field(lbdem.FIELD_PARTICLE_VELOCITY)
        assert u_static.dtype == u_handle.dtype == dt
        assert np.array_equal(u_static, u_handle), f"call {call}: surface velocity"
        assert int(err.item()) == 0
        assert (words & 127).any() and np.abs(u_static).max() > 0
    lat.close()


def test_static_voxelization_rejects_oversize(gpu):
    lbdem = gpu
    null = 0
    # more 8^3 tiles than the static scratch holds
    assert lbdem.voxelize_static((256, 256, 256), 0, 1, 16, 16, 16, 16) == 4
    # more spheres than the static scratch holds
    assert lbdem.voxelize_static((32, 32, 32), 0, lbdem.STATIC_MAX_SPHERES + 1, 16, 16, 16, 16) == 4
    # bad arguments are rejected before any GPU work
    assert lbdem.voxelize_static((32, 32, 32), 5, 1, 16, 16, 16, 16) == 1
    assert lbdem.voxelize_static((32, 32, 32), 0, 1, null, 16, 16, 16) == 1
