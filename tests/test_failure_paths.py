"""Failure detection without a GPU fault.

* Bounded waits: with LBDEM_FLAG_PROBE_TIMEOUT, every warp of the collide-stream
  kernel first waits on a barrier that nothing completes; the wait runs out
  after a few iterations, the kernel sets LBDEM_DEVERR_TIMEOUT, lets its copies
  in flight land and returns.  The host sees LBDEM_ERR_DEVICE with the
  timeout bit from lbdem_get_forces, and the device stays usable: a handle
  created afterwards steps exactly as the oracle.  Covered for the FP64 form
  (aligned rows) and for rows that are not 16-byte aligned in both forms --
  the staging that waits on barriers.
* Allocation failures: lbdem_debug_fail_allocation makes the n-th device or
  pinned allocation of lbdem_create / lbdem_batch_create report failure without
  calling the allocator; every n up to the number of allocations a creation
  makes returns LBDEM_ERR_OUT_OF_MEMORY, and the device's free memory is the
  same afterwards (nothing leaks).
"""
import numpy as np
import pytest

import workloads as W
from helpers import rel_err, small_suspension

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,prec", [((16, 14, 32), 0), ((12, 10, 37), 0), ((12, 10, 37), 1)])
def test_bounded_wait_runs_out_and_reports(gpu, oracle, shape, prec):
    p = small_suspension(shape, 3, 2.0, 3.0, seed=5, overlap=True)
    g = W.with_ghosts(p, shape)
    with gpu.Lattice(*shape, 1 / 0.6, precision=prec, max_particles=32, max_tag=16, max_radius=4,
                     flags=gpu.FLAG_PROBE_TIMEOUT) as L:
        L.set_particles(g.x, g.v, g.w, g.r, g.tag)
        L.collide_and_stream()
        with pytest.raises(gpu.LbdemError) as ei:
            L.get_forces()
        assert ei.value.status == 5
        assert L.device_errors() & gpu.DEVERR_TIMEOUT
    # the context is intact: a new handle steps as the oracle does
    rng = np.random.default_rng(2)
    dt = np.float64 if prec == 0 else np.float32
    f0 = (rng.standard_normal((19, *shape)) * 1e-3).astype(dt)
    ol = oracle.OracleLattice(*shape, 1 / 0.6, precision=prec)
    ol.set_populations(f0)
    with gpu.Lattice(*shape, 1 / 0.6, precision=prec, max_particles=32, max_tag=16, max_radius=4) as L:
        L.set_populations(f0)
        for _ in range(2):
            L.set_particles(g.x, g.v, g.w, g.r, g.tag)
            ol.set_particles(g.x, g.v, g.w, g.r, g.tag)
            L.collide_and_stream()
            ol.collide_and_stream()
            L.get_forces()
        assert rel_err(L.get_populations(), ol.get_populations()) <= (1e-12 if prec == 0 else 2e-5)
        assert L.device_errors() == 0


def _free(torch):
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info(0)[0]


def _fail_every_allocation(gpu, create):
    """create() under the hook for n = 1, 2, ... until a creation no longer meets it."""
    torch = pytest.importorskip("torch")
    create().close()                      # first-use costs (module load, context) outside the count
    before = _free(torch)
    failed = 0
    try:
        for nth in range(1, 200):
            gpu.debug_fail_allocation(nth)
            try:
                obj = create()
            except gpu.LbdemError as e:
                assert e.status == 3, e
                failed += 1
                continue
            obj.close()
            break
    finally:
        gpu.debug_fail_allocation(0)
    assert failed >= 10, failed           # every allocation of the creation was made to fail once
    assert _free(torch) == before


def test_lattice_creation_releases_on_allocation_failure(gpu):
    _fail_every_allocation(gpu, lambda: gpu.Lattice(24, 20, 16, 1.2, max_particles=64, max_tag=64, max_radius=6,
                                                    flags=gpu.FLAG_CELL_FORCE))


def test_batch_creation_releases_on_allocation_failure(gpu):
    doms = [{"shape": (20, 14, 18), "periodic": (1, 1, 1), "omega": 1 / 0.6, "max_particles": 8},
            {"shape": (16, 12, 24), "periodic": (1, 0, 0), "omega": 1 / 0.55, "max_particles": 4}]
    _fail_every_allocation(gpu, lambda: gpu.Batch(doms, precision=gpu.PREC_FP64, max_tag=16, max_radius=6))
