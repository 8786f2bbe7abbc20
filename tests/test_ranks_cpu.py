"""The N > 1 path of bench.py on CPU: replicas on world_size 2 ``gloo`` ranks
agree on the slowest rank's timings (the reduction bench.py applies to its
per-rank timings before rank 0 reports)."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = [10.0 + rank, 5.0 - rank, float("nan") if rank == 1 else 1.0]
        out[rank] = bench.max_over_ranks(mine, dist, "cpu")
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        a, b, c = res[r]
        assert a == 11.0 and b == 5.0
        assert c != c          # a NaN on any rank (a leg that was not run) stays NaN
