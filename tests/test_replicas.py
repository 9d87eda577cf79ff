"""Multi-process path of bench.py on CPU: world size 2 over gloo, each rank a
replica; the reported time is the slowest rank's."""
import os
import socket

import pytest


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    out[rank] = bench.max_over_ranks(1.0 + rank, dist, "cpu")
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import multiprocessing as mp
    torch = pytest.importorskip("torch")
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        ps = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in ps:
            p.start()
        for p in ps:
            p.join(timeout=120)
        assert all(p.exitcode == 0 for p in ps)
        assert dict(out) == {0: 2.0, 1: 2.0}


def test_max_over_ranks_single():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
