"""The replica timing of bench.py across ranks (gloo, world size 2, CPU): the
whole-job time is the slowest rank's, every rank sees the same result."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    bench.barrier(dist)
    got = bench.max_over_ranks([1.0 + rank, 10.0 - 3 * rank], dist)
    bench.barrier(dist)
    out.put((rank, got))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 2000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0] == res[1] == [2.0, 10.0]


def test_single_process_passthrough():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.dist_setup(1) is None
    assert bench.max_over_ranks([3.0, 4.0], None) == [3.0, 4.0]
