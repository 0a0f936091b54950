"""bench.py's multi-rank logic on CPU: two gloo ranks.

The path runs as independent replicas on N GPUs; the only cross-rank step
is the aggregation of the timed region (max over ranks) and of the processed
particle-steps (sum), done by bench.aggregate.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    seconds = [0.5, 0.8][rank]
    units = [1000.0, 3000.0][rank]
    t, u = bench.aggregate(seconds, units, world)
    out[rank] = (t, u)
    bench.barrier(world)
    dist.destroy_process_group()


def test_two_rank_aggregation():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == (0.8, 4000.0) and out[1] == (0.8, 4000.0)


def test_single_rank_is_identity():
    import bench

    assert bench.aggregate(1.5, 10.0, 1) == (1.5, 10.0)
