"""The multi-rank reduction of bench.py on CPU (gloo, world size 2).

The world does not shard, so N ranks step N independent replicas: the job's time is the
slowest rank's and its contact count the sum over ranks.  Two gloo ranks on 127.0.0.1
check that reduction and the single-rank path.
"""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, contacts = bench.reduce_over_ranks(10.0 + 5.0 * rank, 1000 * (rank + 1), dist, device="cpu")
        out[rank] = (ms, contacts)
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time_and_the_summed_contacts():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert dict(out) == {0: (15.0, 3000.0), 1: (15.0, 3000.0)}


def test_single_rank_needs_no_collective():
    import bench
    assert bench.reduce_over_ranks(12.5, 42, None) == (12.5, 42.0)
