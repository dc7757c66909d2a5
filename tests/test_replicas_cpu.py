"""Replica path of bench.py (one process per GPU, no data-path collective), on CPU.

Two gloo ranks run the helpers the multi-GPU bench uses: the slowest rank's time sets
the job's time, request-level dispatch gives every rank a disjoint share that together
covers the stream, and the whole-job rate counts all ranks' units.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        t = bench.max_over_ranks(dist, 1.5 + rank)
        items = list(range(103))
        mine = bench.shard(items, rank, world)
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        q.put((rank, t, sorted(x for part in gathered for x in part), len(mine),
               bench.replica_rate(world, 5, t)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        results = sorted(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert [p.exitcode for p in procs] == [0, 0]
    for rank, t, covered, nmine, rate in results:
        assert t == pytest.approx(2.5)              # the slower rank's time
        assert covered == list(range(103))           # disjoint shares covering the stream
        assert nmine == (52 if rank == 0 else 51)
        assert rate == pytest.approx(2 * 5 / 2.5)    # all ranks' units over the slowest time


def test_single_process_helpers():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(None, 3.0) == 3.0
    assert bench.shard(list(range(5)), 0, 1) == list(range(5))
    assert bench.replica_rate(1, 10, 2.0) == 5.0
