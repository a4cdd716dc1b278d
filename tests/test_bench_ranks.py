"""bench.py's multi-GPU arm on the CPU: two gloo ranks.  The path shards by
chunk pair with no exchange step, so the only cross-rank operation is the
max-over-ranks of the timed region; each rank runs its own seeded shard."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(1.5 + rank, world)          # the slowest rank's time
        items = bench.workload(rank)
        dist.barrier()
        out.put((rank, ms, bench.shard_seed(rank), items[0][0][:64], len(items)))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time_and_distinct_shards():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ms0, s0, head0, n0), (r1, ms1, s1, head1, n1) = got
    assert ms0 == ms1 == 2.5
    assert s0 != s1 and head0 != head1
    assert n0 == n1


def test_single_rank_is_unchanged():
    import bench
    assert bench.max_over_ranks(3.25, 1) == 3.25
    assert bench.shard_seed(0) == bench.SEED
