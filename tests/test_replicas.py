"""Replica sharding and the host-side reductions of the multi-GPU bench,
run as two gloo ranks on the CPU."""
import os
import socket

import pytest

from acts_gb300 import replicas


def test_shard_partitions_items():
    ids = list(range(103))
    for world in (1, 2, 3, 8):
        parts = [replicas.shard(ids, r, world) for r in range(world)]
        flat = sorted(x for p in parts for x in p)
        assert flat == ids
        assert max(map(len, parts)) - min(map(len, parts)) <= 1
    with pytest.raises(ValueError):
        replicas.shard(ids, 2, 2)
    assert replicas.rank_seed(7, 0) != replicas.rank_seed(7, 1)


def test_reductions_without_process_group():
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.sum_over_ranks(2) == 2.0


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, _ = replicas.env()
        mine = replicas.shard(range(10), r, w)
        # a rank's "time" and track count: the job time is the maximum, the
        # tracks the sum
        t = replicas.max_over_ranks(10.0 + r)
        n = replicas.sum_over_ranks(len(mine))
        out.put((r, mine, t, n))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert res[0][1] == [0, 2, 4, 6, 8] and res[1][1] == [1, 3, 5, 7, 9]
    assert all(r[2] == 11.0 for r in res)
    assert all(r[3] == 10.0 for r in res)
