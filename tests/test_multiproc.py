"""Replica logic of bench.py for N > 1 on CPU: two gloo ranks on 127.0.0.1."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from steiner_edge_linear_gb300.benchmarks import shard


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    d = bench.Dist()
    try:
        mine = list(shard(4096 * world, rank, world))
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        top = d.max(float(rank + 1) * 1.5)
        d.barrier()
        out.put((rank, gathered, top))
    finally:
        d.close()


def test_shard_covers_once():
    for count in (1, 7, 4096, 10001):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                seen += list(shard(count, r, world))
            assert seen == list(range(count))


@pytest.mark.timeout(120)
def test_two_gloo_ranks_shard_and_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=100) for _ in procs]
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    for rank, gathered, top in res:
        assert top == 3.0
        flat = gathered[0] + gathered[1]
        assert flat == list(range(8192))
