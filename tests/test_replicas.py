"""The N>1 path (replicas) on CPU with gloo, world_size 2."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from spacetime_gb300.replicas import max_over_ranks, shard


def test_shard_partitions():
    for n in (0, 1, 7, 240, 1080):
        for world in (1, 2, 3, 8):
            got = [list(shard(n, r, world)) for r in range(world)]
            flat = [x for g in got for x in g]
            assert flat == list(range(n))
            sizes = [len(g) for g in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    frames = list(shard(240, rank, world))
    ms = [10.0 + rank, 20.0 - rank]
    out = max_over_ranks(ms)
    q.put((rank, frames[0], frames[-1], out))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_world2_timing_reduction():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1:3] == (0, 119) and res[1][1:3] == (120, 239)
    assert res[0][3] == res[1][3] == [11.0, 20.0]
