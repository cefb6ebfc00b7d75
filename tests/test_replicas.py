"""Host-side logic of the replicas-only multi-GPU path, on CPU with gloo
(world size 2): every view is rendered by exactly one rank and the timed
region is the max over ranks."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from imagevis3d_gb300.replicas import shard


def test_shard_partitions():
    for n in (0, 1, 5, 64, 65):
        for w in (1, 2, 3, 4, 8):
            got = sorted(i for r in range(w) for i in shard(n, r, w))
            assert got == list(range(n))
            sizes = [len(shard(n, r, w)) for r in range(w)]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard(64, rank, world)
    counts = [None] * world
    dist.all_gather_object(counts, mine)
    t = torch.tensor([0.5 + rank], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        q.put((counts, float(t.item())))
    dist.destroy_process_group()


def test_gloo_two_ranks_cover_all_views_once():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    counts, tmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(counts[0] + counts[1]) == list(range(64))
    assert not set(counts[0]) & set(counts[1])
    assert tmax == 1.5
