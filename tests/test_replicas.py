"""Replica sharding and the host-side exchanges, on world-size-2 gloo ranks
(CPU, no GPU)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from mpx_gb300.replicas import gather_rows, max_over_ranks, shard


def test_shard_partitions_exactly():
    for n in (0, 1, 7, 4096, 4097):
        for world in (1, 2, 3, 8):
            spans = [shard(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[r][1] == spans[r + 1][0] for r in range(world - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n_items, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        a, b = shard(n_items, rank, world)
        # each rank "solves" its own instances: row i = (i, 2i, rank)
        idx = torch.arange(a, b, dtype=torch.float32)
        rows = torch.stack([idx, 2 * idx, torch.full_like(idx, rank)], 1)
        t = max_over_ranks(10.0 + rank)
        allrows = gather_rows(rows, n_items)
        q.put((rank, t, allrows.numpy().tolist()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_reduce_and_gather():
    world, n_items = 2, 11
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n_items, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, rows in res:
        assert t == 11.0                               # max over ranks
        assert [r[0] for r in rows] == list(range(n_items))
        assert [r[2] for r in rows] == [0.0] * 6 + [1.0] * 5
