"""Replica sharding on CPU: item ownership is a partition balanced by cost,
and the shared-mesh gradient exchange over world-size-2 gloo processes gives
the same sum as a single process."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp

from diffrp_gb300.replicas import allreduce_gradients, shard_items


def test_shard_items_partition_and_balance():
    items = [(i % 3, (r, r)) for i, r in enumerate([256, 512, 1024, 256, 512, 1024, 256, 256, 512])]
    owned = [shard_items(items, r, 3) for r in range(3)]
    flat = sorted(i for o in owned for i in o)
    assert flat == list(range(len(items)))
    loads = [sum(items[i][1][0] ** 2 for i in o) for o in owned]
    assert max(loads) - min(loads) <= 1024 ** 2
    assert shard_items(items, 0, 1) == list(range(len(items)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=2)
    items = [(0, (64, 64)), (0, (32, 32)), (1, (64, 64)), (1, (16, 16))]
    mine = shard_items(items)
    w = torch.arange(6.0).requires_grad_(True)
    # each rank's "render" contributes a different gradient to the shared parameter
    loss = sum((w * (i + 1)).sum() for i in mine)
    loss.backward()
    allreduce_gradients([w])
    out[rank] = (mine, w.grad.clone())
    dist.destroy_process_group()


def test_allreduce_gradients_gloo_two_ranks():
    port = _free_port()
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    procs = [ctx.Process(target=_worker, args=(r, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    mine0, g0 = out[0]
    mine1, g1 = out[1]
    assert sorted(mine0 + mine1) == [0, 1, 2, 3]
    expected = float(sum(i + 1 for i in range(4)))
    assert torch.equal(g0, g1)
    assert torch.allclose(g0, torch.full((6,), expected))
