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


def _views_scene():
    """Four 32x32 views of a displaced icosphere (2 subdivisions) and its
    per-vertex attributes, all float32 numpy."""
    import numpy as np
    from diffrp_gb300 import synthetic as S
    v, f = S.displaced_icosphere(2, 0.8, 0.03, 2)
    P = S.perspective(30.0, 32, 32, 0.1, 100.0).astype(np.float64)
    mvps = [P @ S.view_matrix(S.lookat_pose(e)).astype(np.float64) for e in S.sphere_eyes(4, 3.2, seed=4)]
    attr = np.random.default_rng(5).uniform(0, 1, (len(v), 3)).astype(np.float32)
    return v, f, attr, mvps


def _render_grads(indices):
    """Sum over the given views of the oracle's gradients of each view's
    sum(out * weight) w.r.t. the shared world vertices and attributes
    (clip = [v, 1] mvp^T chained by torch autograd): the per-rank work of a
    sharded step, on CPU."""
    import numpy as np
    import oracle as O
    v, f, attr, mvps = _views_scene()
    verts = torch.from_numpy(v.astype(np.float64)).requires_grad_(True)
    a = torch.from_numpy(attr.astype(np.float64)).requires_grad_(True)
    nbr = O.topology(f)
    for i in indices:
        M = torch.from_numpy(mvps[i])
        clip = verts @ M[:, :3].T + M[:, 3]
        pos = clip.detach().numpy().astype(np.float32)
        rast, _, _ = O.rasterize(pos, f, (32, 32), grad_db=False)
        col, _ = O.interpolate(attr, rast, f)
        w = np.random.default_rng(100 + i).normal(size=col.shape)
        g_col, g_pos_aa = O.antialias_bwd(col, rast, pos, f, w, nbr)
        g_attr, g_rast, _ = O.interpolate_bwd(attr, rast, f, g_col)
        g_pos = g_pos_aa + O.raster_bwd(pos, f, rast, g_rast)
        clip.backward(torch.from_numpy(g_pos))
        a.grad = torch.from_numpy(g_attr) if a.grad is None else a.grad + torch.from_numpy(g_attr)
    return verts, a


def _render_worker(rank, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=2)
    items = [(0, (32, 32))] * 4
    mine = shard_items(items)
    verts, a = _render_grads(mine)
    allreduce_gradients([verts, a])
    out[rank] = (mine, verts.grad.clone(), a.grad.clone())
    dist.destroy_process_group()


def test_sharded_views_gradients_match_single_process():
    """Four views of one mesh sharded over two gloo ranks: each rank renders
    its views with the CPU oracle and the shared-mesh gradients are summed by
    allreduce_gradients; both ranks end with the gradients of rendering all
    four views in one process."""
    port = _free_port()
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    procs = [ctx.Process(target=_render_worker, args=(r, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    (m0, gv0, ga0), (m1, gv1, ga1) = out[0], out[1]
    assert sorted(m0 + m1) == [0, 1, 2, 3] and m0 and m1
    verts, a = _render_grads(range(4))
    for got in (gv0, gv1):
        assert torch.allclose(got, verts.grad, rtol=1e-10, atol=1e-12)
    for got in (ga0, ga1):
        assert torch.allclose(got, a.grad, rtol=1e-10, atol=1e-12)
    assert float(verts.grad.abs().max()) > 0 and float(a.grad.abs().max()) > 0
