"""Multi-GPU form of the path: replicas with item sharding.

Views and items are independent, so the rasterisation path shards with no
collective on the data path: each rank renders its share of the items.  The
only exchange is optional -- when several ranks render views of the same
meshes and want one gradient per mesh, ``allreduce_gradients`` sums the
(shared-mesh) vertex / attribute gradients with one all-reduce.
"""
import torch
import torch.distributed as dist

__all__ = ["shard_items", "allreduce_gradients", "world"]


def world():
    """(rank, world_size), (0, 1) without an initialised process group."""
    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(), dist.get_world_size()
    return 0, 1


def shard_items(items, rank=None, world_size=None, cost=None):
    """Split ``items`` across ranks, balancing ``cost(item)`` (default: pixel
    count H * W of an (mesh, (H, W)) item) greedily, largest first.  Returns
    the indices owned by ``rank`` in ascending order; every item is owned by
    exactly one rank."""
    if rank is None or world_size is None:
        rank, world_size = world()
    if cost is None:
        def cost(it):
            return it[1][0] * it[1][1]
    order = sorted(range(len(items)), key=lambda i: (-cost(items[i]), i))
    loads = [0] * world_size
    owner = [0] * len(items)
    for i in order:
        r = min(range(world_size), key=lambda k: (loads[k], k))
        owner[i] = r
        loads[r] += cost(items[i])
    return [i for i in range(len(items)) if owner[i] == rank]


def allreduce_gradients(tensors):
    """Sum the gradients of shared parameters over all ranks (one flat
    all-reduce; no-op on a single process)."""
    grads = [t.grad for t in tensors if t.grad is not None]
    rank, ws = world()
    if ws == 1 or not grads:
        return
    flat = torch.cat([g.reshape(-1) for g in grads])
    dist.all_reduce(flat)
    off = 0
    for g in grads:
        n = g.numel()
        g.copy_(flat[off:off + n].view_as(g))
        off += n
