"""Autotuner for the rasteriser's launch shape.

Chooses the fine-raster tile size (8, 16 or 32 pixels), the threads per
primitive (0 = pixel-parallel tiles, else 1..32 threads walking a
primitive's bounding box) and the bin depth (tile-list capacity headroom) by
timing ``drp_rasterize_fwd`` on the caller's own geometry with CUDA events.
Results are cached in a JSON file keyed by (device architecture, views,
resolution, triangle-count bucket) so a workload is tuned once per machine.
The cache path is ``$DRP_AUTOTUNE_CACHE`` or
``~/.cache/diffrp_gb300/autotune.json``.
"""
import json
import math
import os
import threading

import torch

from . import nvdr

__all__ = ["TILE_CHOICES", "TPT_CHOICES", "tune_rasterizer", "tune_batch", "apply", "cache_path", "workload_key"]

TILE_CHOICES = (3, 4, 5)
TPT_CHOICES = (0, 1, 4, 8, 32)
_lock = threading.Lock()


def cache_path():
    return os.environ.get("DRP_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "diffrp_gb300", "autotune.json"))


def _load():
    try:
        with open(cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store(table):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp%d" % os.getpid()
        with open(tmp, "w") as fh:
            json.dump(table, fh, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def workload_key(device, num_views, resolution, num_triangles):
    major, minor = torch.cuda.get_device_capability(device)
    fb = int(round(math.log2(max(1, num_triangles))))
    return "sm%d%d|B%d|%dx%d|F2^%d" % (major, minor, num_views, resolution[0], resolution[1], fb)


def apply(ctx, choice):
    ctx.tile_log2 = int(choice["tile_log2"])
    ctx.threads_per_tri = int(choice["threads_per_tri"])
    if "list_capacity" in choice:
        ctx.ensure_capacity(int(choice["list_capacity"]))
    return ctx


def tune_rasterizer(ctx, pos, tri, resolution, ranges=None, reps=3, burst=8, candidates=None, use_cache=True):
    """Time every (tile size, threads per primitive) candidate on this
    geometry, set the fastest on ``ctx`` and return it (with the measured
    times in milliseconds).  Each timing is ``burst`` rasterisations enqueued
    back to back between two events, the fastest of ``reps`` bursts: a
    single call of about 0.05 ms sat too close to its own launch overhead
    to separate the candidates reliably."""
    B = pos.shape[0] if pos.dim() == 3 else (1 if ranges is None else ranges.shape[0])
    key = workload_key(pos.device, B, resolution, tri.shape[0])
    if use_cache:
        with _lock:
            hit = _load().get(key)
        if hit is not None:
            return apply(ctx, hit) and hit
    if candidates is None:
        candidates = [(t, p) for t in TILE_CHOICES for p in TPT_CHOICES]
    stream = torch.cuda.current_stream(pos.device)
    times = {}
    best = None
    for tl, tpt in candidates:
        probe = nvdr.RasterizeCudaContext(pos.device, tile_log2=tl, threads_per_tri=tpt)
        nvdr.rasterize(probe, pos, tri, resolution, ranges=ranges, grad_db=False)  # sizes the lists
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(burst):
                nvdr.rasterize(probe, pos, tri, resolution, ranges=ranges, grad_db=False)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / burst)
        t = min(ts)
        times["%d/%d" % (tl, tpt)] = t
        if best is None or t < best[0]:
            best = (t, tl, tpt, probe.last_list_entries)
    choice = {"tile_log2": best[1], "threads_per_tri": best[2],
              # bin depth: list capacity with 50% headroom over the measured need
              "list_capacity": int(best[3] * 1.5) + 4096, "ms": best[0], "times_ms": times}
    apply(ctx, choice)
    if use_cache:
        with _lock:
            table = _load()
            table[key] = choice
            _store(table)
    return choice


def tune_batch(renderer, pos, attr, reps=3, burst=8, candidates=None):
    """Time the batched forward (``drp_batch_forward``) of ``renderer`` on
    its own items for every (tile size, threads per primitive) candidate and
    keep the fastest; returns the choice with the measured times.  Each
    timing is ``burst`` forwards enqueued back to back between two events
    (the device, not the host's launch rate, sets the pace: a single eager
    forward of about 0.1 ms was too close to its launch overhead to separate
    16- from 32-pixel tiles), the fastest of ``reps`` bursts per candidate.
    A recompute renderer is timed on its first chunk (the size it renders
    at), so tuning allocates no more than one chunk's buffers."""
    top = renderer
    if renderer.recompute:
        chunk = renderer._chunks[0]
        renderer, pos = chunk.renderer, pos[chunk.rows]
    if candidates is None:
        # pixel-parallel, or 1 / 2 / 4 threads per primitive (tiny triangles
        # favour one thread walking each small bounding box)
        candidates = [(t, p) for t in TILE_CHOICES for p in (0, 1, 2, 4)]
    stream = torch.cuda.current_stream(pos.device)
    times = {}
    best = None
    for tl, tpt in candidates:
        renderer.set_raster_shape(tl, tpt)
        rast, color, out = renderer.forward_buffers(pos, attr)  # sizes the tile lists
        p, a = pos.contiguous(), attr.contiguous().reshape(-1)
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(burst):
                renderer._forward_raw(p, a, rast, color, out)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / burst)
        t = min(ts)
        times["%d/%d" % (tl, tpt)] = t
        if best is None or t < best[0]:
            best = (t, tl, tpt)
    top.set_raster_shape(best[1], best[2])
    renderer.forward_buffers(pos, attr)
    return {"tile_log2": best[1], "threads_per_tri": best[2], "ms": best[0], "times_ms": times}
