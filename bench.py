"""Benchmark: fwd+bwd Mpix/s of rasterize -> interpolate -> antialias -> loss.

Workload (N=1, one GB300): the single-mesh full-gradient configuration --
icosphere with 5 subdivisions (10242 vertices, 20480 triangles, radius 0.8),
every vertex displaced radially by N(0, 0.02) (seed 0), one 1024x1024 view
from (0, 0, 3.2) (fov 30, near 0.1, far 100), 8 float32 attribute channels
(unit vertex normal 3, uv 2 ~ U(0,1), colour 3 ~ U(0,1)), L1 loss to a seeded
U(0,1) target, gradients w.r.t. vertex positions and attributes.  One step =
clip transform, rasterize, interpolate, antialias, loss (the package's fused
L1: one pass for loss and gradient), backward.

Lines printed (rank 0, one JSON line):
  value       Mpix/s with inputs resident in HBM, CUDA-event timed per step,
              L2 flushed (256 MiB write) between steps outside the events;
  e2e         the same step through the public API with the parameters copied
              from pinned host memory and loss + gradients copied back, inside
              the timed region (copies and step captured as one CUDA graph; the
              copies by kernels over the host link, copy_engine_value with
              cudaMemcpyAsync transfers instead);
  roofline    dominant kernel (entry point) of the step: algorithmic bytes /
              CUDA-event time vs the measured HBM copy bandwidth;
  cpu_baseline  the CPU oracle (a restatement of the path, all host threads)
              on a bounded sample of the same workload.
Attached beside the headline (each with ms_per_step, a whole-step roofline
fraction from the path's byte model and, for the batched ones, the peak
device memory): batched_views64 (64 views of the 1280-triangle icosphere at
512x512, batched vs plain per-view), config1_session (the README example at
512x512 through SurfaceDeferredRenderSession), batched_uneven48 (48 meshes,
135 items, batched vs plain), batched_large16 (2.09M-triangle heightfield,
16 views at 2048x2048, recompute in chunks, with the stored-buffer run and
its peak memory beside it).

``--impl reference`` times the CPU implementation of the path (the oracle
port: the reference's own rasteriser is an external CUDA package that does
not exist on this machine) with all host threads on the same workload.
``--gpus N`` under torchrun runs N replicas of the headline step (weak
scaling; no collective on the data path) and attaches ``sharded_views64``:
the 64 views sharded across the ranks with one all-reduce of the shared
mesh's gradients per step (strong scaling).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def l1_loss(pred, target):
    from diffrp_gb300.losses import l1_loss as fused
    return fused(pred, target)

H = W = 1024
C = 8
METRIC = "fwd+bwd Mpix/s (rasterize->interpolate->antialias->L1 loss, backward to positions and attributes)"
UNIT = "Mpix/s"


def make_workload(seed=0):
    from diffrp_gb300 import synthetic as S
    v, f = S.displaced_icosphere(5, 0.8, 0.02, seed)
    rng = np.random.default_rng(seed + 1)
    # unit vertex normals (area-weighted), uv, colour
    fn = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    vn = np.zeros_like(v)
    for k in range(3):
        np.add.at(vn, f[:, k], fn)
    vn /= np.linalg.norm(vn, axis=1, keepdims=True)
    attr = np.concatenate([vn, rng.uniform(0, 1, (len(v), 2)), rng.uniform(0, 1, (len(v), 3))], 1)
    attr = attr.astype(np.float32)
    mvp = S.perspective(30.0, H, W, 0.1, 100.0).astype(np.float64) @ \
        S.view_matrix(S.lookat_pose((0.0, 0.0, 3.2))).astype(np.float64)
    target = rng.uniform(0, 1, (1, H, W, C)).astype(np.float32)
    return v.astype(np.float32), f, attr, mvp.astype(np.float32), target


class Step:
    """One fwd+bwd through the drop-in nvdiffrast API (diffrp_gb300.nvdr)."""

    def __init__(self, dev, f, mvp, target):
        import torch
        from diffrp_gb300 import nvdr as dr
        self.dr = dr
        self.torch = torch
        self.ctx = dr.RasterizeCudaContext(dev)
        self.tri = torch.from_numpy(f).to(dev)
        self.mvp = torch.from_numpy(mvp).to(dev)
        self.target = torch.from_numpy(target).to(dev)
        self.topo = dr.antialias_construct_topology_hash(self.tri)

    def __call__(self, verts, attr):
        torch, dr = self.torch, self.dr
        verts.grad = None
        attr.grad = None
        clip = clip_space(verts, self.mvp)
        rast, _ = dr.rasterize(self.ctx, clip, self.tri, (H, W), grad_db=False)
        col, _ = dr.interpolate(attr, rast, self.tri)
        aa = dr.antialias(col, rast, clip, self.tri, topology_hash=self.topo)
        loss = l1_loss(aa, self.target)
        loss.backward()
        return loss


WORKLOAD_SINGLE = "icosphere5-displaced 20480 tris, 1024x1024, 8 ch, L1 loss, fwd+bwd (single mesh, full gradients)"


def clip_space(verts, mvp):
    """Clip-space positions [v, 1] @ mvp^T of (V, 3) vertices: one transform kernel."""
    from diffrp_gb300.transform import clip_space as cs
    return cs(verts, mvp)


def packed_attr_offset(nv):
    return (nv + 63) // 64 * 64


def pack_inputs(verts_np, attr_np):
    """Vertices, then attributes at a 256-byte aligned offset, in one array."""
    a0 = packed_attr_offset(verts_np.size)
    buf = np.zeros(a0 + attr_np.size, np.float32)
    buf[:verts_np.size] = verts_np.reshape(-1)
    buf[a0:] = attr_np.reshape(-1)
    return buf


class GraphedStep:
    """The same step captured once as a CUDA graph (static parameter tensors,
    gradients allocated in the graph's pool) and replayed.  With io = (h_in,
    h_out) pinned host buffers the graph also copies the parameters in from
    h_in before the step and the loss and gradients out to h_out after it:
    by kernels over the host link (zero_copy, diffrp_gb300.hostio) or by
    copy-engine transfers."""

    def __init__(self, step, verts_np, attr_np, dev, io=None, zero_copy=True):
        import torch
        self.torch = torch
        # parameters as views of one packed buffer: one host->device copy per step
        nv, na = verts_np.size, attr_np.size
        self.inbuf = torch.from_numpy(pack_inputs(verts_np, attr_np)).to(dev)
        a0 = packed_attr_offset(nv)  # attributes start 256-byte aligned (128-bit row access)
        self.verts = self.inbuf[:nv].view(verts_np.shape).requires_grad_(True)
        self.attr = self.inbuf[a0:a0 + na].view(attr_np.shape).requires_grad_(True)
        self.outbuf = torch.empty(1 + nv + na, dtype=torch.float32, device=dev)
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            for _ in range(3):
                step(self.verts, self.attr)
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        self.graph = torch.cuda.CUDAGraph()
        n0 = kernel_launches()
        if io is not None and zero_copy:
            from diffrp_gb300 import hostio
            io = (hostio.device_view(io[0], dev), hostio.device_view(io[1], dev))
        with torch.cuda.graph(self.graph):
            if io is not None:
                with torch.no_grad():
                    if zero_copy:
                        hostio.copy_(self.inbuf, io[0])
                    else:
                        self.inbuf.copy_(io[0], non_blocking=True)
            self.loss = step(self.verts, self.attr)
            if io is not None:
                with torch.no_grad():
                    if zero_copy:  # packed straight into the host buffer
                        torch.cat([self.loss.detach().view(1), self.verts.grad.view(-1),
                                   self.attr.grad.view(-1)], out=io[1])
                    else:
                        io[1].copy_(self.pack_result(), non_blocking=True)
        # our kernels in one step, counted by the library as they are captured
        self.launches_per_step = kernel_launches() - n0
        torch.cuda.synchronize(dev)

    def load(self, h_in):
        """h_in: pinned host floats, vertices then attributes."""
        with self.torch.no_grad():
            self.inbuf.copy_(h_in, non_blocking=True)

    def pack_result(self):
        """Loss and gradients into one device buffer (one device->host copy)."""
        torch = self.torch
        torch.cat([self.loss.detach().view(1), self.verts.grad.view(-1), self.attr.grad.view(-1)], out=self.outbuf)
        return self.outbuf

    def __call__(self):
        self.graph.replay()
        return self.loss


class BatchStep:
    """The same step through the batching form (one item): fused raster +
    interpolation, antialias, fused backward (diffrp_gb300.batch)."""

    def __init__(self, dev, f, mvp, target, V, C, tile=(4, 0), fused_loss=True, grads_in_forward=True):
        import torch
        from diffrp_gb300.batch import BatchRenderer
        self.torch = torch
        self.grads_in_forward = grads_in_forward
        self.tri = torch.from_numpy(f).to(dev)
        self.mvp = torch.from_numpy(mvp).to(dev)
        self.target = torch.from_numpy(target).to(dev).reshape(-1)
        self.fused_loss = fused_loss
        self.renderer = BatchRenderer([(self.tri, V, C)], [(0, (H, W))], device=dev, tile_log2=tile[0],
                                      threads_per_tri=tile[1])

    def __call__(self, verts, attr):
        torch = self.torch
        verts.grad = None
        attr.grad = None
        clip = clip_space(verts, self.mvp)
        if self.fused_loss:
            loss, _ = self.renderer.render_l1(clip, attr.reshape(-1), self.target,
                                              grads_in_forward=self.grads_in_forward)
        else:
            loss = l1_loss(self.renderer(clip, attr.reshape(-1)), self.target)
        loss.backward()
        return loss


def kernel_launches():
    """Kernel launches libdiffrp_gb300 has enqueued (captures included)."""
    from diffrp_gb300 import _ffi
    return _ffi.kernel_launches()


# ---------------------------------------------------------------------------
# Batched workloads (the batching form against plain per-item launches)
# ---------------------------------------------------------------------------
def _graph(fn, dev, warm=3):
    """Capture fn (a fwd+bwd step) in a CUDA graph after warm-up on a side stream."""
    import torch
    side = torch.cuda.Stream(dev)
    side.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(side):
        for _ in range(warm):
            fn()
    torch.cuda.current_stream(dev).wait_stream(side)
    torch.cuda.synchronize(dev)
    g = torch.cuda.CUDAGraph()
    n0 = kernel_launches()
    with torch.cuda.graph(g):
        fn()
    g.launches_per_step = kernel_launches() - n0
    torch.cuda.synchronize(dev)
    return g


class MultiViewWorkload:
    """items = (mesh, view, resolution) renders with per-mesh attributes;
    clip positions come from per-item MVPs applied to the mesh vertices (so
    gradients reach the vertices).  Provides the batched step and the plain
    per-item step over the drop-in nvdr calls, both L1 to a seeded target."""

    def __init__(self, dev, meshes, items, seed=0, recompute=False, tile=None):
        import torch
        from diffrp_gb300.batch import BatchRenderer
        self.torch = torch
        self.dev = dev
        rng = np.random.default_rng(seed)
        self.verts = [torch.from_numpy(v).to(dev).requires_grad_(True) for v, _, _ in meshes]
        self.attrs = [torch.from_numpy(rng.uniform(0, 1, (len(v), c)).astype(np.float32)).to(dev).requires_grad_(True)
                      for v, _, c in meshes]
        self.tris = [torch.from_numpy(f).to(dev) for _, f, _ in meshes]
        self.items = [(m, (H, W)) for m, (H, W), _ in items]
        self.mvps = [torch.from_numpy(mvp.astype(np.float32)).to(dev) for _, _, mvp in items]
        self.pixels = sum(H * W for _, (H, W), _ in items)
        self.channels = [meshes[m][2] for m, _, _ in items]
        tl, tpt = (tile if tile is not None else (4, 0))
        self.renderer = BatchRenderer([(t, len(v), c) for t, (v, _, c) in zip(self.tris, meshes)], self.items,
                                      device=dev, tile_log2=tl, threads_per_tri=tpt, recompute=recompute)
        self.target = torch.from_numpy(rng.uniform(0, 1, self.renderer.image_floats).astype(np.float32)).to(dev)
        self.targets = self.renderer.images(self.target)
        # items grouped by mesh (every workload here): one batched transform per
        # mesh, (n_m, 4, 4) MVPs against the mesh's (V, 4) vertices
        order = [m for m, _ in self.items]
        self.grouped = order == sorted(order)
        self.mesh_mvps = []
        for m in range(len(self.verts)):
            ks = [k for k, (mm, _) in enumerate(self.items) if mm == m]
            self.mesh_mvps.append(torch.stack([self.mvps[k] for k in ks]) if ks else None)
        from diffrp_gb300 import nvdr
        self.nvdr = nvdr
        self.ctx = nvdr.RasterizeCudaContext(dev)
        self.topos = [nvdr.antialias_construct_topology_hash(t) for t in self.tris]

    def _clip(self, m, k):
        return clip_space(self.verts[m], self.mvps[k])

    def _zero(self):
        for t in self.verts + self.attrs:
            t.grad = None

    def _packed_clip(self):
        from diffrp_gb300.transform import clip_space_packed
        if not self.grouped:
            return clip_space_packed([(self.verts[m], self.mvps[k]) for k, (m, _) in enumerate(self.items)])
        # one transform launch per mesh over its (n, 4, 4) view matrices,
        # written straight into the packed position buffer
        return clip_space_packed([(v, mv) for v, mv in zip(self.verts, self.mesh_mvps) if mv is not None])

    def batched_step(self):
        """The batching form with the L1 loss and its gradient formed in its
        antialias pass."""
        self._zero()
        pos = self._packed_clip()
        attr = self.torch.cat([a.reshape(-1) for a in self.attrs])
        loss, _ = self.renderer.render_l1(pos, attr, self.target, grads_in_forward=True)
        loss.backward()
        return loss

    def plain_step(self):
        self._zero()
        dr = self.nvdr
        loss = 0
        n = self.renderer.image_floats
        for k, (m, (H, W)) in enumerate(self.items):
            clip = self._clip(m, k)
            rast, _ = dr.rasterize(self.ctx, clip, self.tris[m], (H, W), grad_db=False)
            col, _ = dr.interpolate(self.attrs[m], rast, self.tris[m])
            aa = dr.antialias(col, rast, clip, self.tris[m], topology_hash=self.topos[m])
            loss = loss + l1_loss(aa[0], self.targets[k]) * (self.targets[k].numel() / n)
        loss.backward()
        return loss


def views64_workload(dev):
    """64 views of the icosphere-3 mesh (642 verts, 1280 tris, radius 0.8),
    eyes uniform on a radius-3.2 sphere (seed 0), fov 30, 512x512, 8 channels."""
    from diffrp_gb300 import synthetic as S
    v, f = S.icosphere(3, 0.8)
    P = S.perspective(30.0, 512, 512, 0.1, 100.0).astype(np.float64)
    items = [(0, (512, 512), P @ S.view_matrix(S.lookat_pose(e)).astype(np.float64))
             for e in S.sphere_eyes(64, 3.2, seed=0)]
    return [(v, f, 8)], items


def uneven48_workload(dev, seed=0):
    """48 meshes (icospheres or displaced grids, triangle counts log-uniform in
    [1e3, 5e5]), random rotation, scale U(0.5, 1.2), 1-4 views each from
    {256, 512, 1024}^2, 4-16 channels."""
    from diffrp_gb300 import synthetic as S
    rng = np.random.default_rng(seed)
    meshes, items = [], []
    for m in range(48):
        F = float(np.exp(rng.uniform(np.log(1e3), np.log(5e5))))
        if rng.uniform() < 0.5:
            sub = int(np.clip(round(np.log(F / 20.0) / np.log(4.0)), 3, 7))
            v, f = S.icosphere(sub, 1.0)
        else:
            n = int(round(np.sqrt(F / 2.0))) + 1
            v, f = S.random_displaced_grid(n, seed=seed * 1000 + m, sigma=0.03)
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        v = (v.astype(np.float64) @ q.T) * rng.uniform(0.5, 1.2)
        c = int(rng.integers(4, 17))
        meshes.append((v.astype(np.float32), f, c))
        for _ in range(int(rng.integers(1, 5))):
            res = int(rng.choice([256, 512, 1024]))
            eye = S.sphere_eyes(1, 3.2, seed=int(rng.integers(1 << 30)))[0]
            mvp = S.perspective(30.0, res, res, 0.1, 100.0).astype(np.float64) @ \
                S.view_matrix(S.lookat_pose(eye)).astype(np.float64)
            items.append((m, (res, res), mvp))
    return meshes, items


def large16_workload(dev, seed=0):
    """1024x1024-vertex heightfield (2,093,058 tris) on [-1, 1]^2 with 6-octave
    value noise of amplitude 0.3, 16 oblique views at 2048x2048, 12 channels."""
    from diffrp_gb300 import synthetic as S
    v, f = S.heightfield(1024, 0.3, 6, seed)
    items = []
    for k in range(16):
        az = 2 * np.pi * k / 16
        el = np.radians(35.0 + 10.0 * np.sin(3 * az))
        eye = 2.6 * np.array([np.cos(az) * np.cos(el), np.sin(az) * np.cos(el), np.sin(el)])
        mvp = S.perspective(40.0, 2048, 2048, 0.1, 20.0).astype(np.float64) @ \
            S.view_matrix(S.lookat_pose(eye, up=(0.0, 0.0, 1.0))).astype(np.float64)
        items.append((0, (2048, 2048), mvp))
    return [(v, f, 12)], items


_WORKLOADS = {}  # generated batched workloads (meshes, items), reused by later runs


def run_batched(dev, name, steps, warmup, plain=True, recompute=False, tune=True, tile=None):
    """Mpix/s of the batched form (graph-captured) and of the plain per-item
    drop-in calls (eager, and graph-captured when it fits) on one workload."""
    import torch
    from diffrp_gb300 import autotune
    if name not in _WORKLOADS:
        _WORKLOADS[name] = {"views64": views64_workload, "uneven48": uneven48_workload,
                            "large16": large16_workload}[name](dev)
    meshes, items = _WORKLOADS[name]
    torch.cuda.empty_cache()
    torch.cuda.reset_peak_memory_stats(dev)
    wl = MultiViewWorkload(dev, meshes, items, recompute=recompute, tile=tile)
    if tune and tile is None:
        with torch.no_grad():
            pos0 = torch.cat([wl._clip(m, k) for k, (m, _) in enumerate(wl.items)])
            attr0 = torch.cat([a.reshape(-1) for a in wl.attrs])
            ch = autotune.tune_batch(wl.renderer, pos0, attr0, reps=3)
        tile = (ch["tile_log2"], ch["threads_per_tri"])
    res = {"items": len(items), "meshes": len(meshes), "pixels_per_step": wl.pixels,
           "triangles_per_step": int(sum(len(meshes[m][1]) for m, _, _ in items)),
           "tile": 1 << (tile or (4, 0))[0], "threads_per_tri": (tile or (4, 0))[1]}
    g = _graph(wl.batched_step, dev, warm=max(2, warmup))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    s = torch.cuda.current_stream(dev)

    def timed(fn, n):
        for _ in range(max(3, warmup)):  # untimed warm-up of this exact callable
            fn()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        torch.cuda.synchronize(dev)
        for i in range(n):
            flush.fill_(i & 0xff)
            evs[i][0].record(s)
            fn()
            evs[i][1].record(s)
        torch.cuda.synchronize(dev)
        return sum(a.elapsed_time(b) for a, b in evs) / n

    ms = timed(g.replay, steps)
    peak, _ = _peaks()
    nbytes = step_bytes(meshes, items, recompute)
    res["step_bytes"] = nbytes
    res["batched"] = {"value": wl.pixels / ms / 1e3, "unit": UNIT, "ms_per_step": ms,
                      "launches_per_step": g.launches_per_step, "path": "batched, one CUDA graph",
                      "step_roofline_frac": nbytes / (ms / 1e3) / 1e9 / peak}
    res["peak_memory_gb"] = torch.cuda.max_memory_allocated(dev) / 1e9
    res["batched"]["recompute"] = bool(recompute)
    if recompute:
        res["batched"]["chunks"] = len(wl.renderer._chunks)
    if plain:
        for _ in range(max(2, warmup)):
            n0 = kernel_launches()
            wl.plain_step()
            plain_launches = kernel_launches() - n0
        ms_p = timed(wl.plain_step, max(3, steps // 4))
        res["plain_eager"] = {"value": wl.pixels / ms_p / 1e3, "unit": UNIT, "ms_per_step": ms_p,
                              "launches_per_step": plain_launches,
                              "step_roofline_frac": step_bytes(meshes, items) / (ms_p / 1e3) / 1e9 / peak}
        try:
            gp = _graph(wl.plain_step, dev, warm=2)
            ms_g = timed(gp.replay, steps)
            res["plain_graphed"] = {"value": wl.pixels / ms_g / 1e3, "unit": UNIT, "ms_per_step": ms_g,
                                    "step_roofline_frac": step_bytes(meshes, items) / (ms_g / 1e3) / 1e9 / peak}
        except RuntimeError as e:  # pragma: no cover
            res["plain_graphed"] = {"unavailable": str(e)[:200]}
    return res


def step_bytes(meshes, items, recompute=False):
    """Algorithmic bytes of one fwd+bwd (the path's byte model): per pixel
    16 rast write + 16 rast read (dropped when rasterisation is recomputed)
    + 4C image write + 4C gradient read; per item V (16 clip read + 16 position
    gradient write) + 24 F; per mesh V * 8C (attribute read + gradient write)."""
    total = 0
    for m, (h, w), _ in items:
        v, f, c = meshes[m]
        total += h * w * ((0 if recompute else 32) + 8 * c) + len(v) * 32 + 24 * len(f)
    for v, f, c in meshes:
        total += len(v) * 8 * c
    return total


WORKLOAD_C1 = ("icosphere3 642 verts / 1280 tris (flat normals: 3840-vertex face soup), 512x512, camera-space "
               "normals (3 ch), nvdr_antialias, L2 loss to a seeded N(0, 0.1) target, fwd+bwd to the leaf vertices")


def c1_target(seed, h, w):
    """N(0, 0.1) target (h, w, 3) by Box-Muller over PCG64 uniform doubles."""
    u = np.random.default_rng(int(seed)).random((2, h, w, 3))
    return (0.1 * np.sqrt(-2.0 * np.log1p(-u[0])) * np.cos(2.0 * np.pi * u[1])).astype(np.float32)


def run_config1(dev, steps, warmup):
    """The README example at benchmark size through the session API
    (SurfaceDeferredRenderSession): scene, mesh object and session built
    every step as a training loop does, camera-space normals, nvdr_antialias,
    L2 loss, backward to the leaf vertices.  Eager with each interpolator
    implementation, and the full-screen form captured as one CUDA graph."""
    import torch
    from diffrp_gb300 import materials, synthetic as S
    from diffrp_gb300.scene import MeshObject, Scene
    from diffrp_gb300.rendering.camera import PerspectiveCamera
    from diffrp_gb300.rendering.surface_deferred import (SurfaceDeferredRenderSession,
                                                         SurfaceDeferredRenderSessionOptions)
    h = w = 512
    v, f = S.icosphere(3, 0.8)
    verts = torch.from_numpy(v).to(dev).requires_grad_(True)
    tris = torch.from_numpy(f).to(dev)
    target = torch.from_numpy(c1_target(0, h, w)).to(dev)
    cam = PerspectiveCamera(h=h, w=w, far=100.0)

    def make_step(impl, leaf):
        opts = SurfaceDeferredRenderSessionOptions(interpolator_impl=impl)

        def step():
            leaf.grad = None
            scene = Scene()
            scene.add_mesh_object(MeshObject(materials.DefaultMaterial(), leaf, tris))
            rp = SurfaceDeferredRenderSession(scene, cam, options=opts)
            n = rp.false_color_camera_space_normal()
            aa = rp.nvdr_antialias(n[..., :3])
            loss = (aa - target).square().mean()
            loss.backward()
            return loss
        return step

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    s = torch.cuda.current_stream(dev)

    def timed(fn, n):
        for _ in range(max(3, warmup)):
            fn()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        torch.cuda.synchronize(dev)
        for i in range(n):
            flush.fill_(i & 0xff)
            evs[i][0].record(s)
            fn()
            evs[i][1].record(s)
        torch.cuda.synchronize(dev)
        return sum(a.elapsed_time(b) for a, b in evs) / n

    px = h * w
    nbytes = step_bytes([(np.zeros((3 * len(f), 3)), f, 3)], [(0, (h, w), None)])
    peak, _ = _peaks()
    res = {"workload": WORKLOAD_C1, "pixels_per_step": px, "step_bytes": nbytes}
    for impl in ("stencil_masked", "full_screen"):
        st = make_step(impl, verts)
        n0 = kernel_launches()
        st()
        launches = kernel_launches() - n0
        ms = timed(st, steps)
        res["eager_" + impl] = {"value": px / ms / 1e3, "unit": UNIT, "ms_per_step": ms,
                                "library_launches_per_step": launches}
    try:
        # a leaf of its own: one first differentiated on the legacy stream
        # (the eager runs above) keeps that stream for its gradient
        # accumulation, which a capture cannot wait on
        leaf = verts.detach().clone().requires_grad_(True)
        g = _graph(make_step("full_screen", leaf), dev, warm=max(2, warmup))
        ms = timed(g.replay, steps)
        res["graphed_full_screen"] = {"value": px / ms / 1e3, "unit": UNIT, "ms_per_step": ms,
                                      "library_launches_per_step": g.launches_per_step,
                                      "step_roofline_frac": nbytes / (ms / 1e3) / 1e9 / peak}
    except RuntimeError as e:  # pragma: no cover
        res["graphed_full_screen"] = {"unavailable": str(e)[:200]}
    return res


WORKLOAD_TEX = ("1024x1024 RGBA texture, trilinear (linear-mipmap-linear, wrap), sampled at the 1024x1024 pixels of a "
                "receding ground plane (uv tiled 16 x 64, uv / uv_da from rasterize + interpolate, levels 0-10), "
                "fwd+bwd to the texture (through the pyramid), uv and uv_da")


def texture_inputs(dev, n=1024, tex_n=1024, seed=0):
    """uv and uv_da of a ground plane seen at a grazing angle (interpolated
    once, outside the timed region), and a random texture."""
    import torch
    from diffrp_gb300 import nvdr as dr
    pos = torch.tensor([[-1, -1, 0.2, 1], [1, -1, 0.2, 1], [-12, 16, 0.99, 16], [12, 16, 0.99, 16]],
                       dtype=torch.float32, device=dev)
    tri = torch.tensor([[0, 1, 2], [1, 3, 2]], dtype=torch.int32, device=dev)
    uvs = torch.tensor([[0, 0], [16, 0], [0, 64], [16, 64]], dtype=torch.float32, device=dev)
    rast, db = dr.rasterize(dr.RasterizeCudaContext(dev), pos, tri, (n, n))
    uv, uv_da = dr.interpolate(uvs, rast, tri, rast_db=db, diff_attrs="all")
    g = torch.Generator(device=dev).manual_seed(seed)
    tex = torch.rand((1, tex_n, tex_n, 4), generator=g, device=dev)
    return tex, uv.contiguous(), uv_da.contiguous()


def run_texture(dev, steps, warmup, cpu=True):
    """Mip-mapped texture sampling (nvdr.texture), fwd+bwd as one CUDA graph,
    L2 flushed between steps; the CPU oracle on a sample of rows beside it."""
    import torch
    from diffrp_gb300 import nvdr as dr
    n = 1024
    tex0, uv0, da0 = texture_inputs(dev, n)
    tex = tex0.clone().requires_grad_(True)
    uv = uv0.clone().requires_grad_(True)
    da = da0.clone().requires_grad_(True)
    gout = torch.rand((1, n, n, 4), device=dev)

    def step():
        tex.grad = uv.grad = da.grad = None
        out = dr.texture(tex, uv, da, filter_mode="linear-mipmap-linear", boundary_mode="wrap")
        out.backward(gout)
        return out

    g = _graph(step, dev, warm=max(2, warmup))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    s = torch.cuda.current_stream(dev)
    for _ in range(max(3, warmup)):
        g.replay()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize(dev)
    for i in range(steps):
        flush.fill_(i & 0xff)
        evs[i][0].record(s)
        g.replay()
        evs[i][1].record(s)
    torch.cuda.synchronize(dev)
    ms = sum(a.elapsed_time(b) for a, b in evs) / steps
    P = n * n
    T = tex.numel() * 4  # texture bytes; the pyramid adds a third
    # pixel streams: uv, uv_da, output (fwd) + grad_out, uv, uv_da, grad_uv,
    # grad_uv_da (bwd); texture streams: pyramid build (read T, write T/3),
    # texels read by fwd and bwd (4T/3 each), gradient pyramid (zero T/3,
    # texel gradients 4T/3, pyramid backward T/3 + grad_tex 2T)
    nbytes = P * (8 + 16 + 16 + 16 + 8 + 16 + 8 + 16) + int(T * (1 + 1 / 3 + 8 / 3 + 1 / 3 + 4 / 3 + 1 / 3 + 2))
    peak, _ = _peaks()
    res = {"workload": WORKLOAD_TEX, "pixels_per_step": P, "value": P / ms / 1e3, "unit": UNIT, "ms_per_step": ms,
           "step_bytes": nbytes, "step_roofline_frac": nbytes / (ms / 1e3) / 1e9 / peak,
           "launches_per_step": g.launches_per_step}
    if cpu:
        import oracle as O
        rows = 64
        t_np, uv_np, da_np = tex0.cpu().numpy(), uv0[:, :rows].cpu().numpy(), da0[:, :rows].cpu().numpy()
        g_np = gout[:, :rows].cpu().numpy()
        L = O.tex_levels(1024, 1024)
        t0 = time.perf_counter()
        pyr = O.tex_mip_build(t_np, L)
        O.tex_fwd(t_np, pyr, L, uv_np, da_np, "linear-mipmap-linear", "wrap")
        g0, gp, _, _ = O.tex_bwd(t_np, pyr, L, uv_np, da_np, g_np, "linear-mipmap-linear", "wrap")
        O.tex_mip_bwd(g0, gp, L)
        el = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": rows * n / el / 1e6, "unit": UNIT, "cores": O.default_threads(),
                               "kind": "port", "sample": "%d rows of the 1024x1024 output, fwd+bwd with the pyramid "
                                                         "of the full texture, in %.2f s (the sampling forward on "
                                                         "the threads given; the pyramid and the backward, whose "
                                                         "texel sums are shared, on one)" % (rows, el)}
    return res


def run_sharded_views64(dev, steps, warmup, rank, world):
    """The 64-view workload sharded across ranks (strong scaling): each rank
    renders its share of the views (diffrp_gb300.replicas.shard_items) as one
    batched CUDA graph and the shared mesh's vertex and attribute gradients
    are summed with one all-reduce per step.  value = all 64 views' pixels /
    the slowest rank's step time."""
    import torch
    import torch.distributed as dist
    from diffrp_gb300.replicas import allreduce_gradients, shard_items
    meshes, items = views64_workload(dev)
    mine = shard_items([(m, hw) for m, hw, _ in items], rank, world)
    wl = MultiViewWorkload(dev, meshes, [items[i] for i in mine], tile=(5, 0))
    g = _graph(wl.batched_step, dev, warm=max(2, warmup))
    params = wl.verts + wl.attrs

    def step():
        g.replay()
        allreduce_gradients(params)

    for _ in range(max(3, warmup)):
        step()
    s = torch.cuda.current_stream(dev)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    dist.barrier()
    torch.cuda.synchronize(dev)
    for i in range(steps):
        evs[i][0].record(s)
        step()
        evs[i][1].record(s)
    torch.cuda.synchronize(dev)
    ms = sum(a.elapsed_time(b) for a, b in evs) / steps
    t = torch.tensor([ms], device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    total_px = sum(h * w for _, (h, w), _ in items)
    return {"value": total_px / float(t[0]) / 1e3, "unit": UNIT, "ms_per_step": float(t[0]), "scaling": "strong",
            "items_per_rank": len(mine), "pixels_per_step": total_px,
            "path": "views sharded across ranks, batched CUDA graph per rank, one all-reduce of the shared "
                    "mesh's gradients per step"}


def _clock_sampler():
    f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
    try:
        p = subprocess.Popen(["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                              "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                             stdout=f, stderr=subprocess.DEVNULL)
    except (OSError, FileNotFoundError):
        return None, f.name
    return p, f.name


def _hold_load(fn, seconds):
    """Replay fn (untimed) for about `seconds`, so that the clock sampler
    (nvidia-smi every 200 ms) sees the GPU under the timed step's own load."""
    import torch
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        for _ in range(20):
            fn()
        torch.cuda.synchronize()


def _clock_summary(proc, path, gpu_index):
    if proc is None:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    proc.terminate()
    try:
        proc.wait(timeout=5)
    except subprocess.TimeoutExpired:
        proc.kill()
    sms, maxs, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    with open(path) as fh:
        for line in fh:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9 or not parts[0].isdigit() or int(parts[0]) != gpu_index:
                continue
            try:
                sms.append(float(parts[1]))
                maxs.append(float(parts[2]))
            except ValueError:
                continue
            for n, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(n)
    os.unlink(path)
    return {"sm_mhz": statistics.median(sms) if sms else None, "sm_max_mhz": max(maxs) if maxs else None,
            "samples": len(sms), "reasons": sorted(reasons)}


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def kernel_breakdown(dev, verts, f, attr, mvp, target, reps=10, tuned=None, batch=None):
    """CUDA-event time of each C-ABI entry point of the step on the same
    inputs: each entry point is captured alone in a CUDA graph and replayed
    between events on the launching stream, L2 flushed before every replay."""
    import torch
    from diffrp_gb300 import _ffi
    from diffrp_gb300 import nvdr as dr
    s = torch.cuda.current_stream(dev)

    class _CurStream:
        """ctypes argument: the stream current at call time (graph capture
        switches streams)."""

        @property
        def _as_parameter_(self):
            return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)

    sp = _CurStream()
    ctx = dr.RasterizeCudaContext(dev)
    if tuned is not None:
        from diffrp_gb300 import autotune
        autotune.apply(ctx, tuned)
    tri = torch.from_numpy(f).to(dev)
    v_t = torch.from_numpy(verts).to(dev)
    clip = clip_space(v_t, torch.from_numpy(mvp).to(dev)).contiguous()
    a_t = torch.from_numpy(attr).to(dev)
    topo = dr.antialias_construct_topology_hash(tri)
    rast, _ = dr.rasterize(ctx, clip, tri, (H, W), grad_db=False)
    col, _ = dr.interpolate(a_t, rast, tri)
    aa = dr.antialias(col, rast, clip, tri, topology_hash=topo)
    g = torch.sign(aa - torch.from_numpy(target).to(dev)) / aa.numel()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    V, F = clip.shape[0], tri.shape[0]
    gpos = torch.zeros_like(clip)
    gattr = torch.zeros_like(a_t)
    gcol = torch.empty_like(col)
    grast = torch.empty_like(rast)
    out = torch.empty_like(col)
    aws = torch.empty(_ffi.size_out("drp_antialias_workspace_size", 1, F), dtype=torch.uint8, device=dev)
    astate = torch.empty(_ffi.size_out("drp_antialias_state_size", 1, H, W), dtype=torch.uint8, device=dev)
    ops = {
        "rasterize_fwd": lambda: ctx._raster_call(clip, tri, None, 1, F, H, W, 0, None, rast, None, None),
        "interpolate_fwd": lambda: _ffi.call("drp_interpolate_fwd", a_t.data_ptr(), 0, V, C, rast.data_ptr(), None,
                                             tri.data_ptr(), F, 1, H, W, None, 0, out.data_ptr(), None, sp),
        "antialias_fwd": lambda: _ffi.call("drp_antialias_fwd", aws.data_ptr(), aws.numel(), col.data_ptr(), C,
                                           rast.data_ptr(), clip.data_ptr(), 0, V, tri.data_ptr(), F,
                                           topo.data_ptr(), 1, H, W, out.data_ptr(), astate.data_ptr(), sp),
        "antialias_bwd": lambda: _ffi.call("drp_antialias_bwd", aws.data_ptr(), aws.numel(), col.data_ptr(), C,
                                           rast.data_ptr(), clip.data_ptr(), 0, V, tri.data_ptr(), F,
                                           topo.data_ptr(), 1, H, W, g.data_ptr(), 1.0, gcol.data_ptr(),
                                           gpos.data_ptr(), astate.data_ptr(), sp),
        "interpolate_bwd": lambda: _ffi.call("drp_interpolate_bwd", a_t.data_ptr(), 0, V, C, rast.data_ptr(), None,
                                             tri.data_ptr(), F, 1, H, W, None, 0, gcol.data_ptr(), None,
                                             gattr.data_ptr(), grast.data_ptr(), None, sp),
        "rasterize_bwd": lambda: _ffi.call("drp_rasterize_bwd", clip.data_ptr(), 0, V, tri.data_ptr(), F, 1, H, W,
                                           rast.data_ptr(), grast.data_ptr(), None, gpos.data_ptr(), sp),
    }
    if batch is not None:
        b_rast, b_color, b_out = batch.forward_buffers(clip, a_t)
        b_g = g.reshape(-1).contiguous()
        b_gp = torch.zeros_like(clip)
        b_ga = torch.zeros_like(a_t).reshape(-1)
        flat_attr = a_t.reshape(-1)
        b_flags = batch._flags()
        ops["batch_forward"] = lambda: batch._forward_raw(clip, flat_attr, b_rast, b_color, b_out, flags=b_flags)
        b_target = torch.from_numpy(target).to(dev).reshape(-1)
        b_grad = torch.empty_like(b_color)
        b_blocks = torch.empty(max(1, batch.pixel_blocks), dtype=torch.float32, device=dev)
        b_loss = torch.empty((), dtype=torch.float32, device=dev)
        ops["batch_forward_l1"] = lambda: batch._forward_raw(
            clip, flat_attr, b_rast, b_color, b_out, (b_target, 1.0 / b_color.numel(), b_grad, b_blocks, b_loss),
            flags=b_flags)
        # the step's backward reuses the antialias records and slot bits of its forward
        ops["batch_backward"] = lambda: batch._backward_raw(clip, flat_attr, b_rast, b_color, b_g, b_gp, b_ga,
                                                            batch._fwd_gen, aa_flags=b_flags)
        # the headline step's forward: loss and its gradient in one pass (its
        # first kernel zeroes the gradient buffers, as in the step)
        b_gbuf = torch.zeros(clip.numel() + flat_attr.numel(), dtype=torch.float32, device=dev)

        def fwd_l1_grad():
            batch._forward_raw(clip, flat_attr, b_rast, b_color, b_out,
                               (b_target, 1.0 / b_color.numel(), b_blocks, b_loss, b_gbuf[:clip.numel()].view_as(clip),
                                b_gbuf[clip.numel():], b_gbuf), flags=b_flags)
        ops["batch_forward_l1_grad"] = fwd_l1_grad
    P = H * W
    # Algorithmic bytes per launch: every input read once, every output written once.
    algo = {
        "rasterize_fwd": P * 16 + V * 16 + F * 12,
        "interpolate_fwd": P * (16 + 4 * C) + V * 4 * C,
        "antialias_fwd": P * (4 * C + 16 + 4 * C),
        "antialias_bwd": P * (4 * C + 4 * C + 16 + 4 * C) + V * 16,
        "interpolate_bwd": P * (4 * C + 16 + 16) + V * 4 * C * 2,
        "rasterize_bwd": P * (16 + 16) + V * 16 * 2,
        # outputs written once (rast, colour, antialiased output), vertex
        # positions / attributes / triangles read once
        "batch_forward": P * (16 + 4 * C + 4 * C) + V * (16 + 4 * C) + F * 12,
        # the same plus the loss: target read, sign gradient written
        "batch_forward_l1": P * (16 + 4 * C * 4) + V * (16 + 4 * C) + F * 12,
        # rast, colour and output gradient read once; vertex / attribute
        # gradients written once
        "batch_backward": P * (16 + 4 * C + 4 * C) + V * (16 + 4 * C) * 2 + F * 12,
        # rast, colour and output written, target read; vertex / attribute
        # gradients written (no sign-gradient image)
        "batch_forward_l1_grad": P * (16 + 4 * C * 3) + V * (16 + 4 * C) * 2 + F * 12,
    }
    times = {}
    for name, fn in ops.items():
        # capture the entry point alone in a CUDA graph so that the timing is
        # the device time of its kernels, not host launch overhead
        fn()
        torch.cuda.synchronize(dev)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            fn()
        graph.replay()
        torch.cuda.synchronize(dev)
        ts = []
        for _ in range(reps):
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            graph.replay()
            e1.record(s)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        times[name] = statistics.median(ts)
    return times, algo


def cpu_baseline(verts, f, attr, mvp, target, budget_s=8.0):
    """The CPU oracle on the same workload: rows of the image are the sample
    unit (whole steps when they fit in the budget)."""
    import oracle as O
    nthreads = O.default_threads()
    clip = (np.concatenate([verts, np.ones((len(verts), 1), np.float32)], 1).astype(np.float64) @
            mvp.astype(np.float64).T).astype(np.float32)
    nbr = O.topology(f)
    steps = 0
    t0 = time.perf_counter()
    while True:
        rast, _, _ = O.rasterize(clip, f, (H, W), grad_db=False, nthreads=nthreads)
        col, _ = O.interpolate(attr, rast, f, nthreads=nthreads)
        aa = O.antialias(col, rast, clip, f, nbr, nthreads=nthreads)
        g = np.sign(aa - target) / aa.size
        gc, gp = O.antialias_bwd(col, rast, clip, f, g, nbr, nthreads=nthreads)
        ga, gr, _ = O.interpolate_bwd(attr, rast, f, gc, nthreads=nthreads)
        O.raster_bwd(clip, f, rast, gr, nthreads=nthreads)
        steps += 1
        el = time.perf_counter() - t0
        if el >= budget_s or steps >= 50:
            break
    return {"value": steps * H * W / el / 1e6, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": "%d full fwd+bwd step(s) of the %dx%d, 20480-triangle, 8-channel workload in %.1f s"
                      % (steps, H, W, el)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    verts, f, attr, mvp, target = make_workload()
    for _ in range(max(args.warmup, 0)):
        pass
    base = cpu_baseline(verts, f, attr, mvp, target, budget_s=max(4.0, 2.0 * args.steps))
    line = {
        "impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": H * W / base["value"] / 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD_SINGLE,
                   "global_batch": 1, "resolution": [H, W], "channels": C, "parallelism": "cpu threads"},
        "cpu_baseline": base,
        "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="full", choices=["full", "steps"],
                    help="steps: only the warm-up and timed device-resident steps (for profilers)")
    ap.add_argument("--workload", default="single", choices=["single", "views64", "uneven48", "large16", "texture"],
                    help="single: the headline single-mesh line (with the 64-view batched comparison "
                         "attached); others: one line for that batched workload, or the mip-mapped "
                         "texture workload")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the attached lines (64 views, config-1 session, 48 meshes, large heightfield)")
    ap.add_argument("--tile", default=None,
                    help="fixed raster shape 'tile_log2,threads_per_tri' instead of autotuning (profiling runs)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    import __graft_entry__
    __graft_entry__.build()
    if args.workload == "texture":
        W_ = max(3, args.warmup)
        res = run_texture(dev, steps=args.steps, warmup=W_, cpu=rank == 0 and not args.no_cpu_baseline)
        if rank == 0:
            print(json.dumps({
                "metric": "fwd+bwd Mpix/s (mip pyramid, trilinear texture sample, backward to texture, uv and uv_da)",
                "value": res["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
                "warmup": W_, "ms_per_step": res["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded texture and gradient)",
                "config": {"workload": WORKLOAD_TEX, "parallelism": "single GPU",
                           "l2": "flushed between steps (256 MiB write outside the timed events)"},
                "gpu_launches": res["launches_per_step"] * args.steps, "detail": res}))
        if world > 1:
            dist.destroy_process_group()
        return 0
    if args.workload != "single":
        W_ = max(3, args.warmup)
        fixed = tuple(int(x) for x in args.tile.split(",")) if args.tile else None
        res = run_batched(dev, args.workload, steps=args.steps, warmup=W_, plain=args.workload != "large16",
                          recompute=args.workload == "large16", tile=fixed)
        if world > 1:
            t = torch.tensor([res["batched"]["ms_per_step"]], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            res["batched"]["ms_per_step"] = float(t[0])
            res["batched"]["value"] = res["pixels_per_step"] * world / float(t[0]) / 1e3
        if rank == 0:
            desc = {"views64": "64 views of icosphere-3 (1280 tris), 512x512, 8 ch",
                    "uneven48": "48 meshes, 1e3-5e5 tris (log-uniform), 1-4 views at 256/512/1024, 4-16 ch",
                    "large16": "2.09M-tri heightfield, 16 views at 2048x2048, 12 ch, recompute in backward"}
            print(json.dumps({
                "metric": METRIC, "value": res["batched"]["value"], "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": W_, "ms_per_step": res["batched"]["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded meshes, cameras, attributes and targets)",
                "config": {"workload": desc[args.workload], "global_batch": res["items"] * world,
                           "parallelism": "replicas" if world > 1 else "single GPU",
                           "l2": "flushed between steps (256 MiB write outside the timed events)"},
                "gpu_launches": res["batched"]["launches_per_step"] * args.steps,
                "detail": res}))
        if world > 1:
            dist.destroy_process_group()
        return 0

    verts_np, f, attr_np, mvp, target = make_workload()
    step = Step(dev, f, mvp, target)
    from diffrp_gb300 import autotune
    with torch.no_grad():
        clip0 = clip_space(torch.from_numpy(verts_np).to(dev), step.mvp)
    if args.tile:
        tl, tpt = [int(x) for x in args.tile.split(",")]
        tuned = {"tile_log2": tl, "threads_per_tri": tpt}
        autotune.apply(step.ctx, tuned)
        step.ctx.ensure_capacity(0)
        step.ctx._sized = False
        tuned["list_capacity"] = None
    else:
        tuned = autotune.tune_rasterizer(step.ctx, clip0.contiguous(), step.tri, (H, W), use_cache=False)
    verts = torch.from_numpy(verts_np).to(dev).requires_grad_(True)
    attr = torch.from_numpy(attr_np).to(dev).requires_grad_(True)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    W_ = max(3, args.warmup)
    if args.mode != "steps":
        for _ in range(W_):
            step(verts, attr)
        torch.cuda.synchronize()
        graphed = GraphedStep(step, verts_np, attr_np, dev)
        for _ in range(W_):
            graphed()
    bstep = BatchStep(dev, f, mvp, target, len(verts_np), C, tile=(tuned["tile_log2"], tuned["threads_per_tri"]))
    if not args.tile:
        with torch.no_grad():
            btuned = autotune.tune_batch(bstep.renderer, clip0.contiguous(),
                                         torch.from_numpy(attr_np).to(dev).reshape(-1))
    else:
        btuned = {"tile_log2": tuned["tile_log2"], "threads_per_tri": tuned["threads_per_tri"]}
    batched = GraphedStep(bstep, verts_np, attr_np, dev)
    for _ in range(W_):
        batched()
    # the same batching form with the loss's gradient from a backward pass,
    # and with the separate l1_loss op (reported beside)
    bstep.grads_in_forward = False
    batched_bwd_pass = None if args.mode == "steps" else GraphedStep(bstep, verts_np, attr_np, dev)
    bstep.grads_in_forward = True
    bstep.fused_loss = False
    batched_unfused = None if args.mode == "steps" else GraphedStep(bstep, verts_np, attr_np, dev)
    bstep.fused_loss = True
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    s = torch.cuda.current_stream(dev)

    def timed(fn, n):
        for _ in range(W_):  # untimed warm-up of this exact callable (first launches load their kernels)
            fn()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        barrier()
        for i in range(n):
            flush.fill_(i & 0xff)
            evs[i][0].record(s)
            fn()
            evs[i][1].record(s)
        barrier()
        return sum(a.elapsed_time(b) for a, b in evs)

    # -- device-resident timing: the batching form captured as one CUDA graph
    # is the headline; the drop-in (plain per-op) path is reported beside it,
    # graph-captured and eager ---------------------------------------------
    # clocks: sampled while the headline graph runs, the same replays
    # continuing untimed around the timed steps so that the 200 ms sampler
    # records several samples under that load
    clk, clk_path = _clock_sampler()
    if args.mode == "full":
        _hold_load(batched, 0.6)
    total_ms = timed(batched, args.steps)
    if args.mode == "full":
        _hold_load(batched, 0.3)
        clocks = _clock_summary(clk, clk_path, dev.index if dev.index is not None else 0)
    if args.mode == "steps":
        if clk is not None:
            clk.terminate()
        if rank == 0:
            print(json.dumps({"mode": "steps", "ms_per_step": total_ms / args.steps}))
        if world > 1:
            dist.destroy_process_group()
        return 0
    plain_ms = timed(graphed, args.steps)
    bwd_pass_ms = timed(batched_bwd_pass, args.steps)
    unfused_ms = timed(batched_unfused, args.steps)
    eager_ms = timed(lambda: step(verts, attr), args.steps)

    # -- end-to-end through the public API with host buffers -----------------
    # inputs from one pinned host buffer (vertices, attributes), outputs (loss,
    # vertex and attribute gradients) back into one pinned host buffer
    h_in = torch.from_numpy(pack_inputs(verts_np, attr_np)).pin_memory()
    h_out = torch.empty(1 + verts_np.size + attr_np.size, dtype=torch.float32).pin_memory()

    def e2e_of(st, zero_copy=True):
        # the host->device copy, the step and the device->host copy of its
        # results captured together as one CUDA graph
        return GraphedStep(st, verts_np, attr_np, dev, io=(h_in, h_out), zero_copy=zero_copy)

    e2e_graphs = [e2e_of(bstep), e2e_of(bstep, zero_copy=False), e2e_of(step)]
    e2e_ms, e2e_engine_ms, e2e_plain_ms = [timed(gs, args.steps) for gs in e2e_graphs]
    if world > 1:
        t = torch.tensor([total_ms, e2e_ms, eager_ms, plain_ms, e2e_plain_ms, e2e_engine_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms, e2e_ms, eager_ms, plain_ms, e2e_plain_ms, e2e_engine_ms = [float(x) for x in t]

    pix = H * W * args.steps * world
    value = pix / (total_ms / 1e3) / 1e6
    e2e_value = pix / (e2e_ms / 1e3) / 1e6
    # the 64 views sharded across the ranks (every rank takes part in its
    # all-reduce; before the attached lines, which rank 0 runs alone)
    sharded = None
    if world > 1 and not args.no_batched:
        sharded = run_sharded_views64(dev, max(5, args.steps // 3), W_, rank, world)
    h2d = h_in.numel() * 4
    d2h = h_out.numel() * 4

    if rank == 0:
        times, algo = kernel_breakdown(dev, verts_np, f, attr_np, mvp, target, tuned=tuned, batch=bstep.renderer)
        # the headline step is batch_forward_l1_grad and one scaling of the
        # gradients: that entry point dominates it
        dom = "batch_forward_l1_grad"
        peak, peak_kind = _peaks()
        achieved = algo[dom] / (times[dom] / 1e3) / 1e9
        traffic = None
        tpath = os.path.join(ROOT, "profiles", "traffic.txt")
        if os.path.exists(tpath):
            with open(tpath) as fh:
                for ln in fh:
                    parts = ln.split()
                    if len(parts) == 2 and parts[0] == dom and not ln.startswith("#"):
                        traffic = int(parts[1])
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": W_, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded icosphere, attributes and target)",
            "config": {"workload": WORKLOAD_SINGLE,
                       "global_batch": world, "resolution": [H, W], "channels": C,
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "l2": "flushed between steps (256 MiB write outside the timed events)",
                       "path": "batching form (diffrp_gb300.batch, one item) with the L1 loss and its gradient "
                               "formed in its antialias pass (BatchRenderer.render_l1, grads_in_forward; the "
                               "backward is one scaling of the gradients), whole fwd+bwd step as one CUDA graph",
                       "raster_tuning": {"tile": 1 << btuned["tile_log2"],
                                         "threads_per_tri": btuned["threads_per_tri"],
                                         "plain_path": {"tile": 1 << tuned["tile_log2"],
                                                        "threads_per_tri": tuned["threads_per_tri"]}}},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "path": "pinned host -> device copy, the step, device -> pinned host copy of loss and "
                            "gradients, captured together as one CUDA graph; the copies are kernels loading / "
                            "storing the mapped pinned buffers over the host link (diffrp_gb300.hostio)",
                    "copy_engine_value": pix / (e2e_engine_ms / 1e3) / 1e6},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                         "algorithmic_bytes": algo[dom], "kernel_ms": times[dom]},
            "kernel_ms": times,
            "batched_loss_grad_in_backward": {"value": pix / (bwd_pass_ms / 1e3) / 1e6, "unit": UNIT,
                                              "ms_per_step": bwd_pass_ms / args.steps,
                                              "note": "batching form, fused L1 loss, its gradient formed by the "
                                                      "backward pass (drp_batch_backward) instead of in the forward"},
            "batched_unfused_loss": {"value": pix / (unfused_ms / 1e3) / 1e6, "unit": UNIT,
                                     "ms_per_step": unfused_ms / args.steps,
                                     "note": "batching form, loss by the separate l1_loss op (image written, "
                                             "then read back by the loss)"},
            "plain": {"value": pix / (plain_ms / 1e3) / 1e6, "unit": UNIT, "ms_per_step": plain_ms / args.steps,
                      "note": "same step through the drop-in nvdr ops, captured as one CUDA graph"},
            "eager": {"value": pix / (eager_ms / 1e3) / 1e6, "unit": UNIT,
                      "note": "same step, drop-in nvdr ops, eager per-op launches (host-launch bound)"},
            "e2e_dropin": {"value": pix / (e2e_plain_ms / 1e3) / 1e6, "unit": UNIT,
                           "note": "end to end through the drop-in nvdr ops, host buffers (copies and step in one graph)"},
            "clocks": clocks,
            # timed regions: batched graph, its two e2e graphs, the unfused-loss batched graph, drop-in
            # graph, its e2e graph and the eager drop-in step
            "gpu_launches": (batched.launches_per_step + batched_unfused.launches_per_step +
                             batched_bwd_pass.launches_per_step +
                             graphed.launches_per_step * 2 + sum(gs.launches_per_step for gs in e2e_graphs)) *
                            args.steps,
            "launches_per_step": {"batched": batched.launches_per_step,
                                  "batched_loss_grad_in_backward": batched_bwd_pass.launches_per_step,
                                  "batched_unfused_loss": batched_unfused.launches_per_step,
                                  "dropin": graphed.launches_per_step},
        }
        if not args.no_batched:
            k_small = max(5, args.steps // 3)
            k_big = max(3, args.steps // 5)
            line["batched_views64"] = run_batched(dev, "views64", steps=k_small, warmup=W_)
            line["config1_session"] = run_config1(dev, steps=k_small, warmup=W_)
            line["batched_uneven48"] = run_batched(dev, "uneven48", steps=k_big, warmup=W_)
            big = run_batched(dev, "large16", steps=k_big, warmup=W_, plain=False, recompute=True)
            stored = run_batched(dev, "large16", steps=k_big, warmup=W_, plain=False, recompute=False,
                                 tile=(big["tile"].bit_length() - 1, big["threads_per_tri"]))
            big["stored_buffers"] = {"batched": stored["batched"], "peak_memory_gb": stored["peak_memory_gb"]}
            line["batched_large16"] = big
            line["texture_trilinear"] = run_texture(dev, steps=k_small, warmup=W_, cpu=not args.no_cpu_baseline)
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(verts_np, f, attr_np, mvp, target)
        if sharded is not None:
            line["sharded_views64"] = sharded
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
