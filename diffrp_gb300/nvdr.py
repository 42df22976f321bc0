"""nvdiffrast-compatible differentiable rasterisation ops on the GB300 kernels.

Drop-in for the ``dr`` module diffrp imports (``import nvdiffrast.torch as dr``
at diffrp/rendering/surface_deferred.py:4 and diffrp/rendering/interpolator.py:12).
diffrp calls exactly these names:

* ``RasterizeCudaContext()``                          surface_deferred.py:225
* ``DepthPeeler(ctx, pos, tri, (h, w), ranges)`` as a context manager and
  ``rasterize_next_layer()``                          surface_deferred.py:260-262
* ``interpolate(attr, rast, tri)``                    interpolator.py:83
* ``antialias(color, rast, pos, tri)``                surface_deferred.py:775

plus ``rasterize``, ``antialias_construct_topology_hash`` and the mip-mapped
``texture`` / ``texture_construct_mip`` (the consumer of interpolate's
derivatives) from the same public API.  Argument order, tensor layouts, return tuples and error types
follow nvdiffrast's documented interface; the arithmetic is this project's own
CUDA (``libdiffrp_gb300.so`` through ``_ffi``).  There is no CPU path: every op
requires CUDA tensors and the built library.
"""
import collections
import ctypes
import numbers
import threading

import numpy as np

import torch

from . import _ffi

__all__ = [
    "RasterizeCudaContext", "RasterizeGLContext", "DepthPeeler", "rasterize", "interpolate", "antialias",
    "antialias_construct_topology_hash", "texture", "texture_construct_mip", "get_log_level", "set_log_level",
]

_log_level = 1


def get_log_level():
    return _log_level


def set_log_level(level):
    global _log_level
    _log_level = int(level)


def _ptr(t):
    return None if t is None else t.data_ptr()


def _stream(device):
    return _ffi.stream_of(device)


def _capturing():
    try:
        return torch.cuda.is_current_stream_capturing()
    except Exception:  # pragma: no cover
        return False


def _check_tensor(name, t, dtype, ndims, device=None, last=None):
    if not isinstance(t, torch.Tensor):
        raise TypeError("%s must be a torch.Tensor" % name)
    if not t.is_cuda:
        raise RuntimeError("%s must reside on a CUDA device" % name)
    if t.dtype != dtype:
        raise RuntimeError("%s must have dtype %s, got %s" % (name, dtype, t.dtype))
    if t.dim() not in ndims:
        raise RuntimeError("%s must have %s dimensions, got shape %s" % (name, " or ".join(map(str, ndims)),
                                                                         tuple(t.shape)))
    if last is not None and t.shape[-1] != last:
        raise RuntimeError("%s must have last dimension %d, got shape %s" % (name, last, tuple(t.shape)))
    if device is not None and t.device != device:
        raise RuntimeError("%s is on %s but the operation runs on %s" % (name, t.device, device))


# ---------------------------------------------------------------------------
# Context
# ---------------------------------------------------------------------------

_CONSTANTS = collections.OrderedDict()  # (device, dtype, shape, bytes) -> device tensor
_CONSTANTS_MAX = 256


def _device_constant(values, dtype, device):
    """A small host array (call ranges, attribute indices, lookup tables) as
    a device tensor, copied once and kept for later calls with the same
    values: repeated calls copy nothing from the host, so they neither wait
    for the GPU nor break CUDA-graph capture.  The returned tensor is shared
    and must not be modified."""
    a = np.ascontiguousarray(values)
    dev = torch.device(device)
    if dev.type == "cuda" and dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    key = (str(dev), str(dtype), a.shape, a.dtype.str, a.tobytes())
    hit = _CONSTANTS.get(key)
    if hit is not None:
        _CONSTANTS.move_to_end(key)
        return hit
    t = torch.from_numpy(a.copy()).to(device=dev, dtype=dtype)
    _CONSTANTS[key] = t
    if len(_CONSTANTS) > _CONSTANTS_MAX:
        _CONSTANTS.popitem(last=False)
    return t

class RasterizeCudaContext:
    """Per-device rasterisation state: the scratch workspace and its sizing.

    Mirrors ``dr.RasterizeCudaContext(device=None)``.  The workspace holds the
    primitive records and tile lists of the binning rasteriser; it is a torch
    allocation that only grows.  The tile-list capacity is sized exactly on the
    first call (one host sync) and afterwards grown from a stats block read
    back asynchronously; an undersized call is still exact (overflowing tiles
    scan all primitives of their view).

    ``tile_log2`` (3/4/5: 8/16/32-pixel tiles) and ``threads_per_tri`` (0 =
    pixel-parallel tiles, else a power of two <= 32 threads per primitive) are
    the fine-raster tuning knobs (see ``diffrp_gb300.autotune``).  ``validate``
    makes every rasterisation synchronise and raise on out-of-range indices.
    """

    def __init__(self, device=None, tile_log2=4, threads_per_tri=0, validate=False):
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        else:
            device = torch.device(device)
            if device.index is None:
                device = torch.device("cuda", torch.cuda.current_device())
        if device.type != "cuda":
            raise RuntimeError("RasterizeCudaContext requires a CUDA device")
        _ffi.load()
        self.device = device
        self.tile_log2 = int(tile_log2)
        self.threads_per_tri = int(threads_per_tri)
        self.validate = bool(validate)
        self._ws = None
        self._retired = []  # replaced buffers, kept alive for CUDA graphs captured on them
        self._capacity = 0
        self._sized = False
        self._pending = []  # (event, pinned stats copy, call shape, bin depth) not read back yet
        self._calls = 0
        self._depth = {}  # call shape (views, triangles, H, W, tile) -> fixed-depth bin size
        self._pinned_free = []
        self._topo_ws = None
        self.last_list_entries = 0
        self.last_max_tile = 0

    # -- workspace management ------------------------------------------------
    def _workspace(self, nbytes):
        if self._ws is None or self._ws.numel() < nbytes:
            n = max(nbytes, int((self._ws.numel() if self._ws is not None else 0) * 1.25))
            if self._ws is not None:
                self._retired.append(self._ws)  # a captured CUDA graph may still use it
            self._ws = torch.empty(n, dtype=torch.uint8, device=self.device)
        return self._ws

    def _choose_depth(self, shape, max_tile, needed):
        """Fixed-depth bins for a call shape, while they stay near the exact
        lists' size (else 0: keep exact lists)."""
        B, _, H, W, tl = shape
        tiles = B * ((W + (1 << tl) - 1) >> tl) * ((H + (1 << tl) - 1) >> tl)
        depth = int(max_tile * 1.25) + 8
        return depth if tiles * depth <= 2 * needed + (4 << 20) else 0

    def _note_stats(self, shape, depth, needed, err, max_tile):
        if depth == 0:
            self.last_list_entries = needed
            if needed > self._capacity:
                self._capacity = int(needed * 1.25) + 1024
            if shape not in self._depth:
                self._depth[shape] = self._choose_depth(shape, max_tile, needed)
        elif err & 2:  # a bin overflowed (still exact, but slow): deeper bins next time
            self._depth[shape] = max(int(depth * 1.5), int(max_tile * 1.25) + 8)

    def _poll_stats(self):
        """Grow the list capacity / bin depth from every finished call's
        stats (a call that needed more than it had was still exact, through
        the slow per-tile scan; the next calls get room)."""
        keep = []
        for ev, pinned, shape, depth in self._pending:
            if ev.query():
                w = pinned.view(torch.int32)
                self._note_stats(shape, depth, int(pinned[0]), int(w[2]), int(w[3]))
                self._pinned_free.append(pinned)
            else:
                keep.append((ev, pinned, shape, depth))
        self._pending = keep

    def _read_stats_sync(self):
        torch.cuda.current_stream(self.device).synchronize()
        st = self._ws[:16].view(torch.int64).cpu()
        needed = int(st[0].item())
        err = int(st[1].item()) & 0xffffffff
        self.last_max_tile = int(st[1].item()) >> 32
        return needed, err

    def _queue_stats(self, shape, depth):
        if _capturing():
            return
        pinned = self._pinned_free.pop() if self._pinned_free else torch.empty(2, dtype=torch.int64,
                                                                               pin_memory=True)
        pinned.copy_(self._ws[:16].view(torch.int64), non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.device))
        self._pending.append((ev, pinned, shape, depth))
        if len(self._pending) > 64:  # bound the queue: wait for the oldest read-back
            self._pending[0][0].synchronize()
            self._poll_stats()

    def ensure_capacity(self, entries):
        """Pre-size the tile-list capacity (used by graph capture paths)."""
        self._capacity = max(self._capacity, int(entries))
        self._sized = True

    def _raster_call(self, pos, tri, ranges_dev, B, max_view_tris, H, W, stride, prev_key, rast, db, out_key):
        if not _capturing():
            self._poll_stats()
        cap = self._capacity
        first = not self._sized
        if first:
            cap = max(cap, 4 * B * max_view_tris + 4096)
        tl = self.tile_log2
        shape = (B, max_view_tris, H, W, tl)
        # fixed-depth bins (one setup pass) once this call shape has been seen
        # with exact lists; validate mode always uses exact lists
        depth = 0 if (first or self.validate) else self._depth.get(shape, 0)
        if depth:
            tiles = B * ((W + (1 << tl) - 1) >> tl) * ((H + (1 << tl) - 1) >> tl)
            cap = max(cap, tiles * depth)
        nbytes = _ffi.size_out("drp_raster_workspace_size", B, max_view_tris, H, W, tl, cap)
        ws = self._workspace(nbytes)
        args = (pos.data_ptr(), stride, pos.shape[-2], tri.data_ptr(), tri.shape[0], B, _ptr(ranges_dev),
                max_view_tris, H, W, tl, self.threads_per_tri, cap, depth, _ptr(prev_key), rast.data_ptr(),
                _ptr(db), _ptr(out_key), _stream(self.device))
        _ffi.call("drp_rasterize_fwd", ws.data_ptr(), ws.numel(), *args)
        if first or self.validate:
            needed, err = self._read_stats_sync()
            self.last_list_entries = needed
            if err & 1:
                raise RuntimeError("rasterize: triangle vertex index out of range")
            if needed > cap:
                self._capacity = int(needed * 1.25) + 1024
                nbytes = _ffi.size_out("drp_raster_workspace_size", B, max_view_tris, H, W, tl, self._capacity)
                ws = self._workspace(nbytes)
                _ffi.call("drp_rasterize_fwd", ws.data_ptr(), ws.numel(), *args[:12], self._capacity,
                          *args[13:])
            else:
                self._capacity = max(self._capacity, cap)
            if shape not in self._depth:
                self._depth[shape] = self._choose_depth(shape, self.last_max_tile, needed)
            self._sized = True
        else:
            # read the stats back on the first calls of a shape, then on
            # every 8th call (an overflowing call is still exact; only the
            # growth waits)
            self._calls += 1
            if shape not in self._depth or self._calls <= 8 or self._calls % 8 == 0:
                self._queue_stats(shape, depth)

    def topology_workspace(self, F):
        nbytes = _ffi.size_out("drp_topology_workspace_size", F)
        if self._topo_ws is None or self._topo_ws.numel() < nbytes:
            if self._topo_ws is not None:
                self._retired.append(self._topo_ws)
            self._topo_ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        return self._topo_ws


class RasterizeGLContext:
    """OpenGL rasteriser context: unavailable (no graphics stack on this target)."""

    def __init__(self, *args, **kwargs):
        raise RuntimeError("RasterizeGLContext is not available: diffrp_gb300 rasterises with CUDA kernels only; "
                           "use RasterizeCudaContext")


# ---------------------------------------------------------------------------
# Rasterize
# ---------------------------------------------------------------------------
def _raster_setup(glctx, pos, tri, resolution, ranges):
    if not isinstance(glctx, RasterizeCudaContext):
        raise TypeError("glctx must be a RasterizeCudaContext")
    _check_tensor("pos", pos, torch.float32, (2, 3), last=4)
    _check_tensor("tri", tri, torch.int32, (2,), device=pos.device, last=3)
    if pos.device != glctx.device:
        raise RuntimeError("pos is on %s but the context is on %s" % (pos.device, glctx.device))
    if not (isinstance(resolution, (tuple, list)) and len(resolution) == 2):
        raise ValueError("resolution must be a (height, width) pair")
    H, W = int(resolution[0]), int(resolution[1])
    if not (0 < H <= 16384 and 0 < W <= 16384):
        raise ValueError("resolution %dx%d out of range (1..16384)" % (H, W))
    F = tri.shape[0]
    if pos.dim() == 3:
        if ranges is not None:
            raise ValueError("ranges must be None when pos is a batch (instanced mode)")
        B = pos.shape[0]
        stride = pos.shape[1] * 4
        ranges_dev = None
        max_view_tris = F
    else:
        stride = 0
        if ranges is None:
            B = 1
            ranges_dev = None
            max_view_tris = F
        else:
            if not isinstance(ranges, torch.Tensor) or ranges.dtype != torch.int32 or ranges.dim() != 2 or \
                    ranges.shape[1] != 2:
                raise ValueError("ranges must be an int32 tensor of shape [minibatch, 2]")
            if ranges.is_cuda:
                raise ValueError("ranges must reside in CPU memory")
            r = ranges.numpy()
            if (r < 0).any() or (r[:, 0] + r[:, 1] > F).any():
                raise ValueError("ranges out of bounds for %d triangles" % F)
            B = r.shape[0]
            max_view_tris = int(r[:, 1].max()) if B else 0
            ranges_dev = _device_constant(r, torch.int32, pos.device)
    return pos.contiguous(), tri.contiguous(), H, W, B, stride, ranges_dev, max_view_tris


class _RasterizeFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, tri, glctx, H, W, B, stride, ranges_dev, max_view_tris, grad_db, prev_key, want_key):
        dev = pos.device
        rast = torch.empty((B, H, W, 4), dtype=torch.float32, device=dev)
        db = torch.empty((B, H, W, 4), dtype=torch.float32, device=dev) if grad_db else \
            torch.empty((B, H, W, 0), dtype=torch.float32, device=dev)
        key = torch.empty((B, H, W), dtype=torch.int64, device=dev) if want_key else None
        glctx._raster_call(pos, tri, ranges_dev, B, max_view_tris, H, W, stride, prev_key, rast,
                           db if grad_db else None, key)
        ctx.save_for_backward(pos, tri, rast)
        ctx.meta = (B, H, W, stride, grad_db)
        ctx.mark_non_differentiable(*([key] if key is not None else []))
        ctx.set_materialize_grads(False)
        return rast, db, key

    @staticmethod
    def backward(ctx, grad_rast, grad_db, grad_key):
        pos, tri, rast = ctx.saved_tensors
        B, H, W, stride, has_db = ctx.meta
        if grad_rast is None and (grad_db is None or not has_db):
            return (None,) * 12
        if grad_rast is None:
            grad_rast = torch.zeros_like(rast)
        grad_rast = grad_rast.contiguous()
        gdb = grad_db.contiguous() if (has_db and grad_db is not None) else None
        grad_pos = torch.zeros_like(pos)
        _ffi.call("drp_rasterize_bwd", pos.data_ptr(), stride, pos.shape[-2], tri.data_ptr(), tri.shape[0], B, H, W,
                  rast.data_ptr(), grad_rast.data_ptr(), _ptr(gdb), grad_pos.data_ptr(), _stream(pos.device))
        return (grad_pos,) + (None,) * 11


def rasterize(glctx, pos, tri, resolution, ranges=None, grad_db=True):
    """Rasterise triangles; returns ``(rast, rast_db)``.

    ``rast`` (B, H, W, 4) holds (u, v, z/w, triangle_id + 1) per pixel, zero
    where nothing is covered; ``rast_db`` (B, H, W, 4) holds
    (du/dX, du/dY, dv/dX, dv/dY) when ``grad_db`` else has 0 channels.
    """
    pos_c, tri_c, H, W, B, stride, ranges_dev, mvt = _raster_setup(glctx, pos, tri, resolution, ranges)
    rast, db, _ = _RasterizeFn.apply(pos_c, tri_c, glctx, H, W, B, stride, ranges_dev, mvt, bool(grad_db), None,
                                     False)
    return rast, db


class DepthPeeler:
    """Depth peeling: successive ``rasterize_next_layer()`` calls return the
    nearest, second-nearest, ... surface per pixel.  Use as a context manager
    (``with DepthPeeler(ctx, pos, tri, (h, w), ranges) as dp:``).  Layers are
    ordered by the (z/w, triangle id) visibility key, so coplanar surfaces
    are peeled one at a time in triangle order."""

    def __init__(self, glctx, pos, tri, resolution, ranges=None, grad_db=True):
        self._setup = _raster_setup(glctx, pos, tri, resolution, ranges)
        self.glctx = glctx
        self.grad_db = bool(grad_db)
        self._prev_key = None
        self._active = False

    def __enter__(self):
        if self._active:
            raise RuntimeError("DepthPeeler is already active")
        self._active = True
        self._prev_key = None
        return self

    def __exit__(self, *args):
        self._active = False
        self._prev_key = None
        return False

    def rasterize_next_layer(self):
        if not self._active:
            raise RuntimeError("DepthPeeler must be used as a context manager")
        pos_c, tri_c, H, W, B, stride, ranges_dev, mvt = self._setup
        rast, db, key = _RasterizeFn.apply(pos_c, tri_c, self.glctx, H, W, B, stride, ranges_dev, mvt, self.grad_db,
                                           self._prev_key, True)
        self._prev_key = key
        return rast, db


# ---------------------------------------------------------------------------
# Interpolate
# ---------------------------------------------------------------------------
def _diff_indices(diff_attrs, C, device):
    if diff_attrs is None:
        return None
    if isinstance(diff_attrs, str):
        if diff_attrs != "all":
            raise ValueError("diff_attrs must be 'all' or a list of attribute indices")
        idx = list(range(C))
    else:
        idx = [int(i) for i in diff_attrs]
        for i in idx:
            if not 0 <= i < C:
                raise ValueError("diff_attrs index %d out of range for %d attributes" % (i, C))
    if not idx:
        return None
    return _device_constant(np.asarray(idx, np.int32), torch.int32, device)


class _InterpolateFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, attr, rast, tri, rast_db, diff_idx):
        B, H, W = rast.shape[:3]
        C = attr.shape[-1]
        stride = attr.shape[1] * C if attr.dim() == 3 else 0
        nd = 0 if diff_idx is None else diff_idx.numel()
        out = torch.empty((B, H, W, C), dtype=torch.float32, device=attr.device)
        da = torch.empty((B, H, W, 2 * nd), dtype=torch.float32, device=attr.device)
        _ffi.call("drp_interpolate_fwd", attr.data_ptr(), stride, attr.shape[-2], C, rast.data_ptr(), _ptr(rast_db),
                  tri.data_ptr(), tri.shape[0], B, H, W, _ptr(diff_idx), nd, out.data_ptr(),
                  da.data_ptr() if nd else None, _stream(attr.device))
        ctx.save_for_backward(attr, rast, tri, rast_db, diff_idx)
        ctx.meta = (B, H, W, C, stride, nd)
        ctx.set_materialize_grads(False)
        return out, da

    @staticmethod
    def backward(ctx, grad_out, grad_da):
        attr, rast, tri, rast_db, diff_idx = ctx.saved_tensors
        B, H, W, C, stride, nd = ctx.meta
        if grad_out is None and (grad_da is None or nd == 0):
            return None, None, None, None, None
        if grad_out is None:
            grad_out = torch.zeros((B, H, W, C), dtype=torch.float32, device=attr.device)
        grad_out = grad_out.contiguous()
        gda = grad_da.contiguous() if (nd and grad_da is not None) else None
        grad_attr = torch.zeros_like(attr)
        grad_rast = torch.empty_like(rast)
        grad_db = torch.empty_like(rast_db) if (rast_db is not None and gda is not None) else None
        _ffi.call("drp_interpolate_bwd", attr.data_ptr(), stride, attr.shape[-2], C, rast.data_ptr(),
                  _ptr(rast_db), tri.data_ptr(), tri.shape[0], B, H, W, _ptr(diff_idx), nd if gda is not None else 0,
                  grad_out.data_ptr(), _ptr(gda), grad_attr.data_ptr(), grad_rast.data_ptr(), _ptr(grad_db),
                  _stream(attr.device))
        return grad_attr, grad_rast, None, grad_db, None


def interpolate(attr, rast, tri, rast_db=None, diff_attrs=None):
    """Interpolate vertex attributes; returns ``(out, da)``.

    ``attr`` (V, C) or (B, V, C); ``out`` (B, H, W, C) with zeros where
    ``rast`` is empty.  With ``diff_attrs`` ('all' or indices) and
    ``rast_db``, ``da`` (B, H, W, 2 * n) holds (dA/dX, dA/dY) per listed
    attribute; otherwise ``da`` has 0 channels.
    """
    _check_tensor("attr", attr, torch.float32, (2, 3))
    _check_tensor("rast", rast, torch.float32, (4,), device=attr.device, last=4)
    _check_tensor("tri", tri, torch.int32, (2,), device=attr.device, last=3)
    if attr.dim() == 3 and attr.shape[0] != rast.shape[0]:
        raise RuntimeError("attr minibatch %d does not match rast minibatch %d" % (attr.shape[0], rast.shape[0]))
    diff_idx = _diff_indices(diff_attrs, attr.shape[-1], attr.device)
    if diff_idx is not None:
        if rast_db is None or rast_db.shape[-1] != 4:
            raise RuntimeError("diff_attrs requires rast_db with 4 channels")
        _check_tensor("rast_db", rast_db, torch.float32, (4,), device=attr.device, last=4)
        rast_db = rast_db.contiguous()
    else:
        rast_db = None
    return _InterpolateFn.apply(attr.contiguous(), rast.contiguous(), tri.contiguous(), rast_db, diff_idx)


# ---------------------------------------------------------------------------
# Antialias
# ---------------------------------------------------------------------------
class _Scratch(threading.local):
    """Per-thread, per-device scratch buffers for the context-free ops
    (topology construction and antialiasing)."""

    def __init__(self):
        self.buffers = {}
        self.retired = []  # replaced buffers, kept alive for CUDA graphs captured on them

    def get(self, device, name, nbytes):
        key = (device.index, name)
        buf = self.buffers.get(key)
        if buf is None or buf.numel() < nbytes:
            if buf is not None:
                self.retired.append(buf)
            buf = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=device)
            self.buffers[key] = buf
        return buf


_scratch = _Scratch()


def antialias_construct_topology_hash(tri):
    """Edge topology of ``tri``: (F, 3) int32 table holding, for each edge
    (edge k joins vertices k+1 and k+2), the vertex of the neighbouring
    triangle opposite that edge, -1 where no single neighbour exists.  Pass it
    as ``topology_hash`` to :func:`antialias` to avoid rebuilding it every
    call."""
    _check_tensor("tri", tri, torch.int32, (2,), last=3)
    tri = tri.contiguous()
    F = tri.shape[0]
    nbr = torch.empty((F, 3), dtype=torch.int32, device=tri.device)
    if F:
        ws = _scratch.get(tri.device, "topology", _ffi.size_out("drp_topology_workspace_size", F))
        _ffi.call("drp_antialias_topology", ws.data_ptr(), ws.numel(), tri.data_ptr(), F, nbr.data_ptr(),
                  _stream(tri.device))
    return nbr


class _AntialiasFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, color, rast, pos, tri, nbr, boost):
        B, H, W, C = color.shape
        stride = pos.shape[1] * 4 if pos.dim() == 3 else 0
        out = torch.empty_like(color)
        ws = _scratch.get(color.device, "antialias", _ffi.size_out("drp_antialias_workspace_size", B, tri.shape[0]))
        # the list of pixels a blending pair touches, for the backward
        state = torch.empty(_ffi.size_out("drp_antialias_state_size", B, H, W), dtype=torch.uint8,
                            device=color.device)
        _ffi.call("drp_antialias_fwd", ws.data_ptr(), ws.numel(), color.data_ptr(), C, rast.data_ptr(),
                  pos.data_ptr(), stride, pos.shape[-2], tri.data_ptr(), tri.shape[0], nbr.data_ptr(), B, H, W,
                  out.data_ptr(), state.data_ptr(), _stream(color.device))
        ctx.save_for_backward(color, rast, pos, tri, nbr, state)
        ctx.meta = (B, H, W, C, stride, boost)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        color, rast, pos, tri, nbr, state = ctx.saved_tensors
        B, H, W, C, stride, boost = ctx.meta
        grad_out = grad_out.contiguous()
        grad_color = torch.empty_like(color)
        need_pos = ctx.needs_input_grad[2]
        grad_pos = torch.zeros_like(pos) if need_pos else None
        ws = _scratch.get(color.device, "antialias", _ffi.size_out("drp_antialias_workspace_size", B, tri.shape[0]))
        _ffi.call("drp_antialias_bwd", ws.data_ptr(), ws.numel(), color.data_ptr(), C, rast.data_ptr(),
                  pos.data_ptr(), stride, pos.shape[-2], tri.data_ptr(), tri.shape[0], nbr.data_ptr(), B, H, W,
                  grad_out.data_ptr(), float(boost), grad_color.data_ptr(), _ptr(grad_pos), state.data_ptr(),
                  _stream(color.device))
        return grad_color, None, grad_pos, None, None, None


def antialias(color, rast, pos, tri, topology_hash=None, pos_gradient_boost=1.0):
    """Analytic silhouette antialiasing; returns the antialiased ``color``.

    ``color`` (B, H, W, C), ``rast`` from :func:`rasterize` on the same
    ``pos`` / ``tri``.  Gradients flow to ``color`` and, through silhouette
    edge positions, to ``pos`` (scaled by ``pos_gradient_boost``).
    """
    _check_tensor("color", color, torch.float32, (4,))
    _check_tensor("rast", rast, torch.float32, (4,), device=color.device, last=4)
    _check_tensor("pos", pos, torch.float32, (2, 3), device=color.device, last=4)
    _check_tensor("tri", tri, torch.int32, (2,), device=color.device, last=3)
    if rast.shape[:3] != color.shape[:3]:
        raise RuntimeError("color %s and rast %s must agree in (B, H, W)" % (tuple(color.shape), tuple(rast.shape)))
    if pos.dim() == 3 and pos.shape[0] != color.shape[0]:
        raise RuntimeError("pos minibatch must match color minibatch")
    if not isinstance(pos_gradient_boost, numbers.Real):
        raise TypeError("pos_gradient_boost must be a real number")
    tri = tri.contiguous()
    if topology_hash is None:
        topology_hash = antialias_construct_topology_hash(tri)
    elif not (isinstance(topology_hash, torch.Tensor) and topology_hash.dtype == torch.int32 and
              tuple(topology_hash.shape) == (tri.shape[0], 3)):
        raise RuntimeError("topology_hash must come from antialias_construct_topology_hash(tri)")
    return _AntialiasFn.apply(color.contiguous(), rast.contiguous(), pos.contiguous(), tri, topology_hash,
                              float(pos_gradient_boost))


# ---------------------------------------------------------------------------
# Texture sampling
# ---------------------------------------------------------------------------
_TEX_FILTERS = {"nearest": 0, "linear": 1, "linear-mipmap-nearest": 2, "linear-mipmap-linear": 3}
# 'mirror' (mirrored repeat) is an addition to nvdiffrast's modes: diffrp's
# sample2d 'reflection' padding and glTF's MIRRORED_REPEAT
_TEX_BOUNDARIES = {"wrap": 0, "clamp": 1, "zero": 2, "mirror": 3}


def _tex_levels(H, W, max_mip_level):
    n = ctypes.c_int(0)
    _ffi.call("drp_texture_levels", H, W, -1 if max_mip_level is None else int(max_mip_level), ctypes.byref(n))
    return n.value


def _tex_pyramid_floats(N, H, W, C, levels):
    n = ctypes.c_longlong(0)
    _ffi.call("drp_texture_pyramid_floats", N, H, W, C, levels, ctypes.byref(n))
    return n.value


def _tex_build(tex, levels):
    N, H, W, C = tex.shape
    pyr = torch.empty(max(1, _tex_pyramid_floats(N, H, W, C, levels)), dtype=torch.float32, device=tex.device)
    if levels > 1:
        _ffi.call("drp_texture_mip_build", tex.data_ptr(), N, H, W, C, levels, pyr.data_ptr(), _stream(tex.device))
    return pyr


class TextureMip:
    """A pre-built mip pyramid (texture_construct_mip): levels 1 and up of
    ``tex``, reused by texture(..., mip=...) instead of being rebuilt."""

    def __init__(self, tex, levels, pyr):
        self.tex, self.levels, self.pyr = tex, levels, pyr


def texture_construct_mip(tex, max_mip_level=None, cube_mode=False):
    """Build the mip pyramid of ``tex`` (N, H, W, C) once, for texture calls
    that sample the same texture again (2x2 box average per level)."""
    if cube_mode:
        raise NotImplementedError("cube map textures are not supported")
    _check_tensor("tex", tex, torch.float32, (4,))
    tex = tex.contiguous()
    levels = _tex_levels(tex.shape[1], tex.shape[2], max_mip_level)
    with torch.no_grad():
        return TextureMip(tex, levels, _tex_build(tex.detach(), levels))


class _TextureFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, tex, uv, uv_da, bias, pyr, levels, filt, bnd):
        Nt, H, W, C = tex.shape
        N, h, w = uv.shape[:3]
        if pyr is None:
            pyr = _tex_build(tex, levels)
        out = torch.empty((N, h, w, C), dtype=torch.float32, device=tex.device)
        _ffi.call("drp_texture_fwd", tex.data_ptr(), pyr.data_ptr(), Nt, H, W, C, levels, uv.data_ptr(),
                  _ptr(uv_da), _ptr(bias), N, h, w, filt, bnd, out.data_ptr(), _stream(tex.device))
        ctx.save_for_backward(tex, uv, uv_da, bias, pyr)
        ctx.meta = (levels, filt, bnd)
        ctx.set_materialize_grads(False)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        tex, uv, uv_da, bias, pyr = ctx.saved_tensors
        levels, filt, bnd = ctx.meta
        if grad_out is None:
            return None, None, None, None, None, None, None, None
        Nt, H, W, C = tex.shape
        N, h, w = uv.shape[:3]
        grad_out = grad_out.contiguous()
        grad_tex = torch.zeros_like(tex)
        grad_pyr = torch.empty_like(pyr)
        grad_uv = torch.empty_like(uv)
        want_da = uv_da is not None and ctx.needs_input_grad[2]
        grad_da = torch.empty_like(uv_da) if want_da else None
        want_bias = bias is not None and ctx.needs_input_grad[3]
        grad_bias = torch.empty_like(bias) if want_bias else None
        _ffi.call("drp_texture_bwd", tex.data_ptr(), pyr.data_ptr(), Nt, H, W, C, levels, uv.data_ptr(),
                  _ptr(uv_da), _ptr(bias), N, h, w, filt, bnd, grad_out.data_ptr(), grad_tex.data_ptr(),
                  grad_pyr.data_ptr(), grad_uv.data_ptr(), _ptr(grad_da), _ptr(grad_bias), _stream(tex.device))
        return (grad_tex if ctx.needs_input_grad[0] else None, grad_uv if ctx.needs_input_grad[1] else None,
                grad_da, grad_bias, None, None, None, None)


def texture(tex, uv, uv_da=None, mip_level_bias=None, mip=None, filter_mode="auto", boundary_mode="wrap",
            max_mip_level=None):
    """Sample ``tex`` (N or 1, H, W, C) at ``uv`` (N, h, w, 2); returns (N, h, w, C).

    Texel (x, y) is centred at ((x + 0.5) / W, (y + 0.5) / H).  filter_mode
    'nearest', 'linear', 'linear-mipmap-nearest', 'linear-mipmap-linear' or
    'auto' (trilinear with ``uv_da`` or ``mip_level_bias``, else bilinear);
    the mip-mapped modes choose the level from ``uv_da`` (N, h, w, 4) =
    (du/dX, du/dY, dv/dX, dv/dY), e.g. interpolate(..., diff_attrs=...)'s
    derivatives of uv, plus ``mip_level_bias`` (N, h, w) when given (alone,
    it sets the level).  boundary_mode 'wrap', 'clamp', 'zero' or 'mirror'
    (mirrored repeat).  ``mip`` reuses a texture_construct_mip pyramid of
    ``tex``.  Gradients reach ``tex`` (through the pyramid), ``uv``, and
    ``uv_da`` and ``mip_level_bias`` (trilinear, where the level of detail is
    not clamped).  Not supported: cube maps.
    """
    if boundary_mode not in _TEX_BOUNDARIES:
        if boundary_mode == "cube":
            raise NotImplementedError("cube map textures are not supported")
        raise ValueError("boundary_mode must be one of %s" % sorted(_TEX_BOUNDARIES))
    if filter_mode == "auto":
        filter_mode = "linear-mipmap-linear" if uv_da is not None or mip_level_bias is not None else "linear"
    if filter_mode not in _TEX_FILTERS:
        raise ValueError("filter_mode must be 'auto' or one of %s" % sorted(_TEX_FILTERS))
    mipmapped = filter_mode.startswith("linear-mipmap")
    if mipmapped and uv_da is None and mip_level_bias is None:
        raise ValueError("filter_mode %r needs uv_da or mip_level_bias" % filter_mode)
    _check_tensor("tex", tex, torch.float32, (4,))
    _check_tensor("uv", uv, torch.float32, (4,), device=tex.device, last=2)
    if tex.shape[0] not in (1, uv.shape[0]):
        raise RuntimeError("tex minibatch %d must be 1 or the uv minibatch %d" % (tex.shape[0], uv.shape[0]))
    if uv_da is not None:
        _check_tensor("uv_da", uv_da, torch.float32, (4,), device=tex.device, last=4)
        if tuple(uv_da.shape[:3]) != tuple(uv.shape[:3]):
            raise RuntimeError("uv_da must have the shape of uv with 4 channels")
        uv_da = uv_da.contiguous() if mipmapped else None
    if mip_level_bias is not None:
        _check_tensor("mip_level_bias", mip_level_bias, torch.float32, (3,), device=tex.device)
        if tuple(mip_level_bias.shape) != tuple(uv.shape[:3]):
            raise RuntimeError("mip_level_bias must have the shape of uv without its last dimension")
        mip_level_bias = mip_level_bias.contiguous() if mipmapped else None
    tex = tex.contiguous()
    pyr = None
    if mipmapped:
        levels = _tex_levels(tex.shape[1], tex.shape[2], max_mip_level)
        if mip is not None:
            if not isinstance(mip, TextureMip) or tuple(mip.tex.shape) != tuple(tex.shape) or mip.levels != levels:
                raise RuntimeError("mip was not built from this texture with this max_mip_level")
            pyr = mip.pyr
    else:
        levels = 1
    return _TextureFn.apply(tex, uv.contiguous(), uv_da, mip_level_bias, pyr, levels, _TEX_FILTERS[filter_mode],
                            _TEX_BOUNDARIES[boundary_mode])
