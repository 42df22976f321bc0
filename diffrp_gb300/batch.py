"""Batching form: many meshes x views x resolutions in one set of launches.

``BatchRenderer`` renders a fixed set of items -- (mesh, view, resolution)
triples -- through rasterize -> interpolate -> antialias in one launch
sequence per forward (persistent fine-raster CTAs pulling (item, tile) work
from a queue, interpolation fused into the raster's shading) and one fused
backward pass.  Each item's output equals what the per-item drop-in calls
(``nvdr.rasterize``, ``nvdr.interpolate``, ``nvdr.antialias`` with the mesh's
topology) produce; the item structure (triangle counts, resolutions,
channels) is static so the whole step can be captured in a CUDA graph.

Packed layouts (see ``drp_batch_item`` in include/diffrp_gb300.h):
  positions   (sum over items of the mesh's V, 4) clip-space rows, item order;
  attributes  (sum over meshes of V * C,) floats, mesh order;
  images      (sum over items of H * W * C,) floats, item order.
``recompute=True`` keeps no per-pixel buffer between forward and backward
except the returned images: items are rendered in chunks of about
``chunk_pixels`` pixels through one scratch set and one workspace sized for
the largest chunk, and the backward re-runs each chunk's forward (raster,
interpolation, antialias pass with its pixel list and, for the fused loss,
the sign gradient) into that scratch before the chunk's backward.  Peak
memory is then the images (and the target), plus one chunk's buffers.
"""
import ctypes

import numpy as np
import torch

from . import _ffi
from . import nvdr

__all__ = ["BatchRenderer"]

REUSE_AA_RECORDS = 1  # DRP_BATCH_REUSE_AA_RECORDS


class _Item(ctypes.Structure):
    _fields_ = [("pos_offset", ctypes.c_longlong), ("attr_offset", ctypes.c_longlong),
                ("tri_first", ctypes.c_int), ("tri_count", ctypes.c_int), ("num_vertices", ctypes.c_int),
                ("height", ctypes.c_int), ("width", ctypes.c_int), ("channels", ctypes.c_int),
                ("tiles_x", ctypes.c_int), ("tiles_y", ctypes.c_int),
                ("prim_offset", ctypes.c_longlong), ("tile_offset", ctypes.c_longlong),
                ("pixel_offset", ctypes.c_longlong), ("image_offset", ctypes.c_longlong)]


assert ctypes.sizeof(_Item) == 80


def _register():
    lib = _ffi.load()
    P, LL, I, ULL = ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int, ctypes.c_ulonglong
    sigs = {
        "drp_batch_plan": [P, I, I, P],
        "drp_batch_block_maps": [P, I, P, P],
        "drp_batch_workspace_size": [LL, LL, ULL, ctypes.POINTER(ctypes.c_size_t)],
        "drp_batch_aa_state_size": [LL, ctypes.POINTER(ctypes.c_size_t)],
        "drp_batch_forward": [P, ctypes.c_size_t, P, I, P, LL, P, LL, LL, LL, P, P, P, P, I, I, ULL, ctypes.c_uint,
                              P, P, P, P, LL, P],
        "drp_batch_forward_l1": [P, ctypes.c_size_t, P, I, P, LL, P, LL, LL, LL, P, P, P, P, I, I, ULL,
                                 ctypes.c_uint, P, P, P, P, LL, P, ctypes.c_float, P, P, P, P],
        "drp_batch_forward_l1_grad": [P, ctypes.c_size_t, P, I, P, LL, P, LL, LL, LL, P, P, P, P, I, I, ULL,
                                      ctypes.c_uint, P, P, P, P, LL, P, ctypes.c_float, P, P, P, P, P, LL, P],
        "drp_scale_floats": [P, P, LL, P, P],
        "drp_batch_backward": [P, ctypes.c_size_t, P, I, P, LL, P, LL, LL, LL, P, P, P, P, P, P, P, LL, P, P, P, P,
                               P, I, P],
    }
    for name, args in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    return lib


class _SharedWorkspace:
    """The batch workspace buffer, shared by a renderer and its recompute
    chunks (one buffer sized for the largest user).  records = (buffer,
    renderer id, forward generation) of the forward whose antialias records
    the buffer holds."""

    def __init__(self):
        self.buf = None
        self.retired = []  # replaced buffers, kept alive for CUDA graphs captured on them
        self.records = None

    def get(self, nbytes, device):
        if self.buf is None or self.buf.numel() < nbytes:
            if self.buf is not None:
                self.retired.append(self.buf)
            self.buf = torch.empty(nbytes, dtype=torch.uint8, device=device)
            self.records = None
        return self.buf


class _Chunk:
    """A contiguous run of items [i0, i1) of a recompute renderer: its own
    plan over those items (sharing the parent's triangles, topology and
    workspace) and its slices of the packed buffers."""

    def __init__(self, parent, i0, i1):
        self.i0, self.i1 = i0, i1
        self.renderer = BatchRenderer(parent.meshes, parent.items[i0:i1], device=parent.device,
                                      tile_log2=parent.tile_log2, threads_per_tri=parent.threads_per_tri,
                                      bin_depth=parent.bin_depth_mode,
                                      _shared=(parent.tri, parent.nbr, parent._wsh))
        it = parent.item_table
        self.rows = slice(parent.pos_offsets[i0], parent.pos_offsets[i0] + self.renderer.pos_rows)
        self.pixels = slice(it[i0].pixel_offset, it[i0].pixel_offset + self.renderer.total_pixels)
        self.floats = slice(it[i0].image_offset, it[i0].image_offset + self.renderer.image_floats)


class BatchRenderer:
    """Render many (mesh, view, resolution) items per launch.

    meshes: list of (tri (F, 3) int32 CUDA tensor, num_vertices, channels).
    items:  list of (mesh index, (height, width)).
    tile_log2 / threads_per_tri: fine-raster shape (see nvdr.RasterizeCudaContext).
    bin_depth: None sizes fixed-depth tile bins from the first forward's
    largest tile (one setup pass per forward afterwards); 0 keeps exact tile
    lists (count, scan and fill passes); n > 0 fixes the depth.
    recompute: keep no per-pixel buffer for the backward but the returned
    images; render in chunks of consecutive items of about chunk_pixels
    pixels (at least one item each) and recompute each chunk's forward in
    the backward.
    """

    def __init__(self, meshes, items, device=None, tile_log2=4, threads_per_tri=0, recompute=False, bin_depth=None,
                 chunk_pixels=1 << 23, _shared=None):
        _register()
        self.bin_depth_mode = bin_depth
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.tile_log2 = int(tile_log2)
        self.threads_per_tri = int(threads_per_tri)
        self.recompute = bool(recompute)
        self.meshes = meshes
        if _shared is None:
            tri_parts, nbr_parts = [], []
            for tri, V, C in meshes:
                tri = tri.to(self.device, torch.int32).contiguous()
                tri_parts.append(tri)
                nbr_parts.append(nvdr.antialias_construct_topology_hash(tri))
            self.tri = torch.cat(tri_parts).contiguous()
            self.nbr = torch.cat(nbr_parts).contiguous()
            self._wsh = _SharedWorkspace()
        else:
            self.tri, self.nbr, self._wsh = _shared
        tri_first, attr_off = [], []
        f0 = a0 = 0
        for tri, V, C in meshes:
            tri_first.append(f0)
            attr_off.append(a0)
            f0 += int(tri.shape[0])
            a0 += int(V) * int(C)
        self.attr_floats = a0
        self.attr_offsets = attr_off
        self._item_specs = []
        p0 = 0
        self.pos_offsets = []
        for m, (H, W) in items:
            tri, V, C = meshes[m]
            self._item_specs.append((p0, attr_off[m], tri_first[m], int(tri.shape[0]), int(V), int(H), int(W),
                                     int(C)))
            self.pos_offsets.append(p0)
            p0 += int(V)
        self.pos_rows = p0
        self.items = items
        self._fwd_gen = 0  # bumped by every forward; the workspace's AA records belong to the latest
        self._plan()
        self._chunks = None
        if self.recompute:
            self._make_chunks(int(chunk_pixels))

    def _plan(self):
        """(Re)build the item table and block maps for the current tile size."""
        arr = (_Item * len(self.items))()
        for i, (po, ao, tf, tc, V, H, W, C) in enumerate(self._item_specs):
            arr[i].pos_offset = po
            arr[i].attr_offset = ao
            arr[i].tri_first = tf
            arr[i].tri_count = tc
            arr[i].num_vertices = V
            arr[i].height = H
            arr[i].width = W
            arr[i].channels = C
        totals = (ctypes.c_longlong * 6)()
        _ffi.call("drp_batch_plan", ctypes.addressof(arr), len(self.items), self.tile_log2, ctypes.addressof(totals))
        (self.total_prims, self.total_tiles, self.total_pixels, self.image_floats, self.prim_blocks,
         self.pixel_blocks) = [int(x) for x in totals]
        pmap = (ctypes.c_int * max(2, 2 * self.prim_blocks))()
        xmap = (ctypes.c_int * max(2, 2 * self.pixel_blocks))()
        _ffi.call("drp_batch_block_maps", ctypes.addressof(arr), len(self.items), ctypes.addressof(pmap),
                  ctypes.addressof(xmap))
        self.item_table = arr
        self._items_dev = torch.from_numpy(np.frombuffer(bytes(arr), dtype=np.uint8).copy()).to(self.device)
        self._pmap = torch.from_numpy(np.frombuffer(bytes(pmap), dtype=np.int32).copy()).to(self.device)
        self._xmap = torch.from_numpy(np.frombuffer(bytes(xmap), dtype=np.int32).copy()).to(self.device)
        self._capacity = 0
        self._depth = 0
        self._pending = None
        self._pinned = None
        self.last_list_entries = 0
        self.last_max_tile = 0
        if getattr(self, "_wsh", None) is not None:
            self._wsh.records = None  # the record offsets depend on the plan

    def set_raster_shape(self, tile_log2, threads_per_tri):
        """Change the fine-raster tile size / threads per primitive (re-plans;
        call before capturing a CUDA graph)."""
        self.threads_per_tri = int(threads_per_tri)
        if int(tile_log2) != self.tile_log2:
            self.tile_log2 = int(tile_log2)
            self._plan()
        for c in self._chunks or []:
            c.renderer.set_raster_shape(tile_log2, threads_per_tri)

    def _make_chunks(self, chunk_pixels):
        bounds, i0, px = [], 0, 0
        for i, (_, (H, W)) in enumerate(self.items):
            if i > i0 and px + H * W > chunk_pixels:
                bounds.append((i0, i))
                i0, px = i, 0
            px += H * W
        bounds.append((i0, len(self.items)))
        self._chunks = [_Chunk(self, a, b) for a, b in bounds]

    def _chunk_scratch(self, l1):
        """One chunk's buffers, sized for the largest chunk: rast, colour,
        output, sign gradient (l1) and antialias state."""
        pix = max(c.renderer.total_pixels for c in self._chunks)
        flt = max(c.renderer.image_floats for c in self._chunks)
        blocks = max(c.renderer.pixel_blocks for c in self._chunks)
        rast = torch.empty((pix, 4), dtype=torch.float32, device=self.device)
        fl = torch.empty((flt + 63) // 64 * 64 * (3 if l1 else 2), dtype=torch.float32, device=self.device)
        flags = torch.empty(_ffi.size_out("drp_batch_aa_state_size", pix), dtype=torch.uint8, device=self.device)
        block_loss = torch.empty(max(1, blocks), dtype=torch.float32, device=self.device)
        return rast, fl, flags, block_loss

    # -- layout helpers ---------------------------------------------------------
    def pack_positions(self, per_item):
        """List of (V, 4) clip positions, one per item -> packed (rows, 4)."""
        return torch.cat([p.reshape(-1, 4) for p in per_item]).contiguous()

    def pack_attributes(self, per_mesh):
        """List of (V, C) attributes, one per mesh -> packed floats."""
        return torch.cat([a.reshape(-1) for a in per_mesh]).contiguous()

    def images(self, packed):
        """Packed image floats -> list of (H, W, C) views, item order."""
        out = []
        for it in self.item_table:
            n = it.height * it.width * it.channels
            out.append(packed[it.image_offset:it.image_offset + n].view(it.height, it.width, it.channels))
        return out

    def rast_views(self, rast):
        out = []
        for it in self.item_table:
            n = it.height * it.width
            out.append(rast[it.pixel_offset:it.pixel_offset + n].view(it.height, it.width, 4))
        return out

    # -- execution -------------------------------------------------------------------
    def _workspace(self, cap):
        nbytes = _ffi.size_out("drp_batch_workspace_size", self.total_prims, self.total_tiles, cap)
        return self._wsh.get(nbytes, self.device)

    def _choose_depth(self, max_tile, needed):
        if self.bin_depth_mode is not None:
            return int(self.bin_depth_mode)
        depth = int(max_tile * 1.25) + 8
        # fixed-depth bins only while they stay near the exact lists' size
        return depth if self.total_tiles * depth <= 2 * needed + (4 << 20) else 0

    def _poll_stats(self):
        """Grow the bins / list from the stats of an earlier forward whose
        lists overflowed (the overflowing tiles were still exact, but slow)."""
        if self._pending is None or not self._pending.query():
            return
        self._pending = None
        st = self._pinned.view(torch.int32)
        if int(st[2]) & 2:
            if self._depth:
                self._depth = max(int(self._depth * 1.5), int(int(st[3]) * 1.25) + 8)
            else:
                self._capacity = max(self._capacity, int(int(self._pinned.view(torch.int64)[0]) * 1.25) + 4096)

    def _queue_stats(self, ws):
        if torch.cuda.is_current_stream_capturing():
            return
        if self._pinned is None:
            self._pinned = torch.empty(16, dtype=torch.uint8, pin_memory=True)
        self._pinned.copy_(ws[:16], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.device))
        self._pending = ev

    def _forward_raw(self, pos, attr, rast, color, out, l1=None, flags=None):
        """out=None writes rast and colour only (no antialias pass).  l1 =
        (target, scale, grad, block_loss, loss) fuses the L1 loss into the
        antialias pass (drp_batch_forward_l1); l1 = (target, scale,
        block_loss, loss, grad_pos, grad_attr) also forms the loss's gradient
        there (drp_batch_forward_l1_grad, flags required; grad_attr and
        grad_pos are accumulated, after the call zeroes the buffer given
        last, when it is not None).  flags: an
        antialias state block (_flags()) the forward fills for its backward,
        or None."""
        if not torch.cuda.is_current_stream_capturing():
            self._poll_stats()
        first = not self._capacity
        depth = 0 if first else self._depth
        if depth:
            cap = self.total_tiles * depth
        else:
            cap = self._capacity if self._capacity else 4 * self.total_prims + 4096
        optr = None if out is None else out.data_ptr()
        fptr = None if flags is None else flags.data_ptr()
        npix = self.total_pixels
        self._fwd_gen += 1
        ws = self._workspace(cap)
        stream = _ffi.stream_of(self.device)
        args = (self._items_dev.data_ptr(), len(self.items), self._pmap.data_ptr(), self.prim_blocks,
                self._xmap.data_ptr(), self.pixel_blocks, self.total_prims, self.total_tiles, pos.data_ptr(),
                self.tri.data_ptr(), attr.data_ptr(), self.nbr.data_ptr(), self.tile_log2, self.threads_per_tri)
        if l1 is not None and len(l1) == 7:
            # the loss's gradient formed in the same pass: (target, scale,
            # block_loss, loss, grad_pos, grad_attr, buffer the call zeroes
            # first or None)
            target, scale, block_loss, loss, gpos, gattr, zero = l1
            tail = (target.data_ptr(), ctypes.c_float(scale), block_loss.data_ptr(), loss.data_ptr(),
                    gpos.data_ptr(), gattr.data_ptr(), None if zero is None else zero.data_ptr(),
                    0 if zero is None else zero.numel(), stream)
            entry = "drp_batch_forward_l1_grad"
        elif l1 is not None:
            target, scale, grad, block_loss, loss = l1
            tail = (target.data_ptr(), ctypes.c_float(scale), grad.data_ptr(), block_loss.data_ptr(),
                    loss.data_ptr(), stream)
            entry = "drp_batch_forward_l1"
        else:
            tail = (stream,)
            entry = "drp_batch_forward"
        _ffi.call(entry, ws.data_ptr(), ws.numel(), *args, cap, depth, rast.data_ptr(), color.data_ptr(), optr,
                  fptr, npix, *tail)
        if first:
            # exact lists, sized synchronously; they also give the largest tile
            torch.cuda.current_stream(self.device).synchronize()
            needed = int(ws[:8].view(torch.int64).cpu()[0])
            words = ws[:16].view(torch.int32).cpu()
            if int(words[2]) & 1:
                raise RuntimeError("BatchRenderer: triangle vertex index out of range")
            self.last_list_entries = needed
            self.last_max_tile = int(words[3])
            self._capacity = max(cap, int(needed * 1.25) + 4096)
            self._depth = self._choose_depth(self.last_max_tile, needed)
            if needed > cap:
                ws = self._workspace(self._capacity)
                _ffi.call(entry, ws.data_ptr(), ws.numel(), *args, self._capacity, 0, rast.data_ptr(),
                          color.data_ptr(), optr, fptr, npix, *tail)
        else:
            self._queue_stats(ws)
        if out is not None or l1 is not None:  # a raster-only forward writes no AA records
            self._wsh.records = (ws, id(self), self._fwd_gen)

    def _backward_raw(self, pos, attr, rast, color, grad_out, grad_pos, grad_attr, gen=None, grad_scale=None,
                      aa_flags=None):
        """gen: the forward generation that produced rast / colour from pos;
        when it is still the latest, its antialias records are reused.
        grad_scale: a one-element device tensor multiplying grad_out.
        aa_flags: the antialias slot bits that forward wrote, or None."""
        ws = self._workspace(0)  # the backward reads no tile list
        stream = _ffi.stream_of(self.device)
        flags = REUSE_AA_RECORDS if gen is not None and self._wsh.records == (ws, id(self), gen) else 0
        _ffi.call("drp_batch_backward", ws.data_ptr(), ws.numel(), self._items_dev.data_ptr(), len(self.items),
                  self._pmap.data_ptr(), self.prim_blocks, self._xmap.data_ptr(), self.pixel_blocks,
                  self.total_prims, self.total_tiles, pos.data_ptr(), self.tri.data_ptr(), attr.data_ptr(),
                  self.nbr.data_ptr(), rast.data_ptr(), color.data_ptr(), None if aa_flags is None else aa_flags.data_ptr(),
                  self.total_pixels, None, grad_out.data_ptr(),
                  grad_pos.data_ptr(),
                  grad_attr.data_ptr(), None if grad_scale is None else grad_scale.data_ptr(), flags, stream)

    def _buffers(self):
        rast = torch.empty((self.total_pixels, 4), dtype=torch.float32, device=self.device)
        color = torch.empty(self.image_floats, dtype=torch.float32, device=self.device)
        return rast, color

    def _flags(self):
        """The antialias state block one forward fills for its backward."""
        n = _ffi.size_out("drp_batch_aa_state_size", self.total_pixels)
        return torch.empty(n, dtype=torch.uint8, device=self.device)

    def __call__(self, pos, attr):
        """pos: packed (rows, 4) clip positions; attr: packed attribute floats.
        Returns packed antialiased images (differentiable w.r.t. both)."""
        if pos.shape != (self.pos_rows, 4) or pos.dtype != torch.float32 or not pos.is_cuda:
            raise RuntimeError("pos must be a float32 CUDA tensor of shape (%d, 4)" % self.pos_rows)
        if attr.numel() != self.attr_floats or attr.dtype != torch.float32 or not attr.is_cuda:
            raise RuntimeError("attr must hold %d float32 values on the GPU" % self.attr_floats)
        return _BatchFn.apply(pos.contiguous(), attr.contiguous().reshape(-1), self)

    def render_l1(self, pos, attr, target, grads_in_forward=False):
        """Render and score in one pass: returns (loss, images) with loss =
        mean |images - target| over all image floats (target packed like
        the images).  Differentiable w.r.t. pos and attr through both
        outputs; the loss path never materialises a per-pixel gradient
        product (the upstream loss gradient is applied inside the fused
        backward).

        grads_in_forward=True (items of at most 32 channels): the forward
        also forms d loss / d pos and d loss / d attr, in the pass that forms
        the loss (drp_batch_forward_l1_grad), so that a backward reaching only
        the loss is one multiplication by its upstream gradient -- and, with
        recompute, re-renders nothing.  A backward that also reaches the
        images runs the full backward instead (the gradients formed in the
        forward are then not used)."""
        if pos.shape != (self.pos_rows, 4) or pos.dtype != torch.float32 or not pos.is_cuda:
            raise RuntimeError("pos must be a float32 CUDA tensor of shape (%d, 4)" % self.pos_rows)
        if attr.numel() != self.attr_floats or attr.dtype != torch.float32 or not attr.is_cuda:
            raise RuntimeError("attr must hold %d float32 values on the GPU" % self.attr_floats)
        if target.numel() != self.image_floats or target.dtype != torch.float32 or not target.is_cuda:
            raise RuntimeError("target must hold %d float32 values on the GPU" % self.image_floats)
        if grads_in_forward and max(int(C) for _, _, C in self.meshes) <= 32:
            return _BatchL1GradFn.apply(pos.contiguous(), attr.contiguous().reshape(-1),
                                        target.contiguous().reshape(-1), self)
        return _BatchL1Fn.apply(pos.contiguous(), attr.contiguous().reshape(-1), target.contiguous().reshape(-1),
                                self)

    def forward_buffers(self, pos, attr):
        """Forward without autograd; returns (rast, colour, output) packed."""
        rast, color = self._buffers()
        out = torch.empty_like(color)
        self._forward_raw(pos.contiguous(), attr.contiguous().reshape(-1), rast, color, out)
        return rast, color, out


def _zero_grads(pos, attr):
    """Zeroed gradient buffers for pos and attr from one fill (the fused
    backward accumulates into them); pos rows stay 16-byte aligned."""
    buf = torch.zeros(pos.numel() + attr.numel(), dtype=torch.float32, device=pos.device)
    return buf[:pos.numel()].view_as(pos), buf[pos.numel():].view_as(attr)


def _chunk_views(r, fl, chunk, l1):
    """A chunk's colour / output (/ sign gradient) views of the float scratch."""
    stride = (max(c.renderer.image_floats for c in r._chunks) + 63) // 64 * 64
    n = chunk.renderer.image_floats
    views = [fl[k * stride:k * stride + n] for k in range(3 if l1 else 2)]
    return views


class _BatchFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, attr, renderer):
        ctx.renderer = renderer
        if renderer.recompute:
            out = torch.empty(renderer.image_floats, dtype=torch.float32, device=pos.device)
            rast, fl, flags, _ = renderer._chunk_scratch(l1=False)
            for c in renderer._chunks:
                color, _ = _chunk_views(renderer, fl, c, False)
                c.renderer._forward_raw(pos[c.rows], attr, rast, color, out[c.floats], flags=flags)
            ctx.save_for_backward(pos, attr)
            return out
        rast, color = renderer._buffers()
        out = torch.empty_like(color)
        flags = renderer._flags()
        renderer._forward_raw(pos, attr, rast, color, out, flags=flags)
        ctx.gen = renderer._fwd_gen
        ctx.save_for_backward(pos, attr, flags, rast, color)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        r = ctx.renderer
        grad_out = grad_out.contiguous()
        if r.recompute:
            pos, attr = ctx.saved_tensors
            grad_pos, grad_attr = _zero_grads(pos, attr)
            rast, fl, flags, _ = r._chunk_scratch(l1=False)
            for c in r._chunks:
                cr = c.renderer
                color, out = _chunk_views(r, fl, c, False)
                cr._forward_raw(pos[c.rows], attr, rast, color, out, flags=flags)
                cr._backward_raw(pos[c.rows], attr, rast, color, grad_out[c.floats], grad_pos[c.rows], grad_attr,
                                 cr._fwd_gen, aa_flags=flags)
            return grad_pos, grad_attr, None
        pos, attr, flags, rast, color = ctx.saved_tensors
        grad_pos, grad_attr = _zero_grads(pos, attr)
        r._backward_raw(pos, attr, rast, color, grad_out, grad_pos, grad_attr, ctx.gen, aa_flags=flags)
        return grad_pos, grad_attr, None


class _BatchL1Fn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, attr, target, renderer):
        ctx.set_materialize_grads(False)
        ctx.renderer = renderer
        scale = 1.0 / renderer.image_floats
        if renderer.recompute:
            out = torch.empty(renderer.image_floats, dtype=torch.float32, device=pos.device)
            losses = torch.empty(len(renderer._chunks), dtype=torch.float32, device=pos.device)
            rast, fl, flags, block_loss = renderer._chunk_scratch(l1=True)
            for k, c in enumerate(renderer._chunks):
                color, _, grad = _chunk_views(renderer, fl, c, True)
                c.renderer._forward_raw(pos[c.rows], attr, rast, color, out[c.floats],
                                        (target[c.floats], scale, grad, block_loss, losses[k]), flags=flags)
            ctx.save_for_backward(pos, attr, target)
            return losses.sum(), out
        rast, color = renderer._buffers()
        out = torch.empty_like(color)
        grad = torch.empty_like(color)
        block_loss = torch.empty(max(1, renderer.pixel_blocks), dtype=torch.float32, device=pos.device)
        loss = torch.empty((), dtype=torch.float32, device=pos.device)
        flags = renderer._flags()
        renderer._forward_raw(pos, attr, rast, color, out, (target, scale, grad, block_loss, loss), flags=flags)
        ctx.gen = renderer._fwd_gen
        ctx.save_for_backward(pos, attr, grad, flags, rast, color)
        return loss, out

    @staticmethod
    def backward(ctx, g_loss, g_out):
        r = ctx.renderer
        if r.recompute:
            pos, attr, target = ctx.saved_tensors
            grad_pos, grad_attr = _zero_grads(pos, attr)
            if g_loss is None and g_out is None:
                return grad_pos, grad_attr, None, None
            scale = None if g_loss is None else g_loss.reshape(1).to(torch.float32).contiguous()
            g_out = None if g_out is None else g_out.contiguous()
            rast, fl, flags, block_loss = r._chunk_scratch(l1=True)
            loss_c = torch.empty((), dtype=torch.float32, device=pos.device)
            for c in r._chunks:
                cr = c.renderer
                color, out, grad = _chunk_views(r, fl, c, True)
                cr._forward_raw(pos[c.rows], attr, rast, color, out,
                                (target[c.floats], 1.0 / r.image_floats, grad, block_loss, loss_c), flags=flags)
                if g_out is None:
                    gout, gsc = grad, scale  # sign / n, scaled by the loss gradient inside the kernel
                elif g_loss is None:
                    gout, gsc = g_out[c.floats], None
                else:
                    gout, gsc = grad * g_loss + g_out[c.floats], None
                cr._backward_raw(pos[c.rows], attr, rast, color, gout, grad_pos[c.rows], grad_attr, cr._fwd_gen,
                                 gsc, aa_flags=flags)
            return grad_pos, grad_attr, None, None
        pos, attr, grad, flags, rast, color = ctx.saved_tensors
        gen = ctx.gen
        grad_pos, grad_attr = _zero_grads(pos, attr)
        if g_loss is None and g_out is None:
            return grad_pos, grad_attr, None, None
        scale = None
        if g_out is None:
            gout = grad  # sign / n, scaled by the loss gradient inside the kernel
            scale = g_loss.reshape(1).to(torch.float32).contiguous()
        elif g_loss is None:
            gout = g_out.contiguous()
        else:
            gout = (grad * g_loss + g_out).contiguous()
        r._backward_raw(pos, attr, rast, color, gout, grad_pos, grad_attr, gen, scale, aa_flags=flags)
        return grad_pos, grad_attr, None, None


class _BatchL1GradFn(torch.autograd.Function):
    """render_l1 with the loss's gradient formed in the forward pass."""

    @staticmethod
    def forward(ctx, pos, attr, target, renderer):
        ctx.set_materialize_grads(False)
        ctx.renderer = renderer
        scale = 1.0 / renderer.image_floats
        # one buffer for both gradients, zeroed by the first forward kernel
        gbuf = torch.empty(pos.numel() + attr.numel(), dtype=torch.float32, device=pos.device)
        gpos, gattr = gbuf[:pos.numel()].view_as(pos), gbuf[pos.numel():].view_as(attr)
        out = torch.empty(renderer.image_floats, dtype=torch.float32, device=pos.device)
        if renderer.recompute:
            losses = torch.empty(len(renderer._chunks), dtype=torch.float32, device=pos.device)
            rast, fl, flags, block_loss = renderer._chunk_scratch(l1=False)
            for k, c in enumerate(renderer._chunks):
                color, _ = _chunk_views(renderer, fl, c, False)
                c.renderer._forward_raw(pos[c.rows], attr, rast, color, out[c.floats],
                                        (target[c.floats], scale, block_loss, losses[k], gpos[c.rows], gattr,
                                         gbuf if k == 0 else None), flags=flags)
            ctx.save_for_backward(pos, attr, target, out, gbuf)
            return losses.sum(), out
        rast, color = renderer._buffers()
        block_loss = torch.empty(max(1, renderer.pixel_blocks), dtype=torch.float32, device=pos.device)
        loss = torch.empty((), dtype=torch.float32, device=pos.device)
        flags = renderer._flags()
        renderer._forward_raw(pos, attr, rast, color, out, (target, scale, block_loss, loss, gpos, gattr, gbuf),
                              flags=flags)
        ctx.gen = renderer._fwd_gen
        ctx.save_for_backward(pos, attr, target, out, gbuf, flags, rast, color)
        return loss, out

    @staticmethod
    def backward(ctx, g_loss, g_out):
        r = ctx.renderer
        saved = ctx.saved_tensors
        pos, attr, target, out, gbuf = saved[:5]
        if g_out is None:
            if g_loss is None:
                return torch.zeros_like(pos), torch.zeros_like(attr), None, None
            g = torch.empty_like(gbuf)
            gl = g_loss.reshape(1).to(torch.float32).contiguous()
            _ffi.call("drp_scale_floats", g.data_ptr(), gbuf.data_ptr(), gbuf.numel(), gl.data_ptr(),
                      _ffi.stream_of(gbuf.device))
            return g[:pos.numel()].view_as(pos), g[pos.numel():].view_as(attr), None, None
        # the images reach the objective too: the full backward of
        # g_loss * loss + <g_out, images>
        gout = g_out.contiguous()
        if g_loss is not None:
            gout = gout + torch.sign(out - target) * (g_loss.to(torch.float32) / r.image_floats)
        grad_pos, grad_attr = _zero_grads(pos, attr)
        if r.recompute:
            rast, fl, flags, _ = r._chunk_scratch(l1=False)
            for c in r._chunks:
                cr = c.renderer
                color, outc = _chunk_views(r, fl, c, False)
                cr._forward_raw(pos[c.rows], attr, rast, color, outc, flags=flags)
                cr._backward_raw(pos[c.rows], attr, rast, color, gout[c.floats], grad_pos[c.rows], grad_attr,
                                 cr._fwd_gen, aa_flags=flags)
            return grad_pos, grad_attr, None, None
        _, rast, color = saved[5:]
        # the gradient-forming forward fills only the state's pixel list, not
        # its per-pixel flags: the backward evaluates every pixel's
        # antialias terms itself
        r._backward_raw(pos, attr, rast, color, gout, grad_pos, grad_attr, ctx.gen)
        return grad_pos, grad_attr, None, None
