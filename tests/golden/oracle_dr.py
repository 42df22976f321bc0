"""A CPU ``nvdiffrast.torch`` stand-in backed by the oracle (test
infrastructure for generating golden vectors from the reference's own
session code).

Exposes the names diffrp calls (RasterizeCudaContext, DepthPeeler,
interpolate, antialias) on CPU tensors, with autograd through the oracle's
backward evaluated like a float32 implementation's: every per-pixel term in
float32 (so each branch -- antialias edge, blended pixel, clamping -- is the
one the float32 forward took) and the sums in float64.  A float64 evaluation
of the terms would resolve a few near-tie antialias pairs the other way than
the forward did, which changes the position gradients of their vertices.
"""
import numpy as np
import torch

import oracle as O


class RasterizeCudaContext:
    def __init__(self, device=None):
        self.device = device


class RasterizeGLContext(RasterizeCudaContext):
    pass


def _np(t, dtype=np.float32):
    return t.detach().cpu().numpy().astype(dtype)


class _Raster(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, tri, res, ranges, prev_key):
        rast, db, key = O.rasterize(_np(pos), _np(tri, np.int32), res,
                                    ranges=None if ranges is None else ranges.numpy(), prev_key=prev_key)
        ctx.save_for_backward(pos)
        ctx.tri = _np(tri, np.int32)
        ctx.rast = rast
        ctx.key = key
        return torch.from_numpy(rast), torch.from_numpy(db)

    @staticmethod
    def backward(ctx, g_rast, g_db):
        pos, = ctx.saved_tensors
        g = O.raster_bwd(_np(pos), ctx.tri, ctx.rast, _np(g_rast), None if g_db is None else _np(g_db),
                         precision="f32")
        return torch.from_numpy(g).to(pos.dtype), None, None, None, None


class DepthPeeler:
    def __init__(self, glctx, pos, tri, resolution, ranges=None, grad_db=True):
        self.pos, self.tri, self.res, self.ranges = pos, tri, tuple(resolution), ranges
        self.prev = None

    def __enter__(self):
        self.prev = None
        return self

    def __exit__(self, *a):
        return False

    def rasterize_next_layer(self):
        keyholder = {}

        class _Layer(_Raster):
            @staticmethod
            def forward(ctx, pos, tri, res, ranges, prev_key):
                out = _Raster.forward(ctx, pos, tri, res, ranges, prev_key)
                keyholder["key"] = ctx.key
                return out

        rast, db = _Layer.apply(self.pos, self.tri, self.res, self.ranges, self.prev)
        self.prev = keyholder["key"]
        return rast, db


def rasterize(glctx, pos, tri, resolution, ranges=None, grad_db=True):
    return _Raster.apply(pos, tri, tuple(resolution), ranges, None)


class _Interp(torch.autograd.Function):
    @staticmethod
    def forward(ctx, attr, rast, tri):
        out, _ = O.interpolate(_np(attr), _np(rast), _np(tri, np.int32))
        ctx.save_for_backward(attr, rast, tri)
        return torch.from_numpy(out)

    @staticmethod
    def backward(ctx, g):
        attr, rast, tri = ctx.saved_tensors
        ga, gr, _ = O.interpolate_bwd(_np(attr), _np(rast), _np(tri, np.int32), _np(g), precision="f32")
        return torch.from_numpy(ga).float(), torch.from_numpy(gr).float(), None


def interpolate(attr, rast, tri, rast_db=None, diff_attrs=None):
    out = _Interp.apply(attr, rast, tri)
    return out, torch.zeros(*out.shape[:-1], 0)


class _AA(torch.autograd.Function):
    @staticmethod
    def forward(ctx, color, rast, pos, tri):
        out = O.antialias(_np(color), _np(rast), _np(pos), _np(tri, np.int32))
        ctx.save_for_backward(color, rast, pos, tri)
        return torch.from_numpy(out)

    @staticmethod
    def backward(ctx, g):
        color, rast, pos, tri = ctx.saved_tensors
        gc, gp = O.antialias_bwd(_np(color), _np(rast), _np(pos), _np(tri, np.int32), _np(g), precision="f32")
        return torch.from_numpy(gc).float(), None, torch.from_numpy(gp).float(), None


def antialias(color, rast, pos, tri, topology_hash=None, pos_gradient_boost=1.0):
    return _AA.apply(color, rast, pos, tri)
