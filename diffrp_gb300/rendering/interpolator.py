"""Varying-attribute interpolators (API of diffrp/rendering/interpolator.py).

``polyfill_interpolate`` / ``MaskedSparseInterpolator`` run the sparse CUDA
kernel (``drp_interpolate_sparse_*``); ``FullScreenInterpolator`` calls the
drop-in ``dr.interpolate``.  The tri-id float encoding of the rast w channel
is interpolator.py:24-29.
"""
import abc
from typing import Optional

import torch

from .. import _ffi
from .. import nvdr as dr

__all__ = ["float_to_triidx", "triidx_to_float", "polyfill_interpolate", "Interpolator", "FullScreenInterpolator",
           "MaskedSparseInterpolator"]

_ENC_BASE = 0x4a800000


def float_to_triidx(x):
    """rast w channel -> triangle id + 1 (0 = background)."""
    return torch.where(x <= 16777216, x.int(), x.view(torch.int32) - _ENC_BASE)


def triidx_to_float(x):
    """triangle id + 1 -> rast w channel value."""
    return torch.where(x <= 0x01000000, x.float(), (x + _ENC_BASE).view(torch.float32))


class _SparseInterp(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vb, vi, tri_idx):
        n, C = vi.shape[0], vb.shape[1]
        out = torch.empty((n, C), dtype=torch.float32, device=vb.device)
        _ffi.call("drp_interpolate_sparse_fwd", vb.data_ptr(), vb.shape[0], C, vi.data_ptr(), tri_idx.data_ptr(), n,
                  out.data_ptr(), _ffi.stream_of(vb.device))
        ctx.save_for_backward(vb, vi, tri_idx)
        return out

    @staticmethod
    def backward(ctx, g):
        vb, vi, tri_idx = ctx.saved_tensors
        g = g.contiguous()
        gvb = torch.zeros_like(vb)
        gvi = torch.empty_like(vi)
        _ffi.call("drp_interpolate_sparse_bwd", vb.data_ptr(), vb.shape[0], vb.shape[1], vi.data_ptr(),
                  tri_idx.data_ptr(), vi.shape[0], g.data_ptr(), gvb.data_ptr(), gvi.data_ptr(),
                  _ffi.stream_of(vb.device))
        return gvb, gvi, None


def _sparse(vertex_buffer, vi_data, tri_idx):
    if not (vertex_buffer.is_cuda and vi_data.is_cuda and tri_idx.is_cuda):
        raise RuntimeError("polyfill_interpolate requires CUDA tensors")
    lead = vi_data.shape[:-1]
    vb = vertex_buffer.contiguous().float()
    vi = vi_data.reshape(-1, vi_data.shape[-1]).contiguous().float()
    ti = tri_idx.reshape(-1, 3).contiguous().long()
    if vi.shape[-1] != 4:
        raise RuntimeError("vi_data must have 4 channels (u, v, z, id)")
    out = _SparseInterp.apply(vb, vi, ti)
    return out.reshape(*lead, vb.shape[-1])


def polyfill_interpolate(vertex_buffer, vi_data, tri_idx, empty_region: Optional[float] = None):
    """out = (v1 - v3) u + (v2 - v3) v + v3 for each row of ``vi_data``
    (``tri_idx`` rows give v1, v2, v3); rows with id 0 get ``empty_region``
    when it is given (interpolator.py:32-65)."""
    out = _sparse(vertex_buffer, vi_data, tri_idx)
    if empty_region is not None:
        out = torch.where(vi_data[..., -1:] > 0, out, empty_region)
    return out


class Interpolator(metaclass=abc.ABCMeta):
    vi_data: torch.Tensor

    @abc.abstractmethod
    def interpolate(self, vertex_buffer):
        raise NotImplementedError

    def derivatives(self, vertex_buffer):
        """Screen-space derivatives (dA/dX, dA/dY per channel) of an
        interpolated attribute; needs the layer's rast_db (the session option
        ``derivatives``)."""
        raise RuntimeError("screen-space derivatives need the layer's rast_db "
                           "(SurfaceDeferredRenderSessionOptions(derivatives=True))")


def _derivatives(vertex_buffer, rast, tris, rast_db):
    if rast_db is None or rast_db.shape[-1] != 4:
        raise RuntimeError("screen-space derivatives need the layer's rast_db "
                           "(SurfaceDeferredRenderSessionOptions(derivatives=True))")
    _, da = dr.interpolate(vertex_buffer.contiguous(), rast, tris, rast_db=rast_db, diff_attrs="all")
    return da


class FullScreenInterpolator(Interpolator):
    """Interpolates over the whole (1, H, W) rast with ``dr.interpolate``;
    with the layer's ``rast_db`` it also gives (1, H, W, 2C) derivatives."""

    def __init__(self, vi_data, tris, rast_db=None):
        self.vi_data = vi_data.contiguous()
        self.tris = tris.contiguous()
        self.rast_db = rast_db

    def interpolate(self, vertex_buffer):
        attr, _ = dr.interpolate(vertex_buffer.contiguous(), self.vi_data, self.tris)
        return attr

    def derivatives(self, vertex_buffer):
        return _derivatives(vertex_buffer, self.vi_data, self.tris, self.rast_db)


class MaskedSparseInterpolator(Interpolator):
    """Interpolates only the pixels selected by ``mask`` (one material's
    stencil); results are (N, C) rows in ``mask.nonzero`` order.  With the
    layer's ``rast_db``, derivatives are (N, 2C) rows in the same order."""

    def __init__(self, vi_data, tris, mask, indices=None, rast_db=None):
        self.tris = tris
        # indices: the mask's nonzero index tuple when the caller already has it
        self.indices = mask.nonzero(as_tuple=True) if indices is None else indices
        self.rast = vi_data
        self.rast_db = rast_db
        self.vi_data = vi_data[self.indices]
        self.tri_idx = tris[float_to_triidx(self.vi_data[..., -1]) - 1].long()

    def interpolate(self, vertex_buffer):
        return polyfill_interpolate(vertex_buffer, self.vi_data, self.tri_idx)

    def derivatives(self, vertex_buffer):
        return _derivatives(vertex_buffer, self.rast.contiguous(), self.tris.contiguous(), self.rast_db)[self.indices]


def stencil_groups(stencil, n_objects):
    """For each object id k = 1..n_objects, the index tuple of
    ``(stencil == k).nonzero(as_tuple=True)`` (row-major order), computed for
    all objects at once: one stable sort of the pixels by stencil value and
    one read-back of the per-value counts, instead of one nonzero (each a
    host wait) per object."""
    if n_objects <= 2:
        return [(stencil == k + 1).nonzero(as_tuple=True) for k in range(n_objects)]
    flat = stencil.reshape(-1).long()
    order = torch.sort(flat, stable=True).indices
    counts = torch.bincount(flat, minlength=n_objects + 1)[:n_objects + 1].cpu().tolist()
    groups, off = [], counts[0]
    for k in range(n_objects):
        idx = order[off:off + counts[k + 1]]
        off += counts[k + 1]
        groups.append(torch.unravel_index(idx, stencil.shape))
    return groups
