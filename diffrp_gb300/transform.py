"""Clip-space transform of vertices by per-view matrices.

``clip_space(verts, mats)`` is ``[verts, 1] @ mats^T`` -- the clip-space
positions of SurfaceDeferredRenderSession.clip_space
(diffrp/rendering/surface_deferred.py:229-238, through transform_point,
diffrp/utils/shader_ops.py:123-136) -- for one (4, 4) matrix or a batch of
views (B, 4, 4), as one kernel (``drp_transform_points_fwd``) instead of a
padded small GEMM.  ``clip_space_packed`` transforms several meshes, each by
its own views, straight into one packed (rows, 4) buffer (the batching form's
position layout), skipping the concatenation.  The vertex gradient sums the
views' contributions per vertex in view order (``drp_transform_points_bwd``,
no atomics); a matrix gradient, when a matrix requires one, is a batched
product over the vertices.
"""
import torch

from . import _ffi

__all__ = ["clip_space", "clip_space_packed"]


def _check(verts, mats):
    if verts.dim() != 2 or verts.shape[1] != 3 or verts.dtype != torch.float32 or not verts.is_cuda:
        raise RuntimeError("clip_space expects (V, 3) float32 CUDA vertices")
    if mats.shape[-2:] != (4, 4) or mats.dim() not in (2, 3) or mats.dtype != torch.float32 or \
            mats.device != verts.device:
        raise RuntimeError("clip_space expects (4, 4) or (B, 4, 4) float32 matrices on the vertices' device")


def _mat_grad(g_rows, verts, mats3):
    # d/dM_b of [v, 1] M_b^T summed over vertices: (B, 4, V) @ (V, 4)
    vh = torch.nn.functional.pad(verts, (0, 1), value=1.0)
    return torch.matmul(g_rows.view(mats3.shape[0], -1, 4).transpose(1, 2), vh)


class _ClipPacked(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rows, *pairs):
        groups = [(pairs[2 * k].contiguous(), pairs[2 * k + 1].reshape(-1, 4, 4).contiguous())
                  for k in range(len(pairs) // 2)]
        dev = groups[0][0].device
        out = torch.empty((rows, 4), dtype=torch.float32, device=dev)
        stream = _ffi.stream_of(dev)
        r = 0
        for v, m in groups:
            n = v.shape[0] * m.shape[0]
            if n:
                _ffi.call("drp_transform_points_fwd", v.data_ptr(), v.shape[0], m.data_ptr(), m.shape[0],
                          out[r:].data_ptr(), stream)
            r += n
        ctx.save_for_backward(*[t for g in groups for t in g])
        ctx.mat_shapes = [pairs[2 * k + 1].shape for k in range(len(pairs) // 2)]
        return out

    @staticmethod
    def backward(ctx, g):
        saved = ctx.saved_tensors
        g = g.contiguous()
        if g.data_ptr() % 16:
            g = g.clone()
        stream = _ffi.stream_of(g.device)
        grads = [None]
        r = 0
        for k in range(len(saved) // 2):
            v, m = saved[2 * k], saved[2 * k + 1]
            n = v.shape[0] * m.shape[0]
            gv = gm = None
            if ctx.needs_input_grad[1 + 2 * k]:
                gv = torch.empty_like(v)
                if n:
                    _ffi.call("drp_transform_points_bwd", g[r:].data_ptr(), v.shape[0], m.data_ptr(), m.shape[0],
                              gv.data_ptr(), stream)
                else:
                    gv.zero_()
            if ctx.needs_input_grad[2 + 2 * k]:
                gm = _mat_grad(g[r:r + n], v, m).reshape(ctx.mat_shapes[k])
            grads += [gv, gm]
            r += n
        return tuple(grads)


def clip_space_packed(groups):
    """groups: [(verts (V, 3), mats (B, 4, 4) or (4, 4))] -> (sum B * V, 4)
    float32, group after group, each group view-major (view b's vertices at
    rows [b * V, (b + 1) * V) of the group)."""
    pairs = []
    rows = 0
    for v, m in groups:
        _check(v, m)
        rows += v.shape[0] * (m.shape[0] if m.dim() == 3 else 1)
        pairs += [v, m]
    if not pairs:
        raise RuntimeError("clip_space_packed expects at least one group")
    return _ClipPacked.apply(rows, *pairs)


def clip_space(verts, mats):
    """[verts, 1] @ mats^T: (V, 3) with (4, 4) -> (V, 4); with (B, 4, 4) ->
    (B, V, 4)."""
    _check(verts, mats)
    out = _ClipPacked.apply(verts.shape[0] * (mats.shape[0] if mats.dim() == 3 else 1), verts, mats)
    return out.view(mats.shape[0], verts.shape[0], 4) if mats.dim() == 3 else out
