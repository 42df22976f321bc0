"""Edge-gradient visibility operator on the GPU (the operator behind
SurfaceDeferredRenderSession.edge_gradient, diffrp/rendering/surface_deferred.py:120-169
and :777-804).  The forward returns the image unchanged; the backward
(``drp_edge_gradient_bwd``) gives the gradient of every fragment's NDC
position from the colour differences across triangle-id boundaries."""
import torch

from .. import _ffi

__all__ = ["EdgeGradientFn"]


class EdgeGradientFn(torch.autograd.Function):
    """apply(frag_xy (H, W, 2), flat_tris_xy (F, 3, 2), rast (H, W, 4),
    rgb (H, W, C)) -> rgb; all in the bottom-up rast frame."""

    @staticmethod
    def forward(ctx, frag_xy, flat_tris_xy, rast, rgb):
        ctx.save_for_backward(frag_xy, flat_tris_xy, rast, rgb)
        return rgb.view_as(rgb)

    @staticmethod
    def backward(ctx, grad_output):
        frag_xy, tris_xy, rast, rgb = ctx.saved_tensors
        H, W = frag_xy.shape[:2]
        g = grad_output.contiguous().float()
        rgb_c = rgb.detach().contiguous().float()
        fxy = frag_xy.detach().contiguous().float()
        txy = tris_xy.detach().contiguous().float()
        r = rast.detach().contiguous()
        out = torch.empty((H, W, 2), dtype=torch.float32, device=frag_xy.device)
        _ffi.call("drp_edge_gradient_bwd", fxy.data_ptr(), txy.data_ptr(), txy.shape[0], r.data_ptr(),
                  rgb_c.data_ptr(), rgb_c.shape[-1], g.data_ptr(), H, W, out.data_ptr(),
                  _ffi.stream_of(frag_xy.device))
        return out.to(frag_xy.dtype), None, None, grad_output.clone()
