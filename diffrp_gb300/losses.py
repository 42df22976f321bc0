"""Fused image losses for fitting renders to targets.

``l1_loss(pred, target)`` equals ``(pred - target).abs().mean()`` (gradient
sign(pred - target) / n, zero at exact ties, as torch's abs) but reads both
images once and writes the gradient in the same pass
(``drp_l1_loss_fwd``), instead of the separate subtract / abs / mean /
sign / multiply passes of the unfused expression.
"""
import torch

from . import _ffi

__all__ = ["l1_loss"]


class _L1(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pred, target):
        n = pred.numel()
        p = pred.contiguous()
        t = target.contiguous()
        grad = torch.empty_like(p)
        loss = torch.empty((), dtype=torch.float32, device=p.device)
        ws = torch.empty(_ffi.size_out("drp_l1_loss_workspace_size", n), dtype=torch.uint8, device=p.device)
        _ffi.call("drp_l1_loss_fwd", ws.data_ptr(), ws.numel(), p.data_ptr(), t.data_ptr(), n, 1.0 / n,
                  loss.data_ptr(), grad.data_ptr(), _ffi.stream_of(p.device))
        ctx.save_for_backward(grad)
        ctx.target_grad = target.requires_grad
        return loss

    @staticmethod
    def backward(ctx, g):
        grad, = ctx.saved_tensors
        gp = grad * g
        return gp, (-gp if ctx.target_grad else None)


def l1_loss(pred, target):
    """Mean absolute error between two float32 CUDA tensors of equal shape."""
    if pred.shape != target.shape or pred.dtype != torch.float32 or target.dtype != torch.float32:
        raise RuntimeError("l1_loss expects float32 tensors of the same shape")
    if not (pred.is_cuda and target.is_cuda):
        raise RuntimeError("l1_loss expects CUDA tensors")
    return _L1.apply(pred, target)
