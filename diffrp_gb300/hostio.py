"""Host <-> device transport of a step's inputs and results by the SMs.

``device_view(t)`` gives a CUDA tensor aliasing a pinned CPU tensor (its
mapped device address, ``drp_host_device_pointer``); ``copy_(dst, src)``
copies between any two CUDA tensors of equal byte size with a kernel
(``drp_copy_async``), stream-ordered and capturable in a CUDA graph.  With
one end a device view this is a host -> device or device -> host transfer
over the host link without a copy engine: for the few hundred kilobytes of a
fitting step (parameters in, loss and gradients out) the DMA set-up latency
otherwise dominates.
"""
import ctypes

import torch

from . import _ffi

__all__ = ["device_view", "copy_"]

_TYPESTR = {torch.float32: "<f4", torch.int32: "<i4", torch.uint8: "|u1", torch.float64: "<f8", torch.int64: "<i8"}


class _Iface:
    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (ptr, False),
                                         "version": 2}


def device_view(t, device=None):
    """CUDA tensor aliasing the contiguous pinned CPU tensor t (no copy).
    Raises RuntimeError when t is not pinned (mapped) host memory."""
    if t.is_cuda or not t.is_pinned() or not t.is_contiguous() or t.dtype not in _TYPESTR:
        raise RuntimeError("device_view expects a contiguous pinned CPU tensor of a plain numeric dtype")
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    out = ctypes.c_void_p()
    _ffi.call("drp_host_device_pointer", ctypes.c_void_p(t.data_ptr()), ctypes.byref(out))
    view = torch.as_tensor(_Iface(out.value, t.shape, _TYPESTR[t.dtype]), device=dev)
    view._host_owner = t  # the host buffer outlives its view
    return view


def copy_(dst, src):
    """dst <- src bytewise with a kernel on the current stream; both CUDA
    tensors (device memory or device views), contiguous, of equal byte size,
    not overlapping."""
    if not (dst.is_cuda and src.is_cuda and dst.is_contiguous() and src.is_contiguous()):
        raise RuntimeError("copy_ expects contiguous CUDA tensors")
    n = dst.numel() * dst.element_size()
    if src.numel() * src.element_size() != n:
        raise RuntimeError("copy_ expects tensors of equal byte size")
    _ffi.call("drp_copy_async", dst.data_ptr(), src.data_ptr(), n, _ffi.stream_of(dst.device))
    return dst
