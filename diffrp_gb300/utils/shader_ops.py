"""GLSL-flavoured tensor helpers used on the rendering path (the subset of
diffrp/utils/shader_ops.py the surface-deferred session and materials need).

Importing this module also installs swizzle properties on ``torch.Tensor``
(``t.xyz``, ``t.rgb``, ``t.w`` ... over the last dimension, keeping it), the
sugar diffrp's materials are written in (shader_ops.py:599-634).
"""
import itertools

import numpy
import torch
import torch.nn.functional as F

__all__ = [
    "gpu_f32", "gpu_i32", "fma", "fsa", "zeros_like_vec", "ones_like_vec", "full_like_vec", "homogeneous",
    "homogeneous_vec", "transform_point", "transform_point4x3", "transform_vector", "transform_vector3x3",
    "normalized", "length", "dot", "cross", "saturate", "float2", "float3", "float4", "floatx",
    "small_matrix_inverse", "split_alpha",
]


def _device():
    return torch.device("cuda", torch.cuda.current_device())


def gpu_f32(x):
    """float32 tensor on the current CUDA device from a number / list / array / tensor."""
    if isinstance(x, torch.Tensor):
        return x.to(device=_device(), dtype=torch.float32)
    if isinstance(x, (int, float)):
        return torch.full([], float(x), dtype=torch.float32, device=_device())
    return torch.tensor(numpy.asarray(x), dtype=torch.float32, device=_device())


def gpu_i32(x):
    if isinstance(x, torch.Tensor):
        return x.to(device=_device(), dtype=torch.int32)
    return torch.tensor(numpy.asarray(x), dtype=torch.int32, device=_device())


def fma(x, y, b, a=1.0):
    """b + a * x * y (torch.addcmul)."""
    return torch.addcmul(b, x, y, value=a)


def fsa(a, x, b):
    """b + a * x."""
    return torch.add(b, x, alpha=a)


def zeros_like_vec(x, v):
    return x.new_zeros(*x.shape[:-1], v)


def ones_like_vec(x, v):
    return x.new_ones(*x.shape[:-1], v)


def full_like_vec(x, value, v):
    return x.new_full([*x.shape[:-1], v], value)


def homogeneous(p):
    return F.pad(p, (0, 1), value=1.0)


def homogeneous_vec(p):
    return F.pad(p, (0, 1), value=0.0)


def transform_point(xyz, matrix):
    """[xyz, 1] @ matrix^T -> (..., 4)."""
    return torch.matmul(homogeneous(xyz), matrix.T)


def transform_point4x3(xyz, matrix):
    """Affine transform of points (B, 3) -> (B, 3)."""
    return torch.addmm(matrix[:-1, -1], xyz, matrix[:-1, :-1].T)


def transform_vector(xyz, matrix):
    return torch.matmul(homogeneous_vec(xyz), matrix.T)[..., :3]


def transform_vector3x3(xyz, matrix):
    return torch.matmul(xyz, matrix[:-1, :-1].T)


def normalized(x, dim=-1, eps=1e-12):
    return F.normalize(x, dim=dim, eps=eps)


def length(x):
    return torch.linalg.norm(x, dim=-1, keepdim=True)


def dot(a, b, keepdim=True):
    r = (a * b).sum(-1)
    return r.unsqueeze(-1) if keepdim else r


def cross(a, b):
    return torch.linalg.cross(a, b)


def saturate(x):
    return torch.clamp(x, 0.0, 1.0)


def _vec(*parts):
    ref = next((p for p in parts if isinstance(p, torch.Tensor)), None)
    out = []
    for p in parts:
        if isinstance(p, torch.Tensor):
            out.append(p)
        else:
            out.append(torch.full([*ref.shape[:-1], 1], float(p), dtype=ref.dtype, device=ref.device))
    shape = torch.broadcast_shapes(*[o.shape[:-1] for o in out])
    return torch.cat([o.expand(*shape, o.shape[-1]) for o in out], dim=-1)


def float2(*parts):
    return _vec(*parts)


def float3(*parts):
    return _vec(*parts)


def float4(*parts):
    return _vec(*parts)


def floatx(*parts):
    return _vec(*parts)


def split_alpha(x):
    return x[..., :-1], x[..., -1:]


class _SmallMatrixInverse(torch.autograd.Function):
    @staticmethod
    def forward(ctx, m):
        inv = torch.linalg.inv(m.double()).to(m.dtype)
        ctx.save_for_backward(inv)
        return inv

    @staticmethod
    def backward(ctx, g):
        inv, = ctx.saved_tensors
        it = inv.transpose(-1, -2)
        return -it @ g @ it


def small_matrix_inverse(m):
    """Inverse of a small (batched) matrix with the analytic backward."""
    return _SmallMatrixInverse.apply(m)


def _install_swizzles():
    for alphabet in ("xyzw", "rgba"):
        for n in range(1, 5):
            for combo in itertools.product(alphabet, repeat=n):
                name = "".join(combo)
                idx = [alphabet.index(c) for c in combo]
                steps = {b - a for a, b in zip(idx, idx[1:])}
                if n == 1:
                    sel = slice(idx[0], idx[0] + 1)
                elif len(steps) == 1 and next(iter(steps)) > 0:
                    s = next(iter(steps))
                    sel = slice(idx[0], idx[-1] + 1, s)
                else:
                    sel = list(idx)
                if not hasattr(torch.Tensor, name):
                    setattr(torch.Tensor, name, property(lambda t, sel=sel: t[..., sel]))


_install_swizzles()
