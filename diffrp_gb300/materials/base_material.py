"""Material (shader) interface of the surface-deferred pipeline (API of
diffrp/materials/base_material.py:12-382).

A material's ``shade(su, si)`` receives uniforms and a batch of fragments and
returns a ``SurfaceOutputStandard``; fragment attributes are interpolated on
demand through ``SurfaceInput.interpolate_ex``, which lands on the CUDA
interpolation kernels.
"""
import abc
from collections.abc import Mapping
from dataclasses import dataclass
from typing import Dict, Optional

import torch

from ..utils.cache import cached, key_cached
from ..utils.shader_ops import float4, normalized, small_matrix_inverse, transform_point4x3, transform_vector3x3

__all__ = ["VertexArrayObject", "SurfaceUniform", "SurfaceInput", "CustomSurfaceInputs", "SurfaceOutputStandard",
           "SurfaceMaterial"]


@dataclass
class VertexArrayObject:
    """Scene-wide vertex and index buffers (built by the render session)."""
    verts: torch.Tensor
    normals: torch.Tensor
    world_pos: torch.Tensor
    tris: torch.Tensor
    stencils: torch.Tensor
    color: torch.Tensor
    uv: torch.Tensor
    tangents: torch.Tensor
    custom_attrs: Dict[str, torch.Tensor]


@dataclass
class SurfaceUniform:
    """Model, view and projection matrices (4x4, GL conventions)."""
    M: torch.Tensor
    V: torch.Tensor
    P: torch.Tensor

    @property
    @cached
    def camera_matrix(self):
        """Camera pose (inverse of V)."""
        return small_matrix_inverse(self.V)

    @property
    @cached
    def camera_position(self):
        return self.camera_matrix[:3, 3]


_WORLD_TRANSFORMS = ("none", "vector", "vectornor", "point", "vector3ex1", "vector3norex1")


class SurfaceInput:
    """Fragment attributes available to ``shade``; each property interpolates
    the corresponding vertex buffer once and caches the result."""

    def __init__(self, uniforms, vertex_buffers, interpolator):
        self.cache = {}
        self.uniforms = uniforms
        self.interpolator = interpolator
        self.vertex_buffers = vertex_buffers
        self.custom_surface_inputs = CustomSurfaceInputs(self)

    def interpolate_ex(self, vertex_buffer, world_transform="none"):
        """Interpolate a (V, C) vertex buffer at the fragments, after an
        optional world-space transform by the model matrix: 'point', 'vector',
        'vectornor' (normalise after transforming), 'vector3ex1' /
        'vector3norex1' (first three channels as a vector, fourth as-is)."""
        M = self.uniforms.M
        if world_transform == "point":
            vertex_buffer = transform_point4x3(vertex_buffer, M)
        elif world_transform == "vector":
            vertex_buffer = transform_vector3x3(vertex_buffer, M)
        elif world_transform == "vectornor":
            vertex_buffer = normalized(transform_vector3x3(vertex_buffer, M))
        elif world_transform == "vector3ex1":
            vertex_buffer = float4(transform_vector3x3(vertex_buffer[..., :3], M), vertex_buffer[..., 3:4])
        elif world_transform == "vector3norex1":
            vertex_buffer = float4(normalized(transform_vector3x3(vertex_buffer[..., :3], M)),
                                   vertex_buffer[..., 3:4])
        elif world_transform != "none":
            raise ValueError("world_transform must be one of %s" % (_WORLD_TRANSFORMS,))
        return self.interpolator.interpolate(vertex_buffer)

    @property
    @cached
    def view_dir(self):
        return normalized(self.world_pos - self.uniforms.camera_position)

    @property
    @cached
    def world_pos(self):
        return self.interpolate_ex(self.vertex_buffers.world_pos)

    @property
    @cached
    def local_pos(self):
        return self.interpolate_ex(self.vertex_buffers.verts)

    @property
    @cached
    def world_normal_unnormalized(self):
        return self.interpolate_ex(self.vertex_buffers.normals, "vectornor")

    @property
    @cached
    def world_normal(self):
        return normalized(self.world_normal_unnormalized)

    @property
    @cached
    def color(self):
        return self.interpolate_ex(self.vertex_buffers.color)

    @property
    @cached
    def uv(self):
        return self.interpolate_ex(self.vertex_buffers.uv)

    @property
    @cached
    def uv_da(self):
        """Screen-space derivatives of ``uv``, (du/dX, du/dY, dv/dX, dv/dY)
        in the layout of ``uv`` with 4 channels: the level of detail of
        mip-mapped texture sampling.  Needs a session with
        ``derivatives=True`` (an addition to the reference API)."""
        return self.interpolator.derivatives(self.vertex_buffers.uv)

    @property
    @cached
    def world_tangent(self):
        return self.interpolate_ex(self.vertex_buffers.tangents, "vector3norex1")

    @property
    def custom_attrs(self):
        return self.custom_surface_inputs


class CustomSurfaceInputs(Mapping):
    """Lazy mapping name -> interpolated custom attribute."""

    def __init__(self, si):
        self.si = si

    @key_cached
    def __getitem__(self, attr):
        return self.si.interpolate_ex(self.si.vertex_buffers.custom_attrs[attr])

    def __len__(self):
        return len(self.si.vertex_buffers.custom_attrs)

    def __iter__(self):
        return iter(self.si.vertex_buffers.custom_attrs)


@dataclass
class SurfaceOutputStandard:
    """Material outputs, all optional (see the defaults in the session's
    G-buffer collectors): albedo (3), normal (3, in ``normal_space``),
    emission (3), metallic / smoothness / occlusion / alpha (1), aovs."""
    albedo: Optional[torch.Tensor] = None
    normal: Optional[torch.Tensor] = None
    emission: Optional[torch.Tensor] = None
    metallic: Optional[torch.Tensor] = None
    smoothness: Optional[torch.Tensor] = None
    occlusion: Optional[torch.Tensor] = None
    alpha: Optional[torch.Tensor] = None
    aovs: Optional[Dict[str, torch.Tensor]] = None
    normal_space: str = "tangent"


class SurfaceMaterial(metaclass=abc.ABCMeta):
    @abc.abstractmethod
    def shade(self, su, si):
        """Return a SurfaceOutputStandard for the fragment batch ``si``; must be
        trivially batched over fragments."""
        raise NotImplementedError
