"""Session helpers: camera matrices, the scene-wide vertex array object and
the stencil-masked G-buffer scatter (API of diffrp/rendering/mixin.py:16-155)."""
from typing import Callable, List, Tuple

import torch

from ..materials.base_material import SurfaceInput, SurfaceOutputStandard, VertexArrayObject
from ..utils.cache import cached
from ..utils.shader_ops import cross, fma, normalized, transform_point4x3, transform_vector3x3, zeros_like_vec

__all__ = ["RenderSessionMixin"]


class RenderSessionMixin:
    scene = None
    camera = None

    @cached
    def camera_VP(self):
        return torch.mm(self.camera_P(), self.camera_V())

    @cached
    def camera_P(self):
        return self.camera.P()

    @cached
    def camera_V(self):
        return self.camera.V()

    @staticmethod
    def _concat(parts):
        return parts[0] if len(parts) == 1 else torch.cat(parts)

    def _checked_concat(self, attrs, verts, dim):
        for v, a in zip(verts, attrs):
            if v.shape[0] != a.shape[0]:
                raise ValueError("attribute length not the same as number of vertices")
            if dim is not None and a.shape[-1] != dim:
                raise ValueError("expected %d dims but got %d for vertex attribute" % (dim, a.shape[-1]))
        return self._concat(attrs)

    @cached
    def vertex_array_object(self) -> VertexArrayObject:
        """Concatenate every object: world positions (model matrix applied),
        triangles offset into the shared vertex range, and a per-triangle
        stencil (object index + 1; entry 0 is the background)."""
        objs = self.scene.objects
        if not objs:
            raise ValueError("the scene has no objects")
        dev = objs[0].verts.device
        world_pos, tris, stencils = [], [], [torch.zeros([1], dtype=torch.int64, device=dev)]
        base = 0
        for s, o in enumerate(objs):
            if o.tris.shape[-1] != 3:
                raise ValueError("Expected 3 vertices per triangle, got %d" % o.tris.shape[-1])
            world_pos.append(transform_point4x3(o.verts, o.M))
            tris.append(o.tris + base)
            stencils.append(torch.full([len(o.tris)], s + 1, dtype=torch.int64, device=o.tris.device))
            base += len(o.verts)
        names = set()
        for o in objs:
            names.update(o.custom_attrs.keys())
        for k in names:
            width = next(o.custom_attrs[k].shape[-1] for o in objs if k in o.custom_attrs)
            for o in objs:
                if k in o.custom_attrs:
                    if len(o.custom_attrs[k]) != len(o.verts):
                        raise ValueError("Attribute length not the same as number of vertices: %s" % k)
                    if o.custom_attrs[k].shape[-1] != width:
                        raise ValueError("Different dimensions for same custom attribute: %d != %d"
                                         % (o.custom_attrs[k].shape[-1], width))
                else:
                    o.custom_attrs[k] = zeros_like_vec(o.verts, width)
        verts = [o.verts for o in objs]
        return VertexArrayObject(
            self._checked_concat(verts, verts, 3),
            self._checked_concat([o.normals for o in objs], verts, 3),
            self._concat(world_pos),
            self._concat(tris).int().contiguous(),
            self._concat(stencils).int().contiguous(),
            self._checked_concat([o.color for o in objs], verts, None),
            self._checked_concat([o.uv for o in objs], verts, 2),
            self._checked_concat([o.tangents for o in objs], verts, 4),
            {k: torch.cat([o.custom_attrs[k] for o in objs]) for k in names},
        )

    def _collector_world_normal(self, si: SurfaceInput, so: SurfaceOutputStandard):
        if so.normal is None:
            return si.world_normal
        if so.normal_space == "tangent":
            vn = si.world_normal_unnormalized
            t = so.normal
            tangent, sign = si.world_tangent[..., :3], si.world_tangent[..., 3:4]
            bitangent = sign * cross(vn, tangent)
            return normalized(fma(t[..., 0:1], tangent, fma(t[..., 1:2], bitangent, t[..., 2:3] * vn)))
        if so.normal_space == "object":
            return normalized(transform_vector3x3(so.normal, si.uniforms.M))
        if so.normal_space == "world":
            return normalized(so.normal)
        raise ValueError("Unknown normal space: " + str(so.normal_space))

    def _gbuffer_collect_layer_impl_stencil_masked(self, mats: List[Tuple[SurfaceInput, SurfaceOutputStandard]],
                                                   operator: Callable, initial_buffer: torch.Tensor):
        """Scatter each material's (N, C) operator output into the
        default-filled (1, H, W, C) buffer at its stencil pixels."""
        index_parts, value_parts = [], []
        for si, so in mats:
            ip = si.interpolator
            if len(ip.indices[0]) == 0:
                continue
            val = operator(si, so)
            if val is not None:
                index_parts.append(ip.indices)
                value_parts.append(val)
        if not index_parts:
            return initial_buffer
        if len(index_parts) == 1:
            return initial_buffer.index_put(index_parts[0], value_parts[0])
        dims = len(index_parts[0])
        idx = tuple(torch.cat([p[d] for p in index_parts]) for d in range(dims))
        return initial_buffer.index_put(idx, torch.cat(value_parts))
