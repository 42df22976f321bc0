"""Surface-deferred rasterisation session on the GB300 kernels (API of
diffrp/rendering/surface_deferred.py:26-804, the rasterisation part).

Stages: ``clip_space`` -> ``rasterize`` (depth peeling through the drop-in
``dr.DepthPeeler``) -> ``layer_material`` (per object: stencil-masked or
full-screen interpolator, then ``material.shade``) -> ``gbuffer_collect`` ->
``compose_layers``; ``nvdr_antialias`` and ``edge_gradient`` add visibility
gradients.  Image-based lighting (``prepare_ibl`` / ``ibl`` / ``pbr``) is
outside this package's scope and raises.
"""
import threading
import warnings
from dataclasses import dataclass
from typing import Callable, List, Optional, Tuple, Union

import numpy
import torch

from .. import nvdr as dr
from ..transform import clip_space
from ..materials.base_material import SurfaceInput, SurfaceOutputStandard, SurfaceUniform
from ..utils.cache import cached
from ..utils.composite import alpha_additive, alpha_blend
from ..utils.shader_ops import (float3, float4, floatx, length, normalized, ones_like_vec,
                                transform_point4x3, transform_vector3x3)
from .camera import Camera
from .interpolator import FullScreenInterpolator, MaskedSparseInterpolator, float_to_triidx, stencil_groups
from .mixin import RenderSessionMixin

__all__ = ["SurfaceDeferredRenderSession", "SurfaceDeferredRenderSessionOptions"]

_tls = threading.local()


@dataclass
class SurfaceDeferredRenderSessionOptions:
    """Session options.

    max_layers: layers composed for transparency (<= 0: unlimited, capped at
        32767); forced to 1 in ``opaque_only`` sessions.
    interpolator_impl: 'stencil_masked' (default; each material sees only its
        own pixels as (N, C) rows) or 'full_screen' ((1, H, W, C) buffers).
    deterministic and the ibl_* fields are accepted for API compatibility;
        lighting is not part of this package.
    derivatives: rasterise with screen-space derivatives (rast_db), so that
        materials can read ``SurfaceInput.uv_da`` for mip-mapped texture
        sampling (an addition; off by default, as the reference discards
        rast_db).
    """
    max_layers: int = 0
    interpolator_impl: str = "stencil_masked"
    deterministic: bool = True
    ibl_specular_samples: int = 512
    ibl_specular_base_resolution: int = 256
    ibl_specular_mip_levels: int = 5
    ibl_diffuse_sample_resolution: int = 64
    ibl_diffuse_base_resolution: int = 16
    derivatives: bool = False

    def __post_init__(self):
        if self.max_layers <= 0:
            self.max_layers = 32767

    @property
    def intepolator_impl(self):
        warnings.warn("`intepolator_impl` is deprecated, please use `interpolator_impl` instead.")
        return self.interpolator_impl

    @intepolator_impl.setter
    def intepolator_impl(self, value):
        warnings.warn("`intepolator_impl` is deprecated, please use `interpolator_impl` instead.")
        self.interpolator_impl = value


def _constant(values, dtype):
    """A list of numbers (or a tensor) as a device tensor on the current
    device; lists are copied from the host once and reused by later calls
    with the same values (no host wait, CUDA-graph capturable)."""
    if isinstance(values, torch.Tensor):
        return values.to(device=torch.device("cuda", torch.cuda.current_device()), dtype=dtype)
    return dr._device_constant(numpy.asarray(values, dtype=numpy.float64 if dtype.is_floating_point else numpy.int64),
                               dtype, "cuda")


def _thread_context():
    device = torch.cuda.current_device()
    cache = getattr(_tls, "ctx_cache", None)
    if cache is None:
        cache = _tls.ctx_cache = {}
    if device not in cache:
        cache[device] = dr.RasterizeCudaContext()
    return cache[device]


class SurfaceDeferredRenderSession(RenderSessionMixin):
    """Deferred rasterisation of ``scene`` through ``camera``.

    Intermediate results are cached on the session; create a new session when
    the scene or the camera changes.  One raster context is shared per thread
    and device unless ``ctx`` is given.  One GPU per process.
    """

    def __init__(self, scene, camera: Camera, opaque_only: bool = True,
                 options: Optional[SurfaceDeferredRenderSessionOptions] = None, ctx=None):
        self.scene = scene
        self.camera = camera
        self.opaque_only = opaque_only
        if options is None:
            options = SurfaceDeferredRenderSessionOptions()
        if opaque_only:
            options.max_layers = 1
        self.options = options
        self.ctx = ctx if ctx is not None else _thread_context()

    # -- geometry -----------------------------------------------------------
    @cached
    def clip_space(self):
        """All vertices in GL clip space, (V, 4) contiguous: [world_pos, 1] @ VP^T
        in one transform kernel."""
        vao = self.vertex_array_object()
        return clip_space(vao.world_pos.contiguous(), self.camera_VP().contiguous())

    @cached
    def rasterize(self):
        """Rasterised layers, front to back; each (1, H, W, 4) =
        (u, v, z/w, triangle id + 1) with u v1 + v v2 + (1 - u - v) v3 = p.

        Peeling stops at the first empty layer, which is dropped unless it is
        the last layer allowed (surface_deferred.py:258-266).  The emptiness
        of a chunk of up to 4 layers is read back at once: one host wait per
        chunk instead of one per layer (layers past the first empty one are
        rasterised, found empty and dropped).  With options.derivatives the
        layers' screen-space derivatives are kept for the interpolators."""
        vao = self.vertex_array_object()
        clip = self.clip_space()
        h, w = self.camera.resolution()
        ranges = torch.tensor([[0, len(vao.tris)]], dtype=torch.int32)
        L = self.options.max_layers
        layers: List[torch.Tensor] = []
        dbs: List[Optional[torch.Tensor]] = []
        with dr.DepthPeeler(self.ctx, clip, vao.tris.contiguous(), (h, w), ranges,
                            grad_db=self.options.derivatives) as peeler:
            i = 0
            while i < L:
                batch = [peeler.rasterize_next_layer() for _ in range(min(4, L - i))]
                checked = [j for j in range(len(batch)) if i + j < L - 1]
                empty = torch.stack([(batch[j][0][..., 3] <= 0).all() for j in checked]).tolist() if checked else []
                stop = next((j for j, e in zip(checked, empty) if e), None)
                keep = batch if stop is None else batch[:stop]
                layers += [r for r, _ in keep]
                dbs += [db if self.options.derivatives else None for _, db in keep]
                if stop is not None:
                    break
                i += len(batch)
        self._layer_db = dbs
        return layers

    # -- materials ----------------------------------------------------------
    @cached
    def layer_material(self) -> List[List[Tuple[SurfaceInput, SurfaceOutputStandard]]]:
        vao = self.vertex_array_object()
        cam_v, cam_p = self.camera_V(), self.camera_P()
        impl = self.options.interpolator_impl
        out = []
        layers = self.rasterize()
        dbs = getattr(self, "_layer_db", None) or []  # absent when rasterize() was injected into the cache
        for li, rast in enumerate(layers):
            db = dbs[li] if li < len(dbs) else None
            mats = []
            if impl == "stencil_masked":
                stencil = vao.stencils[float_to_triidx(rast[..., -1])]
                groups = stencil_groups(stencil, len(self.scene.objects))
            for pi, obj in enumerate(self.scene.objects):
                su = SurfaceUniform(obj.M, cam_v, cam_p)
                if impl == "full_screen":
                    si = SurfaceInput(su, vao, FullScreenInterpolator(rast, vao.tris, rast_db=db))
                elif impl == "stencil_masked":
                    si = SurfaceInput(su, vao, MaskedSparseInterpolator(rast, vao.tris, None, indices=groups[pi],
                                                                        rast_db=db))
                    if len(si.interpolator.indices[0]) == 0:
                        mats.append((si, SurfaceOutputStandard()))
                        continue
                else:
                    raise ValueError("Unrecognized `interpolator_impl` '%s'" % impl)
                mats.append((si, obj.material.shade(su, si)))
            out.append(mats)
        return out

    def gbuffer_collect(self, operator: Callable, default: Union[List[float], torch.Tensor]) -> List[torch.Tensor]:
        """Collect ``operator(si, so)`` from every material into one
        (1, H, W, C) buffer per layer; ``default`` fills background pixels and
        materials whose operator returns None."""
        vao = self.vertex_array_object()
        h, w = self.camera.resolution()
        C = len(default)
        if self.options.interpolator_impl == "stencil_masked":
            if all(d == default[0] for d in default):
                base = torch.full([1, h, w, C], float(default[0]), dtype=torch.float32, device="cuda")
            else:
                base = _constant(default, torch.float32).expand(1, h, w, C)
            return [self._gbuffer_collect_layer_impl_stencil_masked(mats, operator, base)
                    for mats in self.layer_material()]
        if self.options.interpolator_impl != "full_screen":
            raise ValueError("Unrecognized `interpolator_impl` '%s'" % self.options.interpolator_impl)
        result = []
        for rast, mats in zip(self.rasterize(), self.layer_material()):
            buffers = [_constant(default, torch.float32).expand(1, h, w, C)]
            lookup = [0]
            for si, so in mats:
                val = operator(si, so)
                if val is None:
                    lookup.append(0)
                else:
                    lookup.append(len(buffers))
                    buffers.append(val)
            lookup = _constant(lookup, vao.stencils.dtype)
            which = lookup[vao.stencils][float_to_triidx(rast[..., 3:4])]
            result.append(torch.gather(torch.cat(buffers), 0, which.repeat_interleave(C, dim=-1).long()))
        return result

    def compose_layers(self, colors: list, alphas: Optional[list] = None, blend_fn: Optional[Callable] = None,
                       return_alpha: bool = True) -> torch.Tensor:
        """Blend layers back to front (front layer first in the lists); the
        result is flipped to top-down image rows, (H, W, C [+ 1])."""
        if alphas is None:
            alphas = self.alpha_layered()
        if blend_fn is None:
            blend_fn = alpha_blend
        if len(colors) == 0:
            return torch.zeros(*self.camera.resolution(), 4, dtype=torch.float32, device="cuda")
        acc, acc_a = colors[-1], alphas[-1]
        for c, a in zip(reversed(colors[:-1]), reversed(alphas[:-1])):
            acc, acc_a = blend_fn(acc, acc_a, c, a)
        img = floatx(acc, acc_a) if return_alpha else acc
        return torch.flipud(img.squeeze(0))

    # -- G-buffers ----------------------------------------------------------
    @cached
    def alpha_layered(self):
        if self.opaque_only:
            return self.gbuffer_collect(lambda si, so: ones_like_vec(si.interpolator.vi_data, 1), [0.0])
        return self.gbuffer_collect(
            lambda si, so: so.alpha if so.alpha is not None else ones_like_vec(si.interpolator.vi_data, 1), [0.0])

    @cached
    def albedo_layered(self):
        return self.gbuffer_collect(lambda si, so: so.albedo, [1.0, 0.0, 1.0])

    @cached
    def emission_layered(self):
        return self.gbuffer_collect(lambda si, so: so.emission, [0.0, 0.0, 0.0])

    def _collector_mso(self, si, so):
        if so.metallic is None and so.smoothness is None and so.occlusion is None:
            return None
        return float3(so.metallic if so.metallic is not None else 0.0,
                      so.smoothness if so.smoothness is not None else 0.5,
                      so.occlusion if so.occlusion is not None else 1.0)

    @cached
    def mso_layered(self):
        return self.gbuffer_collect(self._collector_mso, [0.0, 0.5, 1.0])

    @cached
    def world_space_normal_layered(self):
        return self.gbuffer_collect(self._collector_world_normal, [0.0, 0.0, 0.0])

    @cached
    def camera_space_normal_layered(self):
        V = self.camera.V()
        return [normalized(transform_vector3x3(n, V)) for n in self.world_space_normal_layered()]

    @cached
    def depth_layered(self):
        return self.gbuffer_collect(lambda si, so: -transform_point4x3(si.world_pos, self.camera.V())[..., 2:3], [0.0])

    @cached
    def distance_layered(self):
        return self.gbuffer_collect(lambda si, so: length(si.world_pos - si.uniforms.camera_position), [0.0])

    @cached
    def world_position_layered(self):
        return self.gbuffer_collect(lambda si, so: si.world_pos, [0.0, 0.0, 0.0])

    @cached
    def local_position_layered(self):
        return self.gbuffer_collect(lambda si, so: si.local_pos, [0.0, 0.0, 0.0])

    # -- composed images ------------------------------------------------------
    @cached
    def albedo(self):
        return self.compose_layers(self.albedo_layered())

    @cached
    def emission(self):
        return self.compose_layers(self.emission_layered(), blend_fn=alpha_additive, return_alpha=False)

    @cached
    def false_color_mask_mso(self):
        return self.compose_layers(self.mso_layered())

    @cached
    def world_space_normal(self):
        return self.compose_layers(self.world_space_normal_layered())

    @cached
    def camera_space_normal(self):
        return self.compose_layers(self.camera_space_normal_layered())

    @cached
    def false_color_world_space_normal(self):
        n = self.world_space_normal()
        return float4(n[..., :3] * 0.5 + 0.5, n[..., 3:4])

    @cached
    def false_color_camera_space_normal(self):
        n = self.camera_space_normal()
        return float4(n[..., :3] * 0.5 + 0.5, n[..., 3:4])

    @cached
    def local_position(self):
        return self.compose_layers(self.local_position_layered())

    @cached
    def world_position(self):
        return self.compose_layers(self.world_position_layered())

    @cached
    def false_color_nocs(self):
        n = self.local_position()
        return float4(n[..., :3] * 0.5 + 0.5, n[..., 3:4])

    @cached
    def depth(self):
        return self.compose_layers(self.depth_layered(), return_alpha=False)

    @cached
    def distance(self):
        return self.compose_layers(self.distance_layered(), return_alpha=False)

    def aov(self, key: str, bg_value: List[float]):
        """Material AOV ``key`` composed over all layers, (H, W, C + 1)."""
        return self.compose_layers(self.gbuffer_collect(lambda si, so: so.aovs and so.aovs.get(key), bg_value))

    # -- lighting (outside the rasterisation path) ---------------------------
    def prepare_ibl(self):
        raise NotImplementedError("image-based lighting is not part of diffrp_gb300")

    def pbr(self):
        raise NotImplementedError("image-based lighting is not part of diffrp_gb300")

    # -- visibility gradients ------------------------------------------------
    def nvdr_antialias(self, rgb: torch.Tensor):
        """Analytic silhouette antialiasing of an (H, W, C) image rendered by
        this session; gives visibility gradients w.r.t. geometry."""
        img = torch.flipud(rgb)[None].contiguous()
        rast = self.rasterize()[0].contiguous()
        vao = self.vertex_array_object()
        return torch.flipud(dr.antialias(img, rast, self.clip_space(), vao.tris.contiguous(),
                                         topology_hash=self._topology()).squeeze(0))

    @cached
    def _topology(self):
        return dr.antialias_construct_topology_hash(self.vertex_array_object().tris.contiguous())

    def edge_gradient(self, rgb: torch.Tensor):
        """Edge-gradient visibility operator (Rasterized Edge Gradients): the
        (H, W, C) image is returned unchanged; its backward adds gradients to
        the fragment positions across every pixel boundary where the triangle
        id changes, and from there to the geometry."""
        from .edge_gradient import EdgeGradientFn
        from .interpolator import polyfill_interpolate
        rast = self.rasterize()[0].squeeze(0)
        clip = self.clip_space()
        tris = self.vertex_array_object().tris
        frag = polyfill_interpolate(clip, rast, tris[float_to_triidx(rast[..., 3]) - 1], 1.0)
        frag_xy = frag[..., :2] / frag[..., 3:4]
        flat_tris_xy = (clip[..., :2] / clip[..., 3:4])[tris.long()]
        return torch.flipud(EdgeGradientFn.apply(frag_xy, flat_tris_xy, rast, torch.flipud(rgb)))
