"""glTF 2.0 PBR material on the mip-mapped sampler.

The reference's ``GLTFMaterial`` (diffrp/materials/gltf_material.py:25-67)
and ``GLTFSampler`` (:9-22) with the same fields and outputs.  Every texture
is read through ``GLTFSampler.sample``:

* without derivatives it gives sample2d's results (bilinear or point samples
  of the image; diffrp/utils/shader_ops.py:199-255);
* with the fragments' uv derivatives (``SurfaceInput.uv_da``, from a session
  with ``derivatives=True``) a 'linear' sampler filters trilinearly from the
  image's mip pyramid, so that minified textures are filtered instead of
  aliased.
"""
from dataclasses import dataclass, field
from typing import Literal, Optional

import torch

from ..utils.shader_ops import fsa, ones_like_vec
from .base_material import SurfaceMaterial, SurfaceOutputStandard
from .textured_material import PyramidCache, sample_texture

__all__ = ["GLTFSampler", "GLTFMaterial"]


@dataclass
class GLTFSampler:
    """A texture image (H, W, 1 | 3 | 4) with its wrap and filter modes.

    wrap_mode 'repeat' takes uv modulo 1 and mirrors the bilinear taps at the
    image's edges, as the reference does (``uv.remainder(1.0)`` then
    sample2d's 'reflection' padding); 'clamp' clamps to the edge texels
    (sample2d's 'border'); 'mirror' repeats the image mirrored.
    interpolation 'point' takes the nearest texel; 'linear' samples
    bilinearly, or trilinearly when derivatives are given.
    """
    image: torch.Tensor
    wrap_mode: Literal['repeat', 'clamp', 'mirror'] = 'repeat'
    interpolation: Literal['point', 'linear'] = 'linear'
    _pyramids: PyramidCache = field(default_factory=PyramidCache, init=False, repr=False, compare=False)

    def sample(self, uv: torch.Tensor, uv_da: Optional[torch.Tensor] = None) -> torch.Tensor:
        """(..., C) at uv (..., 2), (0, 0) at the image's bottom-left corner;
        uv_da (..., 4) = (du/dX, du/dY, dv/dX, dv/dY) or None."""
        if self.wrap_mode not in ('repeat', 'clamp', 'mirror'):
            raise ValueError('bad GLTFSampler.wrap_mode', self.wrap_mode)
        if self.interpolation not in ('point', 'linear'):
            raise ValueError('bad GLTFSampler.interpolation', self.interpolation)
        if self.wrap_mode == 'repeat':
            uv = uv.remainder(1.0)
        wrap = 'clamp' if self.wrap_mode == 'clamp' else 'mirror'
        if self.interpolation == 'point':
            return sample_texture(self.image, uv, None, wrap, filter_mode='nearest')
        if uv_da is None:
            return sample_texture(self.image, uv, None, wrap, filter_mode='linear')
        return sample_texture(self.image, uv, uv_da, wrap, filter_mode='linear-mipmap-linear', mip=self._pyramids.get(self.image))


@dataclass
class GLTFMaterial(SurfaceMaterial):
    """A standard PBR material following the glTF 2.0 specification: the
    reference's fields and outputs, textures through ``GLTFSampler``."""
    base_color_factor: torch.Tensor  # (4,)
    base_color_texture: GLTFSampler

    metallic_factor: float
    roughness_factor: float
    metallic_roughness_texture: GLTFSampler

    normal_texture: Optional[GLTFSampler]
    occlusion_texture: Optional[GLTFSampler]

    emissive_factor: Optional[torch.Tensor]  # (3,)
    emissive_texture: GLTFSampler

    alpha_cutoff: float
    alpha_mode: Literal['OPAQUE', 'MASK', 'BLEND']

    def shade(self, su, si) -> SurfaceOutputStandard:
        try:
            da = si.uv_da
        except RuntimeError:  # a session without derivatives
            da = None
        uv = si.uv
        rgba = self.base_color_factor * si.color * self.base_color_texture.sample(uv, da)
        mr = self.metallic_roughness_texture.sample(uv, da)
        if self.alpha_mode == 'OPAQUE':
            alpha = None
        elif self.alpha_mode == 'MASK':
            alpha = (rgba.a > self.alpha_cutoff).float()
        elif self.alpha_mode == 'BLEND':
            alpha = rgba.a
        else:
            raise ValueError('bad GLTFMaterial.alpha_mode', self.alpha_mode)
        return SurfaceOutputStandard(
            rgba.rgb,
            fsa(2, self.normal_texture.sample(uv, da), -1) if self.normal_texture is not None else None,
            self.emissive_factor * self.emissive_texture.sample(uv, da) if self.emissive_factor is not None else None,
            self.metallic_factor * mr.b,
            fsa(-self.roughness_factor, mr.g, 1.0),
            self.occlusion_texture.sample(uv, da).r if self.occlusion_texture is not None else ones_like_vec(uv, 1),
            alpha,
        )
