"""Texture-mapped material on the mip-mapped sampler (nvdr.texture).

diffrp's materials sample images with ``sample2d`` (bilinear, no mipmaps;
diffrp/utils/shader_ops.py:224, called from
diffrp/materials/gltf_material.py:47-48).  ``sample_texture`` keeps that
call's orientation -- uv (0, 0) at the bottom-left corner, the last image row
-- and adds mip-mapped filtering driven by the fragments' screen-space uv
derivatives (``SurfaceInput.uv_da``, from a session with
``derivatives=True``), so that minified textures are filtered instead of
aliased.  Without derivatives it samples bilinearly, as sample2d does.
"""
import weakref

import torch

from .. import nvdr as dr
from .base_material import SurfaceMaterial, SurfaceOutputStandard

__all__ = ["sample_texture", "TexturedMaterial", "PyramidCache"]

_WRAP = {"repeat": "wrap", "clamp": "clamp", "zero": "zero", "mirror": "mirror"}


class PyramidCache:
    """The mip pyramid of a material's fixed image, built on first use and
    rebuilt when the image is another tensor or was modified in place (its
    version counter moved).  A trained image (requires_grad) gets None:
    texture() then builds the pyramid inside autograd, so that gradients
    reach the image."""

    def __init__(self):
        self._ref, self._version, self._mip = None, None, None

    def get(self, image):
        if image.requires_grad:
            return None
        if self._ref is None or self._ref() is not image or self._version != image._version:
            self._mip = dr.texture_construct_mip(image[None].contiguous())
            self._ref, self._version = weakref.ref(image), image._version
        return self._mip


def sample_texture(image, uv, uv_da=None, wrap="repeat", filter_mode="auto", mip=None):
    """Sample ``image`` (H, W, C) at ``uv`` (..., 2), with (0, 0) at the
    bottom-left (diffrp's sample2d convention: image row (1 - v) H - 0.5);
    returns (..., C).

    ``uv_da`` (..., 4) = (du/dX, du/dY, dv/dX, dv/dY) selects the mip level
    (filter_mode 'auto': trilinear with derivatives, else bilinear).  wrap:
    'repeat', 'clamp' (to the edge, sample2d's 'border'), 'zero' or 'mirror'
    (mirrored repeat, sample2d's 'reflection').
    ``mip``: a dr.texture_construct_mip of ``image[None]``.
    """
    if wrap not in _WRAP:
        raise ValueError("wrap must be one of %s" % sorted(_WRAP))
    lead = uv.shape[:-1]
    uv_t = torch.stack([uv[..., 0], 1.0 - uv[..., 1]], -1).reshape(1, 1, -1, 2).contiguous()
    da_t = None
    if uv_da is not None:
        # v' = 1 - v: the v derivatives change sign
        da_t = torch.stack([uv_da[..., 0], uv_da[..., 1], -uv_da[..., 2], -uv_da[..., 3]], -1)
        da_t = da_t.reshape(1, 1, -1, 4).contiguous()
    tex = image[None].contiguous() if mip is None else mip.tex
    out = dr.texture(tex, uv_t, da_t, mip=mip, filter_mode=filter_mode, boundary_mode=_WRAP[wrap])
    return out.reshape(*lead, image.shape[-1])


class TexturedMaterial(SurfaceMaterial):
    """Albedo = base_color_factor x vertex colour x base_color_texture(uv),
    alpha from the texture's fourth channel when it has one.  The texture is
    sampled mip-mapped (trilinear) when the session provides derivatives,
    bilinearly otherwise."""

    def __init__(self, base_color_texture, base_color_factor=None, wrap="repeat"):
        super().__init__()
        self.image = base_color_texture
        self.factor = base_color_factor
        self.wrap = wrap
        self._pyramids = PyramidCache()

    def shade(self, su, si):
        try:
            uv_da = si.uv_da
        except RuntimeError:
            uv_da = None
        rgba = sample_texture(self.image, si.uv, uv_da, self.wrap, mip=self._pyramids.get(self.image) if uv_da is not None else None)
        rgb = rgba[..., :3] * si.color[..., :3]
        if self.factor is not None:
            rgb = rgb * self.factor[..., :3]
        alpha = rgba[..., 3:4] if rgba.shape[-1] > 3 else None
        return SurfaceOutputStandard(albedo=rgb, alpha=alpha)
