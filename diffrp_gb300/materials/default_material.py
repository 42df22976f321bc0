"""Vertex-colour material (API of diffrp/materials/default_material.py:6-24)."""
from .base_material import SurfaceMaterial, SurfaceOutputStandard


class DefaultMaterial(SurfaceMaterial):
    """Albedo = interpolated vertex colour RGB, times an optional tint."""

    def __init__(self, tint=None):
        super().__init__()
        self.tint = tint

    def shade(self, su, si):
        rgb = si.color[..., :3]
        return SurfaceOutputStandard(rgb * self.tint if self.tint is not None else rgb)
