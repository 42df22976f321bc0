"""Scene container (API of diffrp/scene/scene.py:10-31)."""
from typing import List

__all__ = ["Scene"]


class Scene:
    """Objects (and lights, unused by the rasterisation path) of a render.
    ``add_*`` return the scene for chaining."""

    def __init__(self):
        self.lights: List = []
        self.objects: List = []
        self.metadata = {}

    def add_light(self, light):
        self.lights.append(light)
        return self

    def add_mesh_object(self, mesh_obj):
        self.objects.append(mesh_obj.preprocess())
        return self
