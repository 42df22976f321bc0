from .base_material import *  # noqa: F401,F403
from .default_material import DefaultMaterial  # noqa: F401
from .textured_material import TexturedMaterial, sample_texture  # noqa: F401
from .gltf_material import GLTFMaterial, GLTFSampler  # noqa: F401
