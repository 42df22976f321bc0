from .base_material import *  # noqa: F401,F403
from .default_material import DefaultMaterial  # noqa: F401
