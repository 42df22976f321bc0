from .objects import MeshObject  # noqa: F401
from .scene import Scene  # noqa: F401
