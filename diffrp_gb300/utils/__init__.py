from .cache import *  # noqa: F401,F403
from .composite import *  # noqa: F401,F403
from .geometry import *  # noqa: F401,F403
from .shader_ops import *  # noqa: F401,F403
