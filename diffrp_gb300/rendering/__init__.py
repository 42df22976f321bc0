from .camera import Camera, PerspectiveCamera, RawCamera  # noqa: F401
from .interpolator import (FullScreenInterpolator, Interpolator, MaskedSparseInterpolator,  # noqa: F401
                           polyfill_interpolate)
from .mixin import RenderSessionMixin  # noqa: F401
from .surface_deferred import SurfaceDeferredRenderSession, SurfaceDeferredRenderSessionOptions  # noqa: F401
