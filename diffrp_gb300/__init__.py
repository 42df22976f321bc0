"""diffrp_gb300 -- GB300 (sm_103a) implementation of diffrp's differentiable
rasterisation hot path: rasterize -> interpolate -> antialias (forward and
backward) behind diffrp's Scene / MeshObject / PerspectiveCamera /
SurfaceDeferredRenderSession API.

``diffrp_gb300.nvdr`` is the drop-in for the ``nvdiffrast.torch`` module diffrp
imports; the kernels live in ``libdiffrp_gb300.so`` (C ABI:
``include/diffrp_gb300.h``).
"""
__version__ = "0.1.0"
