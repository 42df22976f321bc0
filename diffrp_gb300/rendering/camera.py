"""Cameras (API of diffrp/rendering/camera.py:10-137), self-contained numpy
maths in place of the trimesh / calibur helpers the reference uses."""
import math

import numpy
import torch

from .. import synthetic
from ..utils.shader_ops import gpu_f32

__all__ = ["Camera", "RawCamera", "PerspectiveCamera"]


def _translation(t):
    m = numpy.eye(4)
    m[:3, 3] = t
    return m


def _device_matrix(cam, name, m):
    """The GPU copy of a camera matrix, kept on the camera while its value
    stays the same: a render step then copies nothing from the host once the
    camera has been used (which also lets the step be captured in a CUDA
    graph).  The returned tensor is shared; do not modify it in place."""
    m = numpy.ascontiguousarray(m, dtype=numpy.float32)
    cache = cam.__dict__.setdefault("_matrix_cache", {})
    hit = cache.get(name)
    dev = torch.cuda.current_device()
    if hit is not None and hit[0] == dev and numpy.array_equal(hit[1], m):
        return hit[2]
    t = gpu_f32(m)
    cache[name] = (dev, m, t)
    return t


class Camera:
    """Abstract camera: ``V()`` (GL view, inverse pose), ``P()`` (GL
    projection) and ``resolution()`` (h, w).  The default pose sits at
    (0, 0, 3.2) looking down -Z."""

    def __init__(self):
        self.t = _translation([0.0, 0.0, 3.2])

    def V(self):
        return _device_matrix(self, "V", numpy.linalg.inv(numpy.asarray(self.t)).astype(numpy.float32))

    def P(self):
        raise NotImplementedError

    def resolution(self):
        raise NotImplementedError


class RawCamera(Camera):
    """Camera driven by given V and P tensors."""

    def __init__(self, h, w, v, p):
        self.h, self.w, self.v, self.p = h, w, v, p

    def V(self):
        return self.v

    def P(self):
        return self.p

    def resolution(self):
        return self.h, self.w


class PerspectiveCamera(Camera):
    """Perspective camera; ``fov`` is the vertical field of view in degrees."""

    def __init__(self, fov=30, h=512, w=512, near=0.1, far=10.0):
        super().__init__()
        self.fov, self.h, self.w, self.near, self.far = fov, h, w, near, far

    def P(self):
        return _device_matrix(self, "P", synthetic.perspective(self.fov, self.h, self.w, self.near, self.far))

    def resolution(self):
        return self.h, self.w

    def set_transform(self, tr):
        self.t = tr

    def lookat(self, point):
        point = numpy.asarray(point, dtype=numpy.float64)
        if point.shape != (3,):
            raise ValueError("lookat expects a 3-vector")
        self.t = synthetic.lookat_pose(self.t[:3, 3].copy(), point)
        return self

    @classmethod
    def from_orbit(cls, h, w, radius, azim, elev, origin, fov=30, near=0.1, far=10.0):
        """Orbit camera: azimuth from +Z, elevation in degrees, looking at origin."""
        cam = cls(h=h, w=w, fov=fov, near=near, far=far)
        th, ph = math.radians(azim), math.radians(elev)
        eye = [radius * math.sin(th) * math.cos(ph) + origin[0], radius * math.sin(ph) + origin[1],
               radius * math.cos(th) * math.cos(ph) + origin[2]]
        cam.t = _translation(eye)
        cam.lookat(origin)
        return cam
