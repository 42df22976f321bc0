"""Seeded synthetic meshes, cameras and attribute sets for the benchmark
workloads and tests (numpy only).

The reference's configurations name meshes by construction (icospheres,
displaced grids, value-noise heightfields) and cameras by eye position; there
is no dataset, so these generators stand in for it.  GL matrices follow
diffrp's camera conventions (diffrp/rendering/camera.py:18-32, :80-108):
camera looks down -Z, +Y up, ``V`` is the inverse of the camera pose, ``P``
the OpenGL perspective projection with the principal point at the image
centre.
"""
import math

import numpy as np


# ---------------------------------------------------------------------------
# Meshes
# ---------------------------------------------------------------------------
def icosphere(subdivisions=3, radius=1.0):
    """Icosahedron subdivided ``subdivisions`` times, vertices on the sphere.
    CCW faces seen from outside.  3 -> 642 verts / 1280 faces,
    5 -> 10242 / 20480."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = np.array(verts, dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array(faces, dtype=np.int64)
    for _ in range(subdivisions):
        edges = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        lo = np.minimum(edges[:, 0], edges[:, 1])
        hi = np.maximum(edges[:, 0], edges[:, 1])
        key = lo * (len(v) + 1) + hi
        uniq, inv = np.unique(key, return_inverse=True)
        ulo = uniq // (len(v) + 1)
        uhi = uniq % (len(v) + 1)
        mid = v[ulo] + v[uhi]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        mid_idx = inv.reshape(3, -1).T + len(v)  # (F, 3): midpoints of edges 01, 12, 20
        v = np.concatenate([v, mid], axis=0)
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        ab, bc, ca = mid_idx[:, 0], mid_idx[:, 1], mid_idx[:, 2]
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1), np.stack([c, ca, bc], 1),
                            np.stack([ab, bc, ca], 1)], axis=0)
    return (v * radius).astype(np.float32), f.astype(np.int32)


def grid_mesh(n, extent=1.0):
    """n x n vertex grid on [-extent, extent]^2 in the XY plane (z = 0);
    2 (n-1)^2 CCW triangles."""
    xs = np.linspace(-extent, extent, n, dtype=np.float64)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    v = np.stack([X.ravel(), Y.ravel(), np.zeros(n * n)], axis=1)
    i = np.arange(n - 1)
    I, J = np.meshgrid(i, i, indexing="xy")
    a = (J * n + I).ravel()
    b = a + 1
    c = a + n
    d = c + 1
    f = np.concatenate([np.stack([a, b, d], 1), np.stack([a, d, c], 1)], axis=0)
    return v.astype(np.float32), f.astype(np.int32)


def value_noise(xy, octaves=6, seed=0, base_freq=2.0):
    """Seeded multi-octave value noise in [-1, 1]-ish at points xy (N, 2)."""
    rng = np.random.default_rng(seed)
    out = np.zeros(len(xy), dtype=np.float64)
    amp, freq, norm = 1.0, base_freq, 0.0
    for _ in range(octaves):
        size = int(math.ceil(freq * 2)) + 3
        lattice = rng.uniform(-1.0, 1.0, (size, size))
        p = (xy + 1.0) * 0.5 * freq + 1.0
        i0 = np.floor(p).astype(np.int64)
        fr = p - i0
        s = fr * fr * (3 - 2 * fr)
        x0, y0 = np.clip(i0[:, 0], 0, size - 2), np.clip(i0[:, 1], 0, size - 2)
        v00, v10 = lattice[y0, x0], lattice[y0, x0 + 1]
        v01, v11 = lattice[y0 + 1, x0], lattice[y0 + 1, x0 + 1]
        top = v00 + (v10 - v00) * s[:, 0]
        bot = v01 + (v11 - v01) * s[:, 0]
        out += amp * (top + (bot - top) * s[:, 1])
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return out / norm


def heightfield(n=1024, amplitude=0.3, octaves=6, seed=0):
    """n x n grid on [-1, 1]^2 with z from seeded value noise (amplitude)."""
    v, f = grid_mesh(n)
    v = v.astype(np.float64)
    v[:, 2] = amplitude * value_noise(v[:, :2], octaves=octaves, seed=seed)
    return v.astype(np.float32), f


def displaced_icosphere(subdivisions, radius, sigma, seed):
    v, f = icosphere(subdivisions, radius)
    rng = np.random.default_rng(seed)
    n = v / np.linalg.norm(v, axis=1, keepdims=True)
    v = v + n * rng.normal(0.0, sigma, (len(v), 1)).astype(np.float32)
    return v.astype(np.float32), f


def random_displaced_grid(n, seed, sigma=0.05):
    rng = np.random.default_rng(seed)
    v, f = grid_mesh(n)
    v = v.copy()
    v[:, 2] += rng.normal(0.0, sigma, len(v)).astype(np.float32)
    return v, f


def face_normals(v, f):
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    return n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-20)


# ---------------------------------------------------------------------------
# Cameras (GL conventions)
# ---------------------------------------------------------------------------
def perspective(fov_deg, h, w, near, far):
    """OpenGL projection for a vertical field of view, principal point at the
    image centre (diffrp/rendering/camera.py:80-88)."""
    f = 1.0 / math.tan(math.radians(fov_deg) / 2.0)
    P = np.zeros((4, 4), dtype=np.float64)
    P[0, 0] = f * h / w
    P[1, 1] = f
    P[2, 2] = -(far + near) / (far - near)
    P[2, 3] = -2.0 * far * near / (far - near)
    P[3, 2] = -1.0
    return P.astype(np.float32)


def lookat_pose(eye, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)):
    """Camera-to-world pose looking from ``eye`` at ``target``
    (diffrp/rendering/camera.py:96-108: z = -forward, x = forward x up,
    y = x x forward)."""
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    z = -fwd
    x = np.cross(fwd, np.asarray(up, np.float64))
    if np.linalg.norm(x) < 1e-12:
        x = np.cross(fwd, np.array([0.0, 0.0, 1.0]))
    y = np.cross(x, fwd)
    T = np.eye(4)
    T[:3, 0] = x / np.linalg.norm(x)
    T[:3, 1] = y / np.linalg.norm(y)
    T[:3, 2] = z / np.linalg.norm(z)
    T[:3, 3] = eye
    return T


def view_matrix(pose):
    return np.linalg.inv(pose).astype(np.float32)


def sphere_eyes(n, radius, seed):
    """n eye positions uniform on a sphere (seeded)."""
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return d * radius


def clip_positions(verts, mvp):
    """[verts, 1] @ mvp^T -> (V, 4) float32 (diffrp's transform_point)."""
    h = np.concatenate([verts.astype(np.float64), np.ones((len(verts), 1))], axis=1)
    return (h @ np.asarray(mvp, np.float64).T).astype(np.float32)
