"""Seeded test scenes in clip space (numpy), shared by CPU and GPU tests."""
import numpy as np

from diffrp_gb300 import synthetic as S


def random_soup(n_tris, seed, depth_range=(-0.6, 0.6), w_range=(0.7, 1.6), xy=0.9):
    """Random triangles with perspective w, all inside the view volume."""
    rng = np.random.default_rng(seed)
    V = 3 * n_tris
    pos = np.zeros((V, 4), np.float64)
    centers = rng.uniform(-xy, xy, (n_tris, 2))
    sizes = rng.uniform(0.05, 0.6, n_tris)
    off = rng.normal(size=(n_tris, 3, 2)) * sizes[:, None, None]
    pos[:, 0:2] = (centers[:, None, :] + off).reshape(-1, 2)
    pos[:, 2] = rng.uniform(*depth_range, V)
    pos[:, 3] = rng.uniform(*w_range, V)
    pos[:, 0:3] *= pos[:, 3:4]
    tri = np.arange(V, dtype=np.int32).reshape(-1, 3)
    return pos.astype(np.float32), tri


def sphere_view(subdiv=3, radius=0.8, res=(64, 64), eye=(0.0, 0.0, 3.2), fov=30.0, far=100.0, sigma=0.0, seed=0):
    """Icosphere (optionally displaced) seen from ``eye``: (clip pos (V,4), tri)."""
    if sigma:
        v, f = S.displaced_icosphere(subdiv, radius, sigma, seed)
    else:
        v, f = S.icosphere(subdiv, radius)
    P = S.perspective(fov, res[0], res[1], 0.1, far)
    V = S.view_matrix(S.lookat_pose(eye))
    return S.clip_positions(v, P.astype(np.float64) @ V.astype(np.float64)), f


def multi_view(subdiv=2, n_views=4, res=(48, 48), seed=1):
    v, f = S.icosphere(subdiv, 0.8)
    P = S.perspective(30.0, res[0], res[1], 0.1, 100.0).astype(np.float64)
    eyes = S.sphere_eyes(n_views, 3.2, seed)
    pos = np.stack([S.clip_positions(v, P @ S.view_matrix(S.lookat_pose(e)).astype(np.float64)) for e in eyes])
    return pos, f


def near_crossing(seed=3):
    """Triangles straddling the near plane and far outside the guard band."""
    rng = np.random.default_rng(seed)
    P = S.perspective(60.0, 32, 32, 0.1, 10.0).astype(np.float64)
    tris = []
    for _ in range(12):
        a = np.array([rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(-3, -0.5)])
        b = np.array([rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(-0.05, 0.5)])
        c = np.array([rng.uniform(-40, 40), rng.uniform(-1, 1), rng.uniform(-4, -0.02)])
        tris.append([a, b, c])
    v = np.array(tris, np.float64).reshape(-1, 3)
    pos = S.clip_positions(v, P)
    return pos, np.arange(len(v), dtype=np.int32).reshape(-1, 3)
