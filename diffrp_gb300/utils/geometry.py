"""Mesh helpers on the preprocessing path (semantics of
diffrp/utils/geometry.py:5-91)."""
import torch

from .shader_ops import cross, normalized

__all__ = ["make_face_soup", "compute_face_normals", "compute_vertex_normals", "sign2d", "point_in_tri2d"]


def make_face_soup(verts, tris, face_normals):
    """Unshare vertices: 3F vertices, tris = arange(3F).reshape(F, 3), per-face
    normals repeated on the three corners."""
    soup_verts = verts[tris].reshape(-1, 3)
    soup_tris = torch.arange(tris.numel(), device=tris.device, dtype=torch.int32).reshape(tris.shape)
    soup_normals = face_normals[:, None, :].expand(-1, 3, -1).reshape(-1, 3)
    return soup_verts, soup_tris, soup_normals


def compute_face_normals(verts, faces, normalize=False):
    """(v1 - v0) x (v2 - v0) per face (CCW winding)."""
    f = faces.long()
    n = cross(verts[f[:, 1]] - verts[f[:, 0]], verts[f[:, 2]] - verts[f[:, 0]])
    return normalized(n) if normalize else n


def compute_vertex_normals(verts, faces):
    """Area-weighted vertex normals, normalised."""
    f = faces.long()
    fn = compute_face_normals(verts, faces)
    vn = torch.zeros_like(verts)
    for k in range(3):
        vn = vn.index_add(0, f[:, k], fn)
    return normalized(vn)


def sign2d(p1, p2, p3):
    return (p1[..., 0:1] - p3[..., 0:1]) * (p2[..., 1:2] - p3[..., 1:2]) - \
        (p2[..., 0:1] - p3[..., 0:1]) * (p1[..., 1:2] - p3[..., 1:2])


def point_in_tri2d(pt, v1, v2, v3):
    """True where pt lies inside or on triangle (v1, v2, v3); (..., 1)."""
    d1, d2, d3 = sign2d(pt, v1, v2), sign2d(pt, v2, v3), sign2d(pt, v3, v1)
    neg = (d1 < 0) | (d2 < 0) | (d3 < 0)
    pos = (d1 > 0) | (d2 > 0) | (d3 > 0)
    return ~(neg & pos)
