"""Mesh object of a scene (API of diffrp/scene/objects.py:12-98)."""
from dataclasses import dataclass
from typing import Any, Dict, Optional, Union

import torch

from ..utils.geometry import compute_face_normals, compute_vertex_normals, make_face_soup
from ..utils.shader_ops import ones_like_vec, zeros_like_vec


@dataclass
class MeshObject:
    """A triangle mesh with a material.

    ``verts`` (V, 3) float32, ``tris`` (F, 3) int32 on the GPU; ``normals`` a
    (V, 3) tensor or 'flat' (default) / 'smooth'; ``M`` the 4x4 model matrix
    (identity); ``color`` (V, 4) linear RGBA (ones); ``uv`` (V, 2) (zeros);
    ``tangents`` (V, 4) (zeros); ``custom_attrs`` name -> (V, C).

    ``preprocess`` fills the defaults.  'flat' normals turn the mesh into a
    face soup (3F unshared vertices, each corner carrying its face normal)
    and gather every vertex attribute accordingly, which is what lets flat
    shading go through plain vertex interpolation.
    """
    material: Any
    verts: torch.Tensor
    tris: torch.Tensor
    normals: Union[str, torch.Tensor] = "flat"
    M: Optional[torch.Tensor] = None
    color: Optional[torch.Tensor] = None
    uv: Optional[torch.Tensor] = None
    tangents: Optional[torch.Tensor] = None
    custom_attrs: Optional[Dict[str, torch.Tensor]] = None
    metadata: Optional[Dict[str, Any]] = None

    def preprocess(self):
        v = self.verts
        if self.M is None:
            self.M = torch.eye(4, device=v.device, dtype=v.dtype)
        if self.color is None:
            self.color = ones_like_vec(v, 4)
        if self.uv is None:
            self.uv = zeros_like_vec(v, 2)
        if self.tangents is None:
            self.tangents = zeros_like_vec(v, 4)
        if self.custom_attrs is None:
            self.custom_attrs = {}
        if self.metadata is None:
            self.metadata = {}
        if isinstance(self.normals, str):
            mode = self.normals
            if mode == "smooth":
                self.normals = compute_vertex_normals(self.verts, self.tris)
            elif mode == "flat":
                corners = self.tris.long()
                fn = compute_face_normals(self.verts, self.tris, normalize=True)
                self.verts, self.tris, self.normals = make_face_soup(self.verts, self.tris, fn)

                def soup(a):
                    return a[corners].flatten(0, 1)

                self.color = soup(self.color)
                self.uv = soup(self.uv)
                self.tangents = soup(self.tangents)
                self.custom_attrs = {k: soup(a) for k, a in self.custom_attrs.items()}
            else:
                raise ValueError("normals must be a tensor, 'flat' or 'smooth', got %r" % mode)
        return self
