"""Host-side logic on CPU: scene preprocessing, the vertex array object and
the camera matrices reproduce the reference session's clip-space vertices
stored in the golden vectors; cache / swizzle / options semantics."""
import os

import numpy as np
import pytest
import torch

from diffrp_gb300 import synthetic as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden(name):
    z = np.load(os.path.join(GOLDEN, "session_%s.npz" % name))
    return {k: z[k] for k in z.files}


class _Mat:
    def shade(self, su, si):  # never called on CPU
        raise AssertionError


def _vao_clip(scene, P, V):
    from diffrp_gb300.rendering.mixin import RenderSessionMixin

    class _S(RenderSessionMixin):
        pass

    s = _S()
    s.scene = scene
    vao = s.vertex_array_object()
    wp = vao.world_pos.double().numpy()
    return (np.concatenate([wp, np.ones((len(wp), 1))], 1) @ (P.astype(np.float64) @ V.astype(np.float64)).T), vao


def test_face_soup_vao_and_camera_reproduce_reference_clip():
    from diffrp_gb300.scene import MeshObject, Scene
    g = _golden("normals")
    verts = torch.from_numpy(g["in_verts"])
    tris = torch.from_numpy(g["in_tris"])
    scene = Scene().add_mesh_object(MeshObject(_Mat(), verts, tris))
    obj = scene.objects[0]
    F = len(g["in_tris"])
    assert obj.verts.shape == (3 * F, 3) and obj.tris.shape == (F, 3)
    np.testing.assert_array_equal(obj.tris.numpy(), np.arange(3 * F).reshape(F, 3))
    h, w = int(g["in_h"]), int(g["in_w"])
    P = S.perspective(float(g["in_fov"]), h, w, float(g["in_near"]), float(g["in_far"]))
    V = S.view_matrix(np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 3.2], [0, 0, 0, 1.0]]))
    clip, vao = _vao_clip(scene, P, V)
    np.testing.assert_allclose(clip, g["out_clip"], rtol=2e-6, atol=2e-6)
    assert vao.stencils.tolist() == [0] + [1] * F


def test_two_objects_vao_and_lookat_reproduce_reference_clip():
    from diffrp_gb300.scene import MeshObject, Scene
    g = _golden("objects_masked")
    t = torch.from_numpy
    scene = Scene()
    scene.add_mesh_object(MeshObject(_Mat(), t(g["in_v1"]), t(g["in_f1"]), normals="smooth", M=t(g["in_M1"]),
                                     color=t(g["in_c1"])))
    scene.add_mesh_object(MeshObject(_Mat(), t(g["in_v2"]), t(g["in_f2"]), M=t(g["in_M2"]),
                                     custom_attrs={"feat": t(g["in_feat2"])}))
    h, w = int(g["in_h"]), int(g["in_w"])
    P = S.perspective(float(g["in_fov"]), h, w, float(g["in_near"]), float(g["in_far"]))
    V = S.view_matrix(S.lookat_pose(g["in_eye"], (0.0, 0.0, 0.0)))
    clip, vao = _vao_clip(scene, P, V)
    np.testing.assert_allclose(clip, g["out_clip"], rtol=2e-6, atol=2e-6)
    # stencils: background, object 1 triangles, object 2 triangles
    n1, n2 = len(g["in_f1"]), len(g["in_f2"])
    assert vao.stencils.tolist() == [0] + [1] * n1 + [2] * n2
    # object 1 has no "feat": zero-filled custom attribute of the shared width
    assert vao.custom_attrs["feat"].shape[1] == 5
    assert float(vao.custom_attrs["feat"][: len(g["in_v1"])].abs().sum()) == 0.0


def test_cache_decorators():
    from diffrp_gb300.utils.cache import cached, key_cached, singleton_cached
    calls = []

    class A:
        @cached
        def f(self):
            calls.append(1)
            return len(calls)

        @key_cached
        def g(self, k):
            calls.append(k)
            return k * 2

    a = A()
    assert a.f() == 1 and a.f() == 1 and a.g(3) == 6 and a.g(3) == 6
    assert calls == [1, 3]
    assert A().f() == 3  # a new instance recomputes

    @singleton_cached
    def h():
        calls.append("h")
        return object()

    assert h() is h() and calls.count("h") == 1


def test_swizzles_and_options():
    from diffrp_gb300.rendering.surface_deferred import SurfaceDeferredRenderSessionOptions
    x = torch.arange(8.0).reshape(2, 4)
    assert x.xyz.shape == (2, 3) and x.a.shape == (2, 1)
    assert x.zx.tolist() == [[2.0, 0.0], [6.0, 4.0]]
    assert x.rgba.tolist() == x.tolist()
    assert SurfaceDeferredRenderSessionOptions().max_layers == 32767
    assert SurfaceDeferredRenderSessionOptions(max_layers=3).max_layers == 3


def test_camera_conventions():
    P = S.perspective(30.0, 512, 512, 0.1, 100.0)
    # a point on the near plane maps to z/w = -1, far plane to +1
    for zc, expect in [(-0.1, -1.0), (-100.0, 1.0)]:
        c = P.astype(np.float64) @ np.array([0.0, 0.0, zc, 1.0])
        assert abs(c[2] / c[3] - expect) < 1e-5
    pose = S.lookat_pose((0.0, 0.0, 3.2))
    np.testing.assert_allclose(pose, np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 3.2], [0, 0, 0, 1.0]]),
                               atol=1e-12)


def test_drop_in_bin_depth_sizing_host_logic():
    """The drop-in context's choice of fixed-depth bins per call shape and
    their growth after an overflow (host logic, no device)."""
    from diffrp_gb300.nvdr import RasterizeCudaContext
    ctx = RasterizeCudaContext.__new__(RasterizeCudaContext)
    ctx._depth, ctx._capacity, ctx.last_list_entries = {}, 0, 0
    shape = (1, 20480, 1024, 1024, 5)  # 1024 tiles of 32 x 32
    assert ctx._choose_depth(shape, 100, 60000) == 133  # 1.25 x largest + 8
    assert ctx._choose_depth(shape, 10 ** 6, 60000) == 0  # bins far beyond the exact lists: keep exact
    ctx._note_stats(shape, 0, 60000, 0, 100)  # an exact-list call: capacity and the shape's depth
    assert ctx._capacity == int(60000 * 1.25) + 1024 and ctx._depth[shape] == 133
    ctx._note_stats(shape, 133, 0, 2, 400)  # a bin overflowed: deeper bins for the next call
    assert ctx._depth[shape] == max(int(133 * 1.5), int(400 * 1.25) + 8)
    ctx._note_stats(shape, 508, 0, 0, 10)  # no overflow: unchanged
    assert ctx._depth[shape] == 508


def test_batch_bin_depth_choice_host_logic():
    from diffrp_gb300.batch import BatchRenderer
    r = BatchRenderer.__new__(BatchRenderer)
    r.bin_depth_mode, r.total_tiles = None, 4096
    assert r._choose_depth(50, 100000) == int(50 * 1.25) + 8
    assert r._choose_depth(5000, 1000) == 0
    r.bin_depth_mode = 7  # a caller-fixed depth wins
    assert r._choose_depth(5000, 1000) == 7


@pytest.mark.parametrize("n_objects", [1, 2, 5, 9])
def test_stencil_groups_match_per_object_nonzero(n_objects):
    """The per-layer grouping of pixels by stencil (one sort, one count
    read-back) gives each object exactly mask.nonzero's index tuple."""
    import torch
    from diffrp_gb300.rendering.interpolator import stencil_groups
    g = torch.Generator().manual_seed(n_objects)
    st = torch.randint(0, n_objects + 2, (1, 41, 67), generator=g, dtype=torch.int32)
    st[st == 3] = 0  # an object with no pixels
    groups = stencil_groups(st, n_objects)
    assert len(groups) == n_objects
    for k in range(n_objects):
        ref = (st == k + 1).nonzero(as_tuple=True)
        assert len(groups[k]) == 3
        for a, b in zip(groups[k], ref):
            assert a.dtype == b.dtype and torch.equal(a, b)


def test_masked_sparse_interpolator_from_mask_and_from_indices():
    """The stencil-masked interpolator built from a mask and from the
    precomputed index tuple holds the same pixels, rows and triangles."""
    from diffrp_gb300.rendering.interpolator import MaskedSparseInterpolator, stencil_groups
    g = torch.Generator().manual_seed(3)
    rast = torch.rand(1, 9, 11, 4, generator=g)
    ids = torch.randint(0, 5, (1, 9, 11), generator=g)
    rast[..., 3] = ids.float()
    tris = torch.arange(12, dtype=torch.int32).reshape(4, 3)
    stencil = (ids > 2).int() * 2 + (ids > 0).int()
    a = MaskedSparseInterpolator(rast, tris, stencil == 1)
    b = MaskedSparseInterpolator(rast, tris, None, indices=stencil_groups(stencil, 3)[0])
    for x, y in zip(a.indices, b.indices):
        assert torch.equal(x, y)
    assert torch.equal(a.vi_data, b.vi_data) and torch.equal(a.tri_idx, b.tri_idx)
