"""The CPU oracle against known answers and finite differences.

The oracle's own correctness is what the GPU parity tests lean on, so it is
pinned here: coverage counts of exactly representable triangles, the fill
rule on shared edges, depth-tie resolution, the tri-id encoding of
diffrp/rendering/interpolator.py:24-29, the interpolation formula of
interpolator.py:39-45, and FP64 central differences for every backward.
"""
import numpy as np
import pytest

import oracle as O
from tests import scenes


def test_single_triangle_area_and_barycentrics():
    pos = np.array([[-0.5, -0.5, 0, 1], [0.5, -0.5, 0, 1], [0, 0.5, 0, 1]], np.float32)
    tri = np.array([[0, 1, 2]], np.int32)
    rast, db, _ = O.rasterize(pos, tri, (16, 16))
    assert (rast[..., 3] > 0).sum() == 32  # 8 px base x 8 px height / 2
    # pixel (8, 8): centre (1/16, 1/16) in NDC = u v0 + v v1 + (1-u-v) v2
    np.testing.assert_allclose(rast[0, 8, 8], [0.15625, 0.28125, 0.0, 1.0])
    np.testing.assert_allclose(db[0, 8, 8], [-0.125, -0.0625, 0.125, -0.0625])


def test_shared_edges_cover_each_pixel_once():
    # 4x4 grid of quads, each split in two, covering NDC [-0.75, 0.75]^2
    n = 5
    xs = np.linspace(-0.75, 0.75, n)
    X, Y = np.meshgrid(xs, xs)
    v = np.stack([X.ravel(), Y.ravel(), np.zeros(n * n), np.ones(n * n)], 1).astype(np.float32)
    faces = []
    for j in range(n - 1):
        for i in range(n - 1):
            a, b, c, d = j * n + i, j * n + i + 1, (j + 1) * n + i, (j + 1) * n + i + 1
            faces += [[a, b, d], [a, d, c]]
    tri = np.array(faces, np.int32)
    for res in [(32, 32), (37, 29)]:
        key = O.raster_ids(v, tri, res)
        # count coverage per pixel by rasterising each triangle alone
        cover = np.zeros(res, np.int32)
        for t in range(len(tri)):
            k = O.raster_ids(v, tri[t:t + 1], res)
            cover += (k[0] != np.uint64(0xFFFFFFFFFFFFFFFF))
        assert cover.max() == 1
        inside = O.key_tri(key[0]) >= 0
        np.testing.assert_array_equal(inside, cover == 1)


def test_depth_tie_lower_index_wins_and_peeling_order():
    pos = np.array([[-0.5, -0.5, 0.2, 1], [0.5, -0.5, 0.2, 1], [0, 0.5, 0.2, 1]], np.float32)
    pos2 = np.concatenate([pos, pos])
    tri = np.array([[3, 4, 5], [0, 1, 2]], np.int32)
    key = O.raster_ids(pos2, tri, (16, 16))
    ids = O.key_tri(key[0])
    assert set(np.unique(ids)) == {-1, 0}
    key2 = O.raster_ids(pos2, tri, (16, 16), prev_key=key)
    assert set(np.unique(O.key_tri(key2[0]))) == {-1, 1}
    key3 = O.raster_ids(pos2, tri, (16, 16), prev_key=key2)
    assert (O.key_tri(key3[0]) == -1).all()


def test_nearest_surface_wins():
    near = [[-0.8, -0.8, -0.5, 1], [0.8, -0.8, -0.5, 1], [0, 0.8, -0.5, 1]]
    far = [[-0.8, -0.8, 0.5, 1], [0.8, -0.8, 0.5, 1], [0, 0.8, 0.5, 1]]
    pos = np.array(far + near, np.float32)
    tri = np.array([[0, 1, 2], [3, 4, 5]], np.int32)
    rast, _, _ = O.rasterize(pos, tri, (8, 8))
    ids = rast[..., 3][rast[..., 3] > 0]
    assert (ids == 2).all()
    np.testing.assert_allclose(rast[..., 2][rast[..., 3] > 0], -0.5, atol=1e-6)


@pytest.mark.parametrize("t", [1, 2, 100, 0x00FFFFFF, 0x01000000, 0x01000001, 0x02345678, 0x34FFFFFF])
def test_triid_encoding_round_trip(t):
    f = O.triidx_to_float(np.array([t]))[0]
    assert O.float_to_triidx(np.array([f]))[0] == t
    if t <= 1 << 24:
        assert f == np.float32(t)
    else:
        assert np.array([f], np.float32).view(np.int32)[0] == 0x4A800000 + t


def test_triid_encoding_matches_torch_mirror():
    import torch
    from diffrp_gb300.rendering.interpolator import float_to_triidx, triidx_to_float
    ids = torch.tensor([1, 77, 1 << 24, (1 << 24) + 1, 123456789], dtype=torch.int32)
    f = triidx_to_float(ids)
    np.testing.assert_array_equal(f.numpy(), O.triidx_to_float(ids.numpy()))
    np.testing.assert_array_equal(float_to_triidx(f).numpy(), ids.numpy())


def test_near_plane_clipping_consistent():
    pos, tri = scenes.near_crossing()
    rast, _, key = O.rasterize(pos, tri, (32, 32))
    cov = rast[..., 3] > 0
    assert cov.sum() > 0
    z = rast[..., 2][cov]
    assert np.isfinite(z).all()


def test_interpolation_formula():
    pos, tri = scenes.sphere_view(2, res=(24, 24))
    rng = np.random.default_rng(0)
    attr = rng.normal(size=(len(pos), 3)).astype(np.float32)
    rast, _, _ = O.rasterize(pos, tri, (24, 24))
    out, _ = O.interpolate(attr, rast, tri)
    m = rast[..., 3] > 0
    t = rast[..., 3][m].astype(np.int64) - 1
    u, v = rast[..., 0][m], rast[..., 1][m]
    a0, a1, a2 = attr[tri[t, 0]], attr[tri[t, 1]], attr[tri[t, 2]]
    ref = (a0 - a2) * u[:, None] + ((a1 - a2) * v[:, None] + a2)
    np.testing.assert_allclose(out[m], ref, rtol=1e-6, atol=1e-6)
    assert (out[~m] == 0).all()


def test_topology_closed_mesh_and_soup():
    _, f = scenes.sphere_view(2, res=(8, 8))
    nbr = O.topology(f)
    assert (nbr >= 0).all()
    # symmetric: t's neighbour across edge k has t as a neighbour
    for t in range(0, len(f), 7):
        for k in range(3):
            assert t in nbr[nbr[t, k]]
    soup = np.arange(30, dtype=np.int32).reshape(10, 3)
    assert (O.topology(soup) == -1).all()


def _fd(fn, x, eps=1e-6):
    g = np.zeros_like(x)
    for idx in np.ndindex(x.shape):
        xp = x.copy()
        xp[idx] += eps
        xm = x.copy()
        xm[idx] -= eps
        g[idx] = (fn(xp) - fn(xm)) / (2 * eps)
    return g


def _small_scene(seed=0):
    rng = np.random.default_rng(seed)
    pos, tri = scenes.random_soup(5, seed=seed)
    return pos.astype(np.float64), tri, rng


def test_fd_raster_bwd():
    pos, tri, rng = _small_scene(1)
    res = (20, 20)
    rast, db, key = O.rasterize(pos, tri, res, precision="f64")
    gr = rng.normal(size=rast.shape)
    gr[..., 3] = 0
    gdb = rng.normal(size=db.shape)

    def loss(p):
        r, d, _ = O.rasterize(p, tri, res, precision="f64", key=key)
        return (r[..., :3] * gr[..., :3]).sum() + (d * gdb).sum()

    g = O.raster_bwd(pos, tri, rast, gr, gdb)
    fd = _fd(loss, pos)
    assert np.abs(g - fd).max() <= 1e-5 * max(1.0, np.abs(fd).max())


def test_fd_interpolate_bwd():
    pos, tri, rng = _small_scene(2)
    res = (20, 20)
    rast, db, _ = O.rasterize(pos, tri, res, precision="f64")
    attr = rng.normal(size=(len(pos), 3))
    go = rng.normal(size=(1, 20, 20, 3))
    gda = rng.normal(size=(1, 20, 20, 6))

    def loss(a):
        o, d = O.interpolate(a, rast, tri, db, diff_attrs="all", precision="f64")
        return (o * go).sum() + (d * gda).sum()

    ga, gr, gd = O.interpolate_bwd(attr, rast, tri, go, db, "all", gda)
    assert np.abs(ga - _fd(loss, attr)).max() < 1e-6


def test_fd_antialias_bwd():
    pos, tri, rng = _small_scene(3)
    res = (20, 20)
    rast, _, _ = O.rasterize(pos, tri, res, precision="f64")
    col = rng.normal(size=(1, 20, 20, 2))
    go = rng.normal(size=col.shape)
    nbr = O.topology(tri)

    def loss_p(p):
        return (O.antialias(col, rast, p, tri, nbr, precision="f64") * go).sum()

    def loss_c(c):
        return (O.antialias(c, rast, pos, tri, nbr, precision="f64") * go).sum()

    gc, gp = O.antialias_bwd(col, rast, pos, tri, go, nbr)
    fdp = _fd(loss_p, pos)
    assert np.abs(gp - fdp).max() <= 1e-5 * max(1.0, np.abs(fdp).max())
    assert np.abs(gc - _fd(loss_c, col)).max() < 1e-6


def test_backward_precision_f32_terms_match_f64():
    """The oracle's float32-term backward (used to mirror the CUDA path's
    branches at full size) stays within float32 rounding of the float64
    one on a small scene."""
    from tests import scenes
    pos, tri = scenes.sphere_view(3, res=(48, 48), sigma=0.03, seed=6)
    rng = np.random.default_rng(6)
    rast, _, _ = O.rasterize(pos, tri, (48, 48), grad_db=False)
    color = rng.uniform(0, 1, (1, 48, 48, 3)).astype(np.float32)
    go = rng.normal(size=(1, 48, 48, 3)).astype(np.float32)
    out = {}
    for prec in ("f32", "f64"):
        gc, gp = O.antialias_bwd(color, rast, pos, tri, go, precision=prec)
        ga, gr, _ = O.interpolate_bwd(color[0, :1, :1].reshape(1, 3).repeat(len(pos), 0), rast, tri, gc,
                                      precision=prec)
        out[prec] = (gp + O.raster_bwd(pos, tri, rast, gr, precision=prec), ga)
    for a, b in zip(out["f32"], out["f64"]):
        assert np.abs(a - b).max() <= 1e-4 * np.abs(b).max()


def test_fixed_visibility_l1_matches_forward_and_backward():
    """The fixed-decision float64 loss of tests/fd.py equals the float forward
    at the base point, and its Ridders-refined central differences (from
    eps 1e-3) reproduce the oracle backward that takes the float forward's
    decisions: positions (clip and world coordinates) and attributes of 24
    seeded vertices of a displaced icosphere at 192 x 192, 8 channels."""
    from diffrp_gb300 import synthetic as S
    from tests.fd import FixedVisibilityL1
    H = W = 192
    v, f = S.displaced_icosphere(3, 0.8, 0.02, 5)
    rng = np.random.default_rng(6)
    attr = rng.uniform(0, 1, (len(v), 8)).astype(np.float32)
    mvp = S.perspective(30.0, H, W, 0.1, 100.0).astype(np.float64) @ \
        S.view_matrix(S.lookat_pose((0.3, 0.2, 3.1))).astype(np.float64)
    pos = S.clip_positions(v, mvp)
    target = rng.uniform(0, 1, (H, W, 8)).astype(np.float32)
    rast, _, _ = O.rasterize(pos, f, (H, W), grad_db=False)
    col, _ = O.interpolate(attr, rast, f)
    nbr = O.topology(f)
    out = O.antialias(col, rast, pos, f, nbr)
    fd = FixedVisibilityL1(pos, f, attr, target, rast[0], out[0], nbr)
    assert len(fd.plan) > 100
    base = fd.loss_terms()
    ref = (fd.sign.astype(np.float64) * out.reshape(-1)).sum()
    assert abs(base - ref) <= 1e-6 * abs(ref)

    g_out = (np.sign(out - target[None]) / np.float32(out.size)).astype(np.float32)
    g_col, g_pos_aa = O.antialias_bwd(col, rast, pos, f, g_out, nbr, precision="f32")
    g_attr, g_rast, _ = O.interpolate_bwd(attr, rast, f, g_col, precision="f32")
    g_pos = g_pos_aa + O.raster_bwd(pos, f, rast, g_rast, precision="f32")
    pick = fd.pick_vertices(24, seed=3)
    G = np.array([fd.grad_pos(j)[0] for j in pick])
    assert np.abs(G - g_pos[pick]).max() <= 1e-4 * np.abs(G).max()
    assert np.abs(G[:, 2]).max() == 0.0  # clip z carries no gradient with the decisions held
    Gw = np.array([fd.grad_pos(j, (0, 1, 2), mvp=mvp, verts=v)[0] for j in pick[:8]])
    gw = g_pos[pick[:8]] @ mvp[:, :3]
    assert np.abs(Gw - gw).max() <= 1e-4 * np.abs(Gw).max()
    A = np.array([fd.grad_attr(j) for j in pick])
    assert np.abs(A - g_attr[pick]).max() <= 1e-5 * np.abs(A).max()
