"""GPU parity: the CUDA ops (through the C ABI via diffrp_gb300.nvdr) against
the CPU oracle on the same seeded inputs.

Bars: visibility (tri id), rast, rast_db, interpolation and antialias forward
are bit-exact (both sides round once per float op in the same order);
gradients agree with the float64 oracle within 1e-4 relative to the largest
gradient magnitude of the tensor (atomics reorder float additions).
"""
import numpy as np
import pytest
import torch

import oracle as O
from tests import scenes

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-4


def _dr():
    from diffrp_gb300 import nvdr
    return nvdr


def _ctx(**kw):
    return _dr().RasterizeCudaContext(**kw)


def _t(a, dtype=None):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda() if dtype is None else \
        torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).cuda()


def _grad_close(got, ref, rtol=GRAD_RTOL):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = max(np.abs(ref).max(), 1e-12)
    err = np.abs(got - ref).max() / scale
    assert err <= rtol, "gradient max error %.3g relative to max |ref| %.3g" % (err, scale)


CASES = [
    ("soup", lambda: scenes.random_soup(200, seed=0), (61, 77), None),
    ("sphere", lambda: scenes.sphere_view(3, res=(128, 128)), (128, 128), None),
    ("near_crossing", scenes.near_crossing, (32, 32), None),
]


@pytest.mark.parametrize("tile_log2,tpt", [(4, 0), (3, 0), (5, 0), (4, 8), (3, 1), (5, 32)])
@pytest.mark.parametrize("name,make,res,ranges", CASES, ids=[c[0] for c in CASES])
def test_rasterize_bit_exact(cuda_lib, name, make, res, ranges, tile_log2, tpt):
    pos, tri = make()
    rast_ref, db_ref, key_ref = O.rasterize(pos, tri, res)
    dr = _dr()
    rast, db = dr.rasterize(_ctx(tile_log2=tile_log2, threads_per_tri=tpt), _t(pos), _t(tri), res)
    rast = rast.cpu().numpy()
    db = db.cpu().numpy()
    assert (rast[..., 3] > 0).sum() > 0
    np.testing.assert_array_equal(rast[..., 3], rast_ref[..., 3])
    np.testing.assert_array_equal(rast, rast_ref)
    np.testing.assert_array_equal(db, db_ref)


def test_rasterize_instanced_and_ranges(cuda_lib):
    pos, tri = scenes.multi_view(2, n_views=5, res=(40, 56))
    dr = _dr()
    rast, _ = dr.rasterize(_ctx(), _t(pos), _t(tri), (40, 56), grad_db=False)
    ref, _, _ = O.rasterize(pos, tri, (40, 56), grad_db=False)
    np.testing.assert_array_equal(rast.cpu().numpy(), ref)
    # range mode: two meshes in one vertex buffer, one view each
    p1, t1 = scenes.random_soup(50, seed=5)
    p2, t2 = scenes.random_soup(70, seed=6)
    pos2 = np.concatenate([p1, p2])
    tri2 = np.concatenate([t1, t2 + len(p1)]).astype(np.int32)
    ranges = np.array([[0, len(t1)], [len(t1), len(t2)]], np.int32)
    rast, _ = dr.rasterize(_ctx(), _t(pos2), _t(tri2), (33, 47), ranges=torch.from_numpy(ranges), grad_db=False)
    ref, _, _ = O.rasterize(pos2, tri2, (33, 47), ranges=ranges, grad_db=False)
    np.testing.assert_array_equal(rast.cpu().numpy(), ref)


def test_list_overflow_fallback_exact(cuda_lib):
    """An undersized tile-list capacity must not change the result."""
    pos, tri = scenes.random_soup(300, seed=11)
    ctx = _ctx()
    ctx.ensure_capacity(16)  # far too small: every tile falls back to the full scan
    rast, _ = _dr().rasterize(ctx, _t(pos), _t(tri), (64, 64), grad_db=False)
    ref, _, _ = O.rasterize(pos, tri, (64, 64), grad_db=False)
    np.testing.assert_array_equal(rast.cpu().numpy(), ref)


def test_tile_scan_across_chunks(cuda_lib):
    """More tiles than one scan chunk of 4096: 14 views of 300x260 with 8x8
    tiles is 17556 tiles (five chunks, the last one ragged).  The image is
    exact, no tile overflows its list, and the list total equals the sum of
    the per-view totals (each view alone fits in one chunk)."""
    res = (300, 260)
    pos, tri = scenes.multi_view(2, n_views=14, res=res)
    dr = _dr()
    ctx = _ctx(tile_log2=3, validate=True)
    rast, _ = dr.rasterize(ctx, _t(pos), _t(tri), res, grad_db=False)
    total, err = ctx._read_stats_sync()
    assert err & 2 == 0, "a tile list overflowed"
    ref, _, _ = O.rasterize(pos, tri, res, grad_db=False)
    np.testing.assert_array_equal(rast.cpu().numpy(), ref)
    per_view = 0
    for v in range(pos.shape[0]):
        c = _ctx(tile_log2=3, validate=True)
        dr.rasterize(c, _t(pos[v:v + 1]), _t(tri), res, grad_db=False)
        per_view += c._read_stats_sync()[0]
    assert total == per_view > 0


def test_list_capacity_grows_across_mixed_calls(cuda_lib):
    """One context serving a small and then a much denser view: the dense
    call overflows the capacity sized by the first (still exact), its stats
    are read back later, and the next dense call has room."""
    dr = _dr()
    ctx = _ctx()
    small_pos, small_tri = scenes.random_soup(20, seed=1)
    dr.rasterize(ctx, _t(small_pos), _t(small_tri), (64, 64), grad_db=False)
    cap0 = ctx._capacity
    pos, tri = scenes.random_soup(3000, seed=2)
    ref, _, _ = O.rasterize(pos, tri, (64, 64), grad_db=False)
    rast, _ = dr.rasterize(ctx, _t(pos), _t(tri), (64, 64), grad_db=False)
    np.testing.assert_array_equal(rast.cpu().numpy(), ref)
    torch.cuda.synchronize()
    rast, _ = dr.rasterize(ctx, _t(pos), _t(tri), (64, 64), grad_db=False)  # polls the earlier stats first
    assert ctx._capacity > cap0
    _, err = ctx._read_stats_sync()
    assert err & 2 == 0, "the list still overflowed after the read-back"
    np.testing.assert_array_equal(rast.cpu().numpy(), ref)


@pytest.mark.parametrize("tile_log2,tpt", [(4, 0), (3, 1), (5, 4)])
def test_fixed_depth_bins_exact(cuda_lib, tile_log2, tpt):
    """After the first call of a shape (exact lists, synchronous sizing) the
    context bins in one pass; repeated calls stay bit-exact, including a
    forced too-shallow depth (overflowing tiles scan the view exactly)."""
    pos, tri = scenes.multi_view(2, n_views=3, res=(72, 56))
    ref, _, _ = O.rasterize(pos, tri, (72, 56), grad_db=False)
    ctx = _ctx(tile_log2=tile_log2, threads_per_tri=tpt)
    for _ in range(3):
        rast, _ = _dr().rasterize(ctx, _t(pos), _t(tri), (72, 56), grad_db=False)
        np.testing.assert_array_equal(rast.cpu().numpy(), ref)
    assert any(d > 0 for d in ctx._depth.values())
    for k in ctx._depth:
        ctx._depth[k] = 1
    rast, _ = _dr().rasterize(ctx, _t(pos), _t(tri), (72, 56), grad_db=False)
    np.testing.assert_array_equal(rast.cpu().numpy(), ref)
    _, err = ctx._read_stats_sync()
    assert err & 2


def test_depth_peeling(cuda_lib):
    pos, tri = scenes.random_soup(120, seed=2)
    dr = _dr()
    ctx = _ctx()
    prev = None
    with dr.DepthPeeler(ctx, _t(pos), _t(tri), (48, 48)) as dp:
        for layer in range(3):
            rast, db = dp.rasterize_next_layer()
            ref, dref, prev = O.rasterize(pos, tri, (48, 48), prev_key=prev)
            np.testing.assert_array_equal(rast.cpu().numpy(), ref)
            np.testing.assert_array_equal(db.cpu().numpy(), dref)


def test_rasterize_bwd(cuda_lib):
    pos, tri = scenes.sphere_view(3, res=(96, 96), sigma=0.02, seed=1)
    rng = np.random.default_rng(0)
    posg = _t(pos).requires_grad_(True)
    rast, db = _dr().rasterize(_ctx(), posg, _t(tri), (96, 96))
    g = rng.normal(size=(1, 96, 96, 4)).astype(np.float32)
    gdb = rng.normal(size=(1, 96, 96, 4)).astype(np.float32)
    ((rast * _t(g)).sum() + (db * _t(gdb)).sum()).backward()
    rr = rast.detach().cpu().numpy()
    ref = O.raster_bwd(pos, tri, rr, g, gdb)
    _grad_close(posg.grad.cpu().numpy(), ref)


@pytest.mark.parametrize("C,diff", [(3, None), (8, "all"), (5, [0, 3])])
def test_interpolate_fwd_bwd(cuda_lib, C, diff):
    pos, tri = scenes.sphere_view(3, res=(80, 80), sigma=0.02, seed=2)
    rng = np.random.default_rng(C)
    attr = rng.uniform(0, 1, (len(pos), C)).astype(np.float32)
    dr = _dr()
    rast, db = dr.rasterize(_ctx(), _t(pos), _t(tri), (80, 80))
    attr_t = _t(attr).requires_grad_(True)
    rast_in = rast.clone().requires_grad_(True)
    db_in = db.clone().requires_grad_(True)
    out, da = dr.interpolate(attr_t, rast_in, _t(tri), rast_db=db_in, diff_attrs=diff)
    r_np, db_np = rast.cpu().numpy(), db.cpu().numpy()
    oref, daref = O.interpolate(attr, r_np, tri, db_np, diff_attrs=diff)
    np.testing.assert_array_equal(out.detach().cpu().numpy(), oref)
    if diff is not None:
        np.testing.assert_array_equal(da.detach().cpu().numpy(), daref)
    go = rng.normal(size=out.shape).astype(np.float32)
    loss = (out * _t(go)).sum()
    gda = None
    if diff is not None:
        gda = rng.normal(size=da.shape).astype(np.float32)
        loss = loss + (da * _t(gda)).sum()
    loss.backward()
    ga, gr, gd = O.interpolate_bwd(attr, r_np, tri, go, db_np, diff, gda)
    _grad_close(attr_t.grad.cpu().numpy(), ga)
    _grad_close(rast_in.grad.cpu().numpy()[..., :2], gr[..., :2])
    if diff is not None:
        _grad_close(db_in.grad.cpu().numpy(), gd)


def test_interpolate_batched_attr(cuda_lib):
    pos, tri = scenes.multi_view(2, n_views=3, res=(32, 32))
    rng = np.random.default_rng(4)
    attr = rng.uniform(0, 1, (3, pos.shape[1], 4)).astype(np.float32)
    dr = _dr()
    rast, _ = dr.rasterize(_ctx(), _t(pos), _t(tri), (32, 32), grad_db=False)
    out, _ = dr.interpolate(_t(attr), rast, _t(tri))
    ref, _ = O.interpolate(attr, rast.cpu().numpy(), tri)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


def _opposite_vertices(f, nbr):
    """The oracle's neighbour-triangle table as opposite vertices: for edge k
    of triangle t, the vertex of its neighbour not on the edge."""
    opp = np.full(f.shape, -1, np.int32)
    for t in range(f.shape[0]):
        for k in range(3):
            n = nbr[t, k]
            if n >= 0:
                edge = {f[t, (k + 1) % 3], f[t, (k + 2) % 3]}
                opp[t, k] = [x for x in f[n] if x not in edge][-1]
    return opp


def test_topology_matches_oracle(cuda_lib):
    _, f = scenes.sphere_view(3, res=(8, 8))
    opp = _dr().antialias_construct_topology_hash(_t(f)).cpu().numpy()
    np.testing.assert_array_equal(opp, _opposite_vertices(f, O.topology(f)))
    soup = np.arange(30, dtype=np.int32).reshape(10, 3)
    assert (_dr().antialias_construct_topology_hash(_t(soup)).cpu().numpy() == -1).all()


@pytest.mark.parametrize("soup", [False, True])
def test_antialias_fwd_bwd(cuda_lib, soup):
    pos, tri = scenes.sphere_view(3, res=(96, 96), sigma=0.03, seed=3)
    if soup:
        pos = pos[tri].reshape(-1, 4)
        tri = np.arange(len(pos), dtype=np.int32).reshape(-1, 3)
    rng = np.random.default_rng(7)
    dr = _dr()
    rast, _ = dr.rasterize(_ctx(), _t(pos), _t(tri), (96, 96), grad_db=False)
    color = rng.uniform(0, 1, (1, 96, 96, 3)).astype(np.float32)
    col_t = _t(color).requires_grad_(True)
    pos_t = _t(pos).requires_grad_(True)
    out = dr.antialias(col_t, rast, pos_t, _t(tri))
    r_np = rast.cpu().numpy()
    ref = O.antialias(color, r_np, pos, tri)
    np.testing.assert_array_equal(out.detach().cpu().numpy(), ref)
    assert (np.abs(ref - color).sum(-1) > 0).sum() > 10
    go = rng.normal(size=out.shape).astype(np.float32)
    (out * _t(go)).sum().backward()
    gc, gp = O.antialias_bwd(color, r_np, pos, tri, go)
    _grad_close(col_t.grad.cpu().numpy(), gc)
    _grad_close(pos_t.grad.cpu().numpy(), gp)


def test_antialias_bwd_with_and_without_pixel_list(cuda_lib):
    """drp_antialias_bwd given the forward's pixel list equals the full
    per-pixel evaluation (no list): the same colour gradient bit for bit and
    the same position gradient up to atomic order; two views exercise the
    list's view index."""
    from diffrp_gb300 import _ffi
    pos, tri = scenes.multi_view(2, n_views=2, res=(72, 88))
    rng = np.random.default_rng(4)
    dr = _dr()
    pos_t, tri_t = _t(pos), _t(tri)
    rast, _ = dr.rasterize(_ctx(), pos_t, tri_t, (72, 88), grad_db=False)
    B, H, W, C = 2, 72, 88, 4
    col = _t(rng.uniform(0, 1, (B, H, W, C)).astype(np.float32))
    go = _t(rng.normal(size=(B, H, W, C)).astype(np.float32))
    nbr = dr.antialias_construct_topology_hash(tri_t)
    F, V = tri.shape[0], pos.shape[1]
    ws = torch.empty(_ffi.size_out("drp_antialias_workspace_size", B, F), dtype=torch.uint8, device="cuda")
    state = torch.empty(_ffi.size_out("drp_antialias_state_size", B, H, W), dtype=torch.uint8, device="cuda")
    out = torch.empty_like(col)
    sp = torch.cuda.current_stream().cuda_stream
    common = (col.data_ptr(), C, rast.data_ptr(), pos_t.data_ptr(), V * 4, V, tri_t.data_ptr(), F, nbr.data_ptr(),
              B, H, W)
    _ffi.call("drp_antialias_fwd", ws.data_ptr(), ws.numel(), *common, out.data_ptr(), state.data_ptr(), sp)
    grads = []
    for st in (None, state.data_ptr()):
        gc = torch.empty_like(col)
        gp = torch.zeros_like(pos_t)
        _ffi.call("drp_antialias_bwd", ws.data_ptr(), ws.numel(), *common, go.data_ptr(), 1.0, gc.data_ptr(),
                  gp.data_ptr(), st, sp)
        grads.append((gc, gp))
    assert torch.equal(grads[0][0], grads[1][0])
    assert not torch.equal(grads[0][0], go)  # some pixels blend
    scale = grads[0][1].abs().max()
    assert scale > 0 and float((grads[0][1] - grads[1][1]).abs().max() / scale) <= 1e-5


def test_sparse_interpolate(cuda_lib):
    from diffrp_gb300.rendering.interpolator import polyfill_interpolate
    rng = np.random.default_rng(9)
    V, N, C = 50, 333, 6
    vb = rng.normal(size=(V, C)).astype(np.float32)
    vi = np.concatenate([rng.uniform(0, 0.5, (N, 2)), rng.uniform(0, 1, (N, 1)), np.ones((N, 1))], 1)
    vi = vi.astype(np.float32)
    ti = rng.integers(0, V, (N, 3)).astype(np.int64)
    vb_t = _t(vb).requires_grad_(True)
    vi_t = _t(vi).requires_grad_(True)
    out = polyfill_interpolate(vb_t, vi_t, _t(ti))
    np.testing.assert_array_equal(out.detach().cpu().numpy(), O.interpolate_sparse(vb, vi, ti))
    go = rng.normal(size=out.shape).astype(np.float32)
    (out * _t(go)).sum().backward()
    # float64 reference of the gather + FMA (interpolator.py:39-45)
    w = np.stack([vi[:, 0], vi[:, 1], 1 - vi[:, 0] - vi[:, 1]], 1).astype(np.float64)
    gvb = np.zeros((V, C))
    for k in range(3):
        np.add.at(gvb, ti[:, k], go * w[:, k:k + 1])
    _grad_close(vb_t.grad.cpu().numpy(), gvb)
    gu = (go * (vb[ti[:, 0]] - vb[ti[:, 2]])).sum(1)
    _grad_close(vi_t.grad.cpu().numpy()[:, 0], gu)


def test_autotuner_choice_is_exact(cuda_lib, tmp_path, monkeypatch):
    from diffrp_gb300 import autotune
    monkeypatch.setenv("DRP_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    pos, tri = scenes.sphere_view(3, res=(96, 96), sigma=0.02, seed=5)
    ctx = _ctx()
    choice = autotune.tune_rasterizer(ctx, _t(pos), _t(tri), (96, 96), reps=2,
                                      candidates=[(3, 0), (4, 0), (4, 8), (5, 1)])
    assert (ctx.tile_log2, ctx.threads_per_tri) == (choice["tile_log2"], choice["threads_per_tri"])
    rast, _ = _dr().rasterize(ctx, _t(pos), _t(tri), (96, 96), grad_db=False)
    ref, _, _ = O.rasterize(pos, tri, (96, 96), grad_db=False)
    np.testing.assert_array_equal(rast.cpu().numpy(), ref)
    again = autotune.tune_rasterizer(_ctx(), _t(pos), _t(tri), (96, 96))
    assert again["tile_log2"] == choice["tile_log2"] and again["threads_per_tri"] == choice["threads_per_tri"]


def test_triangle_ids_above_2_pow_24(cuda_lib):
    """Triangle ids past 2^24 use the float-bit encoding of the rast w channel
    (diffrp/rendering/interpolator.py:24-29); the last triangles of a
    2^24 + 64 triangle buffer (all earlier ones degenerate) must come back
    with exactly the oracle's encoded ids, and decode to their indices."""
    from diffrp_gb300.rendering.interpolator import float_to_triidx
    n_deg = 1 << 24
    soup, st = scenes.random_soup(64, seed=21)
    pos = np.concatenate([np.array([[0.0, 0.0, 0.0, 1.0]], np.float32), soup])
    tri = np.zeros((n_deg + 64, 3), np.int32)
    tri[n_deg:] = st + 1
    rast, _ = _dr().rasterize(_ctx(), _t(pos), _t(tri), (24, 24), grad_db=False)
    ref, _, _ = O.rasterize(pos, tri, (24, 24), grad_db=False, nthreads=8)
    r = rast.cpu().numpy()
    np.testing.assert_array_equal(r, ref)
    ids = float_to_triidx(rast[..., 3]).cpu().numpy()
    covered = ids > 0
    assert covered.sum() > 0 and (ids[covered] > n_deg).all()
