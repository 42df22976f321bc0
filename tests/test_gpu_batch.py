"""The batching form against the per-item drop-in calls.

Every item of a BatchRenderer (mixed meshes, views, resolutions and channel
counts in one launch sequence) must reproduce, bit for bit, the rast,
interpolated colour and antialiased image of calling nvdr.rasterize /
interpolate / antialias on that item alone (which the op tests pin to the
oracle), and its gradients must agree with the per-item autograd chain
within 1e-4 of the largest gradient magnitude.
"""
import numpy as np
import pytest
import torch

from diffrp_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


SMALL_ITEMS = [(0, (48, 64)), (1, (32, 32)), (0, (40, 40)), (2, (24, 56)), (1, (64, 48))]
# 8x8 tiles: 4875 + 1536 + 2764 tiles, more than two 4096-tile scan chunks
LARGE_ITEMS = [(0, (520, 600)), (1, (384, 256)), (2, (700, 252))]


def _scene(items=SMALL_ITEMS):
    rng = np.random.default_rng(0)
    meshes_np = [S.icosphere(2, 0.8), S.random_displaced_grid(9, seed=1, sigma=0.1), S.icosphere(1, 0.6)]
    chans = [8, 5, 3]
    attrs = [rng.uniform(0, 1, (len(v), c)).astype(np.float32) for (v, _), c in zip(meshes_np, chans)]
    views = []
    for k, (m, (H, W)) in enumerate(items):
        v, _ = meshes_np[m]
        eye = S.sphere_eyes(1, 2.6, seed=10 + k)[0]
        mvp = S.perspective(40.0, H, W, 0.1, 20.0).astype(np.float64) @ \
            S.view_matrix(S.lookat_pose(eye)).astype(np.float64)
        views.append(S.clip_positions(v, mvp))
    return meshes_np, chans, attrs, items, views


# recompute modes: stored buffers, recompute in one chunk, recompute in
# chunks of at most 3000 pixels (one or two items each)
RECOMPUTE = [False, True, "chunked"]


def _renderer(recompute=False, tile_log2=4, tpt=0, items=SMALL_ITEMS, bin_depth=None):
    from diffrp_gb300.batch import BatchRenderer
    meshes_np, chans, attrs, items, views = _scene(items)
    meshes = [(torch.from_numpy(f).cuda(), len(v), c) for (v, f), c in zip(meshes_np, chans)]
    r = BatchRenderer(meshes, items, tile_log2=tile_log2, threads_per_tri=tpt, recompute=bool(recompute),
                      bin_depth=bin_depth, chunk_pixels=3000 if recompute == "chunked" else 1 << 23)
    if recompute == "chunked":
        assert len(r._chunks) >= 3
    pos = r.pack_positions([torch.from_numpy(p).cuda() for p in views])
    attr = r.pack_attributes([torch.from_numpy(a).cuda() for a in attrs])
    return r, pos, attr, (meshes_np, chans, attrs, items, views)


@pytest.mark.parametrize("tile_log2,tpt,items", [(4, 0, SMALL_ITEMS), (5, 0, SMALL_ITEMS), (3, 4, SMALL_ITEMS),
                                                 (3, 0, LARGE_ITEMS)], ids=["t4", "t5", "t3p4", "t3_many_tiles"])
def test_batch_forward_matches_per_item_calls(cuda_lib, tile_log2, tpt, items):
    from diffrp_gb300 import nvdr as dr
    r, pos, attr, (meshes_np, chans, attrs, items, views) = _renderer(tile_log2=tile_log2, tpt=tpt, items=items)
    rast, color, out = r.forward_buffers(pos, attr)
    rv = r.rast_views(rast)
    cv = r.images(color)
    ov = r.images(out)
    ctx = dr.RasterizeCudaContext()
    for k, (m, (H, W)) in enumerate(items):
        tri = torch.from_numpy(meshes_np[m][1]).cuda()
        p = torch.from_numpy(views[k]).cuda()
        rr, _ = dr.rasterize(ctx, p, tri, (H, W), grad_db=False)
        cc, _ = dr.interpolate(torch.from_numpy(attrs[m]).cuda(), rr, tri)
        oo = dr.antialias(cc, rr, p, tri)
        assert torch.equal(rv[k], rr[0]), "rast differs for item %d" % k
        assert torch.equal(cv[k], cc[0]), "colour differs for item %d" % k
        assert torch.equal(ov[k], oo[0]), "antialiased image differs for item %d" % k


@pytest.mark.parametrize("recompute", RECOMPUTE)
def test_batch_gradients_match_per_item_autograd(cuda_lib, recompute):
    from diffrp_gb300 import nvdr as dr
    r, pos, attr, (meshes_np, chans, attrs, items, views) = _renderer(recompute=recompute)
    rng = np.random.default_rng(3)
    w = torch.from_numpy(rng.normal(size=r.image_floats).astype(np.float32)).cuda()
    pos_b = pos.clone().requires_grad_(True)
    attr_b = attr.clone().requires_grad_(True)
    (r(pos_b, attr_b) * w).sum().backward()
    ctx = dr.RasterizeCudaContext()
    wv = r.images(w)
    attr_ts = [torch.from_numpy(a).cuda().requires_grad_(True) for a in attrs]
    pos_ts = []
    loss = 0
    for k, (m, (H, W)) in enumerate(items):
        tri = torch.from_numpy(meshes_np[m][1]).cuda()
        p = torch.from_numpy(views[k]).cuda().requires_grad_(True)
        pos_ts.append(p)
        rr, _ = dr.rasterize(ctx, p, tri, (H, W), grad_db=False)
        cc, _ = dr.interpolate(attr_ts[m], rr, tri)
        oo = dr.antialias(cc, rr, p, tri)
        loss = loss + (oo[0] * wv[k]).sum()
    loss.backward()
    gp_ref = torch.cat([p.grad for p in pos_ts]).cpu().numpy()
    ga_ref = torch.cat([a.grad.reshape(-1) for a in attr_ts]).cpu().numpy()
    for got, ref in [(pos_b.grad.cpu().numpy(), gp_ref), (attr_b.grad.cpu().numpy(), ga_ref)]:
        scale = max(np.abs(ref).max(), 1e-12)
        assert np.abs(got - ref).max() / scale <= 1e-4


def test_batch_backward_after_interleaved_forward(cuda_lib):
    """A second forward on other positions before the first backward replaces
    the workspace's antialias records: the first backward must rebuild its
    own and give the same gradients as an uninterrupted forward / backward."""
    r, pos, attr, _ = _renderer()
    w = torch.linspace(-1, 1, r.image_floats, device="cuda")
    pa = pos.clone().requires_grad_(True)
    (r(pa, attr) * w).sum().backward()
    ref = pa.grad.clone()
    pb = pos.clone().requires_grad_(True)
    out1 = r(pb, attr)
    other = pos.clone()
    other[:, :2] *= 1.1
    r(other, attr)  # overwrites the records
    (out1 * w).sum().backward()
    scale = ref.abs().max()
    assert float((pb.grad - ref).abs().max() / scale) <= 1e-5


@pytest.mark.parametrize("depth", [None, 2], ids=["sized", "overflowing"])
def test_batch_fixed_depth_bins_exact(cuda_lib, depth):
    """The first forward uses exact tile lists and sizes fixed-depth bins from
    its largest tile; later forwards bin in one pass.  Both give the same
    images; bins too shallow for their tiles still rasterise exactly and grow
    for the next forward."""
    r, pos, attr, _ = _renderer(bin_depth=depth)
    first = r.forward_buffers(pos, attr)
    assert r._depth > 0
    second = r.forward_buffers(pos, attr)
    for a, b in zip(first, second):
        assert torch.equal(a, b)
    if depth == 2:
        assert r.last_max_tile > 2
        torch.cuda.synchronize()
        r._poll_stats()
        assert r._depth > 2


@pytest.mark.parametrize("recompute", RECOMPUTE)
@pytest.mark.parametrize("use_images", [False, True])
def test_batch_render_l1_matches_unfused(cuda_lib, recompute, use_images):
    """render_l1 gives the images of the plain forward bit for bit, the loss
    of l1_loss on them (summation order aside) and the same gradients, with
    a non-unit upstream loss gradient and, optionally, a second loss on the
    images."""
    from diffrp_gb300.losses import l1_loss
    r, pos, attr, _ = _renderer(recompute=recompute)
    g = torch.Generator(device="cuda").manual_seed(5)
    target = torch.rand(r.image_floats, device="cuda", generator=g)
    w = torch.linspace(-1, 1, r.image_floats, device="cuda")

    def run(fused):
        p = pos.clone().requires_grad_(True)
        a = attr.clone().requires_grad_(True)
        if fused:
            loss, img = r.render_l1(p, a, target)
        else:
            img = r(p, a)
            loss = l1_loss(img, target)
        total = 3.0 * loss + ((img * w).sum() if use_images else 0.0)
        total.backward()
        return loss.detach(), img.detach(), p.grad, a.grad

    lf, imf, gpf, gaf = run(True)
    lu, imu, gpu_, gau = run(False)
    assert torch.equal(imf, imu)
    assert torch.allclose(lf, lu, rtol=2e-6, atol=0)
    for got, ref in [(gpf, gpu_), (gaf, gau)]:
        assert float((got - ref).abs().max() / ref.abs().max()) <= 1e-5


def test_batch_raster_only_forward(cuda_lib):
    """A forward without an output buffer writes the same rast and colour as
    the full forward (the antialias pass is skipped)."""
    r, pos, attr, _ = _renderer()
    rast, color, out = r.forward_buffers(pos, attr)
    rast2, color2 = r._buffers()
    r._forward_raw(pos, attr, rast2, color2, None)
    assert torch.equal(rast, rast2) and torch.equal(color, color2)


def test_batch_cuda_graph_replay(cuda_lib):
    r, pos, attr, _ = _renderer()
    pos_b = pos.clone().requires_grad_(True)
    attr_b = attr.clone().requires_grad_(True)
    w = torch.linspace(-1, 1, r.image_floats, device="cuda")

    def step():
        pos_b.grad = None
        attr_b.grad = None
        loss = (r(pos_b, attr_b) * w).sum()
        loss.backward()
        return loss

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(2):
            ref_loss = step()
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    ref_gp = pos_b.grad.clone()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        loss = step()
    g.replay()
    torch.cuda.synchronize()
    assert torch.allclose(loss, ref_loss)
    scale = ref_gp.abs().max()
    assert float((pos_b.grad - ref_gp).abs().max() / scale) <= 1e-5


def test_backward_on_a_side_stream_matches_default_stream(cuda_lib):
    """The batching form's backward forks its listed-pixel kernel onto a
    library stream and joins it back into the caller's stream: run on a
    non-default torch stream (and from a second host thread), the gradients
    equal the default-stream ones up to atomic summation order."""
    import threading
    from diffrp_gb300.batch import BatchRenderer
    H = W = 256
    v, f = S.displaced_icosphere(3, 0.8, 0.02, 5)
    mvp = S.perspective(30.0, H, W, 0.1, 100.0).astype(np.float64) @ \
        S.view_matrix(S.lookat_pose((0.0, 0.0, 3.2))).astype(np.float64)
    pos = torch.from_numpy(S.clip_positions(v, mvp)).cuda()
    attr = torch.from_numpy(np.random.default_rng(5).uniform(0, 1, (len(v), 4)).astype(np.float32)).cuda()
    tri = torch.from_numpy(f).cuda()
    target = torch.rand(H * W * 4, device="cuda", generator=torch.Generator(device="cuda").manual_seed(5))

    def run(stream):
        r = BatchRenderer([(tri, len(v), 4)], [(0, (H, W))], tile_log2=4)
        p = pos.clone().requires_grad_(True)
        a = attr.reshape(-1).clone().requires_grad_(True)
        with torch.cuda.stream(stream):
            for _ in range(2):  # the second call forks (side stream created by the first)
                p.grad = a.grad = None
                loss, _ = r.render_l1(p, a, target)
                loss.backward()
        stream.synchronize()
        return p.grad.clone(), a.grad.clone()

    ref = run(torch.cuda.current_stream())
    side = run(torch.cuda.Stream())
    out = {}
    th = threading.Thread(target=lambda: out.setdefault("g", run(torch.cuda.Stream())))
    th.start()
    th.join()
    for got in (side, out["g"]):
        for x, y in zip(got, ref):
            assert torch.allclose(x, y, rtol=1e-5, atol=1e-7)


def test_batch_recompute_chunks_match_stored(cuda_lib):
    """Recompute in chunks (each chunk's forward re-run in the backward) gives
    the stored-buffer path's images bit for bit and its gradients to 1e-5,
    eagerly and replayed from a CUDA graph, with the fused L1 loss."""
    r0, pos, attr, _ = _renderer(recompute=False)
    r1, _, _, _ = _renderer(recompute="chunked")
    g = torch.Generator(device="cuda").manual_seed(7)
    target = torch.rand(r0.image_floats, device="cuda", generator=g)

    def run(r):
        p = pos.clone().requires_grad_(True)
        a = attr.clone().requires_grad_(True)

        def step():
            p.grad = None
            a.grad = None
            loss, img = r.render_l1(p, a, target)
            loss.backward()
            return loss, img
        loss, img = step()
        return step, p, a, loss.detach().clone(), img.detach().clone(), p.grad.clone(), a.grad.clone()

    _, _, _, l0, im0, gp0, ga0 = run(r0)
    step, p1, a1, l1, im1, gp1, ga1 = run(r1)
    assert torch.equal(im0, im1)
    assert torch.allclose(l0, l1, rtol=2e-6, atol=0)
    for got, ref in [(gp1, gp0), (ga1, ga0)]:
        assert float((got - ref).abs().max() / ref.abs().max()) <= 1e-5
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(2):
            step()
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        gl, gimg = step()
    p1.grad.zero_()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(gimg, im1)
    for got, ref in [(p1.grad, gp0), (a1.grad, ga0)]:
        assert float((got - ref).abs().max() / ref.abs().max()) <= 1e-5


@pytest.mark.parametrize("recompute,tile_log2", [(m, 4) for m in RECOMPUTE] + [(False, 3), (False, 5)])
@pytest.mark.parametrize("use_images", [False, True])
def test_batch_render_l1_grads_in_forward(cuda_lib, recompute, tile_log2, use_images):
    """render_l1 with the loss's gradient formed in the forward pass gives
    the images bit for bit, the same loss and the gradients of the ordinary
    backward (to 1e-5), with a non-unit upstream loss gradient; when the
    images reach the objective too, the full backward runs instead.  On 8-,
    16- and 32-pixel tiles (stored buffers), and in the three recompute modes
    on 16-pixel tiles."""
    r, pos, attr, _ = _renderer(recompute=recompute, tile_log2=tile_log2)
    g = torch.Generator(device="cuda").manual_seed(11)
    target = torch.rand(r.image_floats, device="cuda", generator=g)
    w = torch.linspace(-1, 1, r.image_floats, device="cuda")

    def run(eager):
        p = pos.clone().requires_grad_(True)
        a = attr.clone().requires_grad_(True)
        loss, img = r.render_l1(p, a, target, grads_in_forward=eager)
        total = 3.0 * loss + ((img * w).sum() if use_images else 0.0)
        total.backward()
        return loss.detach(), img.detach(), p.grad, a.grad

    le, ime, gpe, gae = run(True)
    lr, imr, gpr, gar = run(False)
    assert torch.equal(ime, imr)
    assert torch.allclose(le, lr, rtol=2e-6, atol=0)
    for got, ref in [(gpe, gpr), (gae, gar)]:
        assert float((got - ref).abs().max() / ref.abs().max()) <= 1e-5


def test_batch_render_l1_grads_in_forward_graph_replay(cuda_lib):
    """The forward that forms the gradient, captured with its backward in a
    CUDA graph and replayed, matches an eager step.  (Every step before the
    capture runs on a side stream: a leaf first differentiated on the legacy
    default stream keeps that stream for its gradient accumulation, which
    a capture cannot wait on.)"""
    r, pos, attr, _ = _renderer()
    g = torch.Generator(device="cuda").manual_seed(12)
    target = torch.rand(r.image_floats, device="cuda", generator=g)
    p = pos.clone().requires_grad_(True)
    a = attr.clone().requires_grad_(True)

    def step():
        p.grad = None
        a.grad = None
        loss, img = r.render_l1(p, a, target, grads_in_forward=True)
        loss.backward()
        return loss, img
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        l0, im0 = step()
        ref = (l0.detach().clone(), im0.detach().clone(), p.grad.clone(), a.grad.clone())
        for _ in range(2):
            step()
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        gl, gimg = step()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(gimg, ref[1])
    assert torch.allclose(gl, ref[0], rtol=0, atol=0)
    for got, want in [(p.grad, ref[2]), (a.grad, ref[3])]:
        assert float((got - want).abs().max() / want.abs().max()) <= 1e-6
