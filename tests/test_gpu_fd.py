"""Gradients at the single-mesh benchmark size against FP64 central
differences.

Workload: the benchmark's single-mesh configuration (icosphere with 5
subdivisions, 10242 vertices / 20480 triangles displaced by N(0, 0.02),
1024 x 1024, 8 channels, L1 loss to a seeded U(0, 1) target).  64 seeded
vertices (32 of visible triangles, 32 of antialias front triangles) get
central differences of the loss in float64 (tests/fd.py: the loss with the
forward's discrete decisions held, steps from eps = 1e-3 refined by Ridders'
extrapolation), and the CUDA gradients must agree with them:
  - every position / attribute component within 1e-4 of the largest
    finite-difference component of its kind (the relative gradient bar);
  - each vertex's position gradient within 1e-3 of its own norm (a vertex
    whose gradient is a small sum of larger float32 terms keeps the float32
    accumulation error of those terms).
Two paths: the benchmark's step (clip transform kernel, batching form with
the fused L1, gradients to world-space vertices and attributes) and the
drop-in nvdiffrast ops (rasterize, interpolate, antialias with topology,
l1_loss; gradients to clip-space positions and attributes).
"""
import numpy as np
import pytest
import torch

import oracle as O
from tests.fd import FixedVisibilityL1

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-4
VERTEX_RTOL = 1e-3
H = W = 1024


def _workload():
    import bench
    return bench.make_workload(0)


def _fd_reference(clip, f, attr, target, rast, out):
    """FixedVisibilityL1 around the GPU's own forward, after checking that
    forward against the oracle (so the held decisions are the GPU's)."""
    rast_ref, _, _ = O.rasterize(clip, f, (H, W), grad_db=False)
    np.testing.assert_array_equal(rast.reshape(rast_ref.shape), rast_ref)
    nbr = O.topology(f)
    col_ref, _ = O.interpolate(attr, rast_ref, f)
    out_ref = O.antialias(col_ref, rast_ref, clip, f, nbr)
    np.testing.assert_array_equal(out.reshape(out_ref.shape), out_ref)
    return FixedVisibilityL1(clip, f, attr, target.reshape(H, W, -1), rast_ref[0], out_ref[0], nbr)


def _gate(got, fd_vals, what, per_vertex=False):
    got = np.asarray(got, np.float64)
    scale = np.abs(fd_vals).max()
    err = np.abs(got - fd_vals).max() / scale
    assert err <= GRAD_RTOL, "%s: max error %.3g of the largest component (bar %g)" % (what, err, GRAD_RTOL)
    if per_vertex:
        pv = np.linalg.norm(got - fd_vals, axis=1) / np.maximum(np.linalg.norm(fd_vals, axis=1), 1e-30)
        assert pv.max() <= VERTEX_RTOL, "%s: per-vertex error %.3g (bar %g)" % (what, pv.max(), VERTEX_RTOL)
    return err


@pytest.mark.parametrize("grads_in_forward", [False, True], ids=["backward_pass", "grads_in_forward"])
def test_benchmark_step_gradients_match_finite_differences(cuda_lib, grads_in_forward):
    """Clip transform kernel + batching form with the fused L1 (gradient
    from the backward pass, or formed in the forward pass as the benchmark
    step does): world-space vertex and attribute gradients against central
    differences."""
    from diffrp_gb300.batch import BatchRenderer
    from diffrp_gb300.transform import clip_space
    v, f, attr, mvp, target = _workload()
    C = attr.shape[1]
    dev = torch.device("cuda", 0)
    verts_t = torch.from_numpy(v).to(dev).requires_grad_(True)
    attr_t = torch.from_numpy(attr).to(dev).reshape(-1).requires_grad_(True)
    clip_t = clip_space(verts_t, torch.from_numpy(mvp).to(dev))
    r = BatchRenderer([(torch.from_numpy(f).to(dev), len(v), C)], [(0, (H, W))], device=dev, tile_log2=5)
    rast, _, _ = r.forward_buffers(clip_t.detach(), attr_t.detach())
    loss, out = r.render_l1(clip_t, attr_t, torch.from_numpy(target).to(dev).reshape(-1),
                            grads_in_forward=grads_in_forward)
    loss.backward()
    torch.cuda.synchronize()
    clip = clip_t.detach().cpu().numpy()
    fd = _fd_reference(clip, f, attr, target, rast.cpu().numpy(), out.detach().cpu().numpy())
    pick = fd.pick_vertices(64)
    mvp64 = mvp.astype(np.float64)
    G = np.array([fd.grad_pos(j, (0, 1, 2), mvp=mvp64, verts=v)[0] for j in pick])
    _gate(verts_t.grad.cpu().numpy()[pick], G, "world-space vertex gradient", per_vertex=True)
    A = np.array([fd.grad_attr(j) for j in pick])
    _gate(attr_t.grad.view(-1, C).cpu().numpy()[pick], A, "attribute gradient")


def test_dropin_ops_gradients_match_finite_differences(cuda_lib):
    """nvdr.rasterize -> interpolate -> antialias (topology) -> l1_loss:
    clip-space position and attribute gradients against central differences."""
    from diffrp_gb300 import nvdr as dr
    from diffrp_gb300.losses import l1_loss
    from diffrp_gb300 import synthetic as S
    v, f, attr, mvp, target = _workload()
    C = attr.shape[1]
    dev = torch.device("cuda", 0)
    clip = S.clip_positions(v, mvp.astype(np.float64))
    pos_t = torch.from_numpy(clip).to(dev).requires_grad_(True)
    attr_t = torch.from_numpy(attr).to(dev).requires_grad_(True)
    tri_t = torch.from_numpy(f).to(dev)
    ctx = dr.RasterizeCudaContext(dev)
    rast, _ = dr.rasterize(ctx, pos_t, tri_t, (H, W), grad_db=False)
    col, _ = dr.interpolate(attr_t, rast, tri_t)
    out = dr.antialias(col, rast, pos_t, tri_t, topology_hash=dr.antialias_construct_topology_hash(tri_t))
    loss = l1_loss(out, torch.from_numpy(target).to(dev))
    loss.backward()
    torch.cuda.synchronize()
    fd = _fd_reference(clip, f, attr, target, rast.detach().cpu().numpy(), out.detach().cpu().numpy())
    pick = fd.pick_vertices(64)
    G = np.array([fd.grad_pos(j)[0] for j in pick])
    got = pos_t.grad.cpu().numpy()[pick]
    assert np.abs(got[:, 2]).max() <= 1e-12 * np.abs(G).max() and np.abs(G[:, 2]).max() == 0.0  # clip z: no gradient
    _gate(got, G, "clip-space position gradient", per_vertex=True)
    A = np.array([fd.grad_attr(j) for j in pick])
    _gate(attr_t.grad.cpu().numpy()[pick], A, "attribute gradient")
