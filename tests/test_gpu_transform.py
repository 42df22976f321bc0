"""Clip-space transform kernels (drp_transform_points_fwd / _bwd) against a
float64 restatement of [v, 1] @ M^T (diffrp/utils/shader_ops.py:123-136, as
used by diffrp/rendering/surface_deferred.py:229-238).

Tolerances: the forward is three fused multiply-adds per output in float32,
so each output is within 4 ulp-scale units of the float64 product (bound
below: 2e-7 x the sum of |terms|); the backward sums B views in float32, so
the bound grows with B (1e-6 x B x the sum of |terms|).
"""
import numpy as np
import pytest
import torch

from diffrp_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _views(n, H=512, W=512, seed=0):
    rng = np.random.default_rng(seed)
    P = S.perspective(35.0, H, W, 0.1, 50.0).astype(np.float64)
    out = []
    for _ in range(n):
        az, el = rng.uniform(0, 2 * np.pi), rng.uniform(-1.0, 1.0)
        eye = 3.0 * np.array([np.cos(az) * np.cos(el), np.sin(az) * np.cos(el), np.sin(el)])
        out.append((P @ S.view_matrix(S.lookat_pose(eye, up=(0.0, 0.0, 1.0))).astype(np.float64)).astype(np.float32))
    return np.stack(out)


def _fwd_ref(v, m):
    vh = np.concatenate([v.astype(np.float64), np.ones((len(v), 1))], 1)
    return np.einsum("vj,bij->bvi", vh, m.astype(np.float64)), np.einsum("vj,bij->bvi", np.abs(vh), np.abs(m.astype(np.float64)))


def test_forward_and_vertex_gradient(cuda_lib):
    from diffrp_gb300.transform import clip_space
    rng = np.random.default_rng(1)
    for V, B in [(1, 1), (257, 3), (10242, 16), (40962, 64)]:
        v = rng.uniform(-1, 1, (V, 3)).astype(np.float32)
        m = _views(B, seed=V)
        vt = torch.from_numpy(v).cuda().requires_grad_(True)
        mt = torch.from_numpy(m).cuda()
        out = clip_space(vt, mt)
        assert out.shape == (B, V, 4)
        ref, mag = _fwd_ref(v, m)
        assert (np.abs(out.detach().cpu().numpy() - ref) <= 2e-7 * mag + 1e-30).all()
        g = rng.standard_normal((B, V, 4)).astype(np.float32)
        out.backward(torch.from_numpy(g).cuda())
        gref = np.einsum("bvi,bij->vj", g.astype(np.float64), m.astype(np.float64))[:, :3]
        gmag = np.einsum("bvi,bij->vj", np.abs(g.astype(np.float64)), np.abs(m.astype(np.float64)))[:, :3]
        assert (np.abs(vt.grad.cpu().numpy() - gref) <= 1e-6 * B * gmag + 1e-30).all()
        # the single-matrix form gives (V, 4)
        one = clip_space(vt.detach(), mt[0])
        assert one.shape == (V, 4) and torch.equal(one, out[0].detach())


def test_reproducible_gradient(cuda_lib):
    from diffrp_gb300.transform import clip_space
    v = torch.rand(5000, 3, device="cuda", requires_grad=True)
    m = torch.from_numpy(_views(32)).cuda()
    g = torch.randn(32, 5000, 4, device="cuda")
    grads = []
    for _ in range(3):
        v.grad = None
        clip_space(v, m).backward(g)
        grads.append(v.grad.clone())
    assert torch.equal(grads[0], grads[1]) and torch.equal(grads[1], grads[2])


def test_packed_groups_and_matrix_gradient(cuda_lib):
    from diffrp_gb300.transform import clip_space, clip_space_packed
    rng = np.random.default_rng(2)
    v0 = torch.from_numpy(rng.uniform(-1, 1, (1001, 3)).astype(np.float32)).cuda().requires_grad_(True)
    v1 = torch.from_numpy(rng.uniform(-1, 1, (77, 3)).astype(np.float32)).cuda().requires_grad_(True)
    v2 = torch.zeros(0, 3, device="cuda", requires_grad=True)
    m0 = torch.from_numpy(_views(5, seed=3)).cuda().requires_grad_(True)
    m1 = torch.from_numpy(_views(1, seed=4)[0]).cuda()
    m2 = torch.from_numpy(_views(2, seed=5)).cuda()
    out = clip_space_packed([(v0, m0), (v1, m1), (v2, m2)])
    assert out.shape == (5 * 1001 + 77, 4)
    assert torch.equal(out[:5 * 1001].detach(), clip_space(v0.detach(), m0.detach()).reshape(-1, 4))
    assert torch.equal(out[5 * 1001:].detach(), clip_space(v1.detach(), m1))
    g = torch.randn_like(out)
    out.backward(g)
    # the same sums through torch's own ops, in float64
    def torch_ref(v, m):
        vh = torch.nn.functional.pad(v.double(), (0, 1), value=1.0)
        return torch.matmul(vh, m.double().transpose(-1, -2)).reshape(-1, 4)
    a0 = v0.detach().double().requires_grad_(True)
    b0 = m0.detach().double().requires_grad_(True)
    a1 = v1.detach().double().requires_grad_(True)
    ref = torch.cat([torch_ref(a0, b0), torch_ref(a1, m1)])
    ref.backward(g.double())
    torch.testing.assert_close(v0.grad.double(), a0.grad, rtol=1e-5, atol=1e-5)
    torch.testing.assert_close(v1.grad.double(), a1.grad, rtol=1e-5, atol=1e-5)
    torch.testing.assert_close(m0.grad.double(), b0.grad, rtol=1e-4, atol=1e-3)
    assert v2.grad.shape == (0, 3)


def test_bad_arguments(cuda_lib):
    from diffrp_gb300 import _ffi
    from diffrp_gb300.transform import clip_space
    with pytest.raises(RuntimeError):
        clip_space(torch.zeros(4, 4, device="cuda"), torch.eye(4, device="cuda"))
    with pytest.raises(RuntimeError):
        clip_space(torch.zeros(4, 3, device="cuda"), torch.eye(4, device="cuda", dtype=torch.float64))
    v = torch.zeros(8, 3, device="cuda")
    out = torch.empty(40, device="cuda")
    # a float4 output row that is not 16-byte aligned is rejected before launch
    with pytest.raises(RuntimeError):
        _ffi.call("drp_transform_points_fwd", v.data_ptr(), 8, torch.eye(4, device="cuda").data_ptr(), 1,
                  out.data_ptr() + 4, 0)
