"""Edge-gradient operator: the CUDA backward against the reference's own
_EdgeGradient.backward (diffrp/rendering/surface_deferred.py:126-169) on the
golden inputs made by tests/golden/make_golden.py, and the session method
end to end."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "edge_gradient.npz")


def test_edge_gradient_backward_matches_reference(cuda_lib):
    from diffrp_gb300.rendering.edge_gradient import EdgeGradientFn
    g = np.load(GOLDEN)
    t = lambda k: torch.from_numpy(g[k]).cuda()  # noqa: E731
    frag = t("frag_xy").requires_grad_(True)
    rgb = t("rgb").requires_grad_(True)
    out = EdgeGradientFn.apply(frag, t("flat_tris_xy"), t("rast"), rgb)
    assert torch.equal(out.detach(), t("rgb"))
    out.backward(t("grad_out"))
    ref = g["grad_frag_xy"]
    got = frag.grad.cpu().numpy()
    assert (np.abs(ref) > 0).sum() > 50
    np.testing.assert_array_equal(got != 0, ref != 0)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    np.testing.assert_array_equal(rgb.grad.cpu().numpy(), g["grad_rgb"])


def test_session_edge_gradient_runs_end_to_end(cuda_lib):
    from diffrp_gb300.materials import DefaultMaterial
    from diffrp_gb300.rendering import PerspectiveCamera, SurfaceDeferredRenderSession
    from diffrp_gb300.scene import MeshObject, Scene
    from diffrp_gb300 import synthetic as S
    v, f = S.icosphere(2, 0.8)
    verts = torch.from_numpy(v).cuda().requires_grad_(True)
    scene = Scene().add_mesh_object(MeshObject(DefaultMaterial(), verts, torch.from_numpy(f).cuda()))
    rp = SurfaceDeferredRenderSession(scene, PerspectiveCamera(h=64, w=64, far=100.0))
    img = rp.false_color_camera_space_normal()[..., :3]
    out = rp.edge_gradient(img)
    assert torch.equal(out, img)
    (out * torch.linspace(-1, 1, out.numel(), device="cuda").reshape(out.shape)).sum().backward()
    assert torch.isfinite(verts.grad).all()
