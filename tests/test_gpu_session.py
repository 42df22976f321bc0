"""Session-level parity on the GPU: diffrp_gb300's Scene / MeshObject /
PerspectiveCamera / SurfaceDeferredRenderSession against golden vectors made
by running the reference diffrp session code (tests/golden/make_golden.py).

Each scenario is rebuilt from the stored inputs with this package's API and
rendered on cuda:0 through the CUDA kernels.  The clip-space transform runs on
different hardware on the two sides (CPU matmul in the generator, GPU here),
so a pixel whose centre sits on a triangle edge may flip; the bar is:
  - clip-space vertices within 1e-6 relative;
  - at least 99.5% of pixels with the same triangle id;
  - outputs within 2e-5 where the pixel and its 4 neighbours agree on ids;
  - gradients within 1e-3 of the largest reference gradient magnitude
    (3e-3 for config 1, whose 512x512 image has more edge pixels).
With the reference's own clip-space vertices injected into the session
(forward value replaced, gradient passed straight through to this package's
clip transform) the visibility is the same on both sides, and the bar is:
  - the raster buffer bit-identical;
  - outputs within 2e-5 on every pixel;
  - gradients within 1e-4 of the largest reference gradient magnitude.
Config 1 (icosphere with 3 subdivisions, 512x512, camera-space normals
through nvdr_antialias, L2 loss) is checked against the signature stored by
make_golden.py (ids, raster hash, row sums, a pixel sample, loss, gradients).
"""
import os

import numpy as np
import pytest
import torch

from tests.golden import make_golden

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCENARIOS = ["normals", "objects_masked", "objects_full", "layers"]
GRAD_RTOL = 1e-4  # injected clip space: visibility identical on both sides
GRAD_RTOL_OWN_CLIP = 1e-3  # own clip transform: a few edge pixels flip
# config 1 with its own clip transform: 512x512 and 1280 face-soup triangles
# put more pixels on edges, and each flipped silhouette pixel moves the
# gradient of its triangle's vertices
GRAD_RTOL_OWN_CLIP_C1 = 3e-3


def _api():
    from diffrp_gb300 import materials, scene
    from diffrp_gb300.rendering import camera
    return dict(Scene=scene.Scene, MeshObject=scene.MeshObject, DefaultMaterial=materials.DefaultMaterial,
                SurfaceMaterial=materials.SurfaceMaterial, SurfaceOutputStandard=materials.SurfaceOutputStandard,
                PerspectiveCamera=camera.PerspectiveCamera, device="cuda")


def _load(name):
    z = np.load(os.path.join(GOLDEN, "session_%s.npz" % name))
    inputs = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    outs = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return inputs, outs


def _stable_mask(ids_a, ids_b):
    same = ids_a == ids_b
    st = same.copy()
    st[1:] &= same[:-1]
    st[:-1] &= same[1:]
    st[:, 1:] &= same[:, :-1]
    st[:, :-1] &= same[:, 1:]
    return same, st


class _Inject(torch.autograd.Function):
    """Forward: the injected tensor; backward: the gradient passed straight
    to the computed one."""

    @staticmethod
    def forward(ctx, computed, injected):
        return injected.clone()

    @staticmethod
    def backward(ctx, g):
        return g, None


def _injector(ref_clip):
    from diffrp_gb300.rendering.surface_deferred import SurfaceDeferredRenderSession
    key = SurfaceDeferredRenderSession.clip_space.__qualname__

    def hook(rp):
        computed = rp.clip_space()
        rp._cache[key] = _Inject.apply(computed, torch.from_numpy(ref_clip).to(computed.device))
    return hook


def _render(name, inject=False):
    from diffrp_gb300.rendering.surface_deferred import (SurfaceDeferredRenderSession,
                                                         SurfaceDeferredRenderSessionOptions)
    d, ref = _load(name)
    if name not in ("normals", "c1"):
        d["impl"] = "full_screen" if name == "objects_full" else "stencil_masked"
    if name == "layers":
        d["alpha"] = float(d["alpha"])
    hook = _injector(ref["clip"]) if inject else None
    got = make_golden.render(_api(), d, name, SurfaceDeferredRenderSession, SurfaceDeferredRenderSessionOptions,
                             on_session=hook)
    return d, ref, got


def _grad_gate(got, ref, rtol):
    for key in [k for k in ref if k.startswith("grad_")]:
        g, r = got[key], ref[key]
        scale = max(np.abs(r).max(), 1e-12)
        err = np.abs(g.astype(np.float64) - r).max() / scale
        assert err <= rtol, "%s relative error %g (bar %g)" % (key, err, rtol)


@pytest.mark.parametrize("name", SCENARIOS)
def test_session_matches_reference(cuda_lib, name):
    d, ref, got = _render(name)

    np.testing.assert_allclose(got["clip"], ref["clip"], rtol=1e-6, atol=1e-6)
    ids_g = got["rast"][0, ..., 3]
    ids_r = ref["rast"][0, ..., 3]
    same, stable = _stable_mask(ids_g, ids_r)
    assert same.mean() >= 0.995, "only %.4f of pixels agree on triangle id" % same.mean()
    stable_img = np.flipud(stable)  # composed images are top-down
    for key in ["normals", "aa", "albedo", "world_position", "depth", "world_normal", "aov"]:
        if key not in ref or ref[key].size == 0:
            continue
        diff = np.abs(got[key] - ref[key])[stable_img]
        assert diff.max() <= 2e-5, "%s differs by %g on stable pixels" % (key, diff.max())
    if "n_layers" in ref:
        assert int(got["n_layers"]) == int(ref["n_layers"])
    _grad_gate(got, ref, GRAD_RTOL_OWN_CLIP)


@pytest.mark.parametrize("name", SCENARIOS)
def test_session_clip_injected_matches_reference(cuda_lib, name):
    """The reference's clip space injected: raster bit-identical, every
    output pixel within 2e-5, gradients to every leaf within 1e-4."""
    d, ref, got = _render(name, inject=True)
    np.testing.assert_array_equal(got["clip"], ref["clip"])
    np.testing.assert_array_equal(got["rast"], ref["rast"])
    for key in ["normals", "aa", "albedo", "world_position", "depth", "world_normal", "aov"]:
        if key not in ref or ref[key].size == 0:
            continue
        diff = np.abs(got[key] - ref[key])
        assert diff.max() <= 2e-5, "%s differs by %g" % (key, diff.max())
    if "n_layers" in ref:
        assert int(got["n_layers"]) == int(ref["n_layers"])
    _grad_gate(got, ref, GRAD_RTOL)


def _c1_check(got, ref, inject):
    sig = make_golden.c1_signature(got)
    ids_g, ids_r = sig["ids"], ref["ids"]
    if inject:
        np.testing.assert_array_equal(sig["clip"], ref["clip"])
        np.testing.assert_array_equal(ids_g, ids_r)
        assert bytes(sig["rast_sha256"]) == bytes(ref["rast_sha256"]), "raster buffer differs"
        np.testing.assert_array_equal(sig["rast_sample"], ref["rast_sample"])
        np.testing.assert_allclose(sig["rast_rowsum"], ref["rast_rowsum"], rtol=1e-12, atol=1e-12)
        for key in ("normals", "aa"):
            assert np.abs(sig[key + "_sample"] - ref[key + "_sample"]).max() <= 2e-5, key
            assert np.abs(sig[key + "_rowsum"] - ref[key + "_rowsum"]).max() <= 512 * 2e-5, key
        assert abs(float(sig["loss"]) - float(ref["loss"])) <= 1e-5 * float(ref["loss"])
        rtol = GRAD_RTOL
    else:
        np.testing.assert_allclose(sig["clip"], ref["clip"], rtol=1e-6, atol=1e-6)
        assert (ids_g == ids_r).mean() >= 0.995
        assert abs(float(sig["loss"]) - float(ref["loss"])) <= 1e-3 * float(ref["loss"])
        rtol = GRAD_RTOL_OWN_CLIP_C1
    scale = np.abs(ref["grad_verts"]).max()
    err = np.abs(sig["grad_verts"].astype(np.float64) - ref["grad_verts"]).max() / scale
    assert err <= rtol, "grad_verts relative error %g (bar %g)" % (err, rtol)


@pytest.mark.parametrize("inject", [True, False], ids=["clip_injected", "own_clip"])
def test_session_config1_matches_reference(cuda_lib, inject):
    """Config 1 at its size: 642-vertex icosphere (face soup: 3840 vertices),
    512x512, far 100, camera-space normals, nvdr_antialias, L2 loss to a
    seeded N(0, 0.1) target, gradients to the leaf vertices."""
    d, ref, got = _render("c1", inject=inject)
    _c1_check(got, ref, inject)

