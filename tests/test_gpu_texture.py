"""Mip-mapped texture sampling (nvdr.texture, csrc/texture.cu) against the
oracle (oracle/drp_oracle_tex.c, itself pinned against grid_sample and
float64 central differences in test_cpu_texture.py).

* the pyramid and every filter x boundary forward: bit-exact;
* gradients to the texture (through the pyramid), uv and uv_da: within 1e-5
  of the largest component of the oracle's float32 backward (float atomics
  change only the order of the texel sums);
* the derivatives interpolate() produces, fed to texture(): the drop-in
  chain rasterize -> interpolate(diff_attrs) -> texture, against the oracle;
* argument errors.
"""
import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu

FILTERS = ["nearest", "linear", "linear-mipmap-nearest", "linear-mipmap-linear"]
BOUNDARIES = ["wrap", "clamp", "zero", "mirror"]


def _case(Nt, N, H, W, C, h, w, seed=0):
    rng = np.random.default_rng(seed)
    tex = rng.uniform(-1, 1, (Nt, H, W, C)).astype(np.float32)
    uv = rng.uniform(-0.4, 1.4, (N, h, w, 2)).astype(np.float32)
    # footprints from below one texel to beyond the whole texture
    da = (rng.uniform(-1, 1, (N, h, w, 4)) * 2.0 ** rng.uniform(-2, np.log2(max(H, W)) + 1, (N, h, w, 1))
          / max(H, W)).astype(np.float32)
    return tex, uv, da


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_pyramid_matches_oracle(cuda_lib):
    from diffrp_gb300 import nvdr as dr
    for (Nt, H, W, C) in [(1, 64, 64, 4), (2, 37, 53, 3), (1, 1, 9, 2), (3, 16, 1, 1)]:
        tex = _case(Nt, 1, H, W, C, 1, 1)[0]
        mip = dr.texture_construct_mip(_t(tex))
        L = O.tex_levels(H, W)
        assert mip.levels == L
        ref = O.tex_mip_build(tex, L)
        n = ref.size if L > 1 else 0
        np.testing.assert_array_equal(mip.pyr.cpu().numpy()[:n], ref[:n])


@pytest.mark.parametrize("filter_mode", FILTERS)
@pytest.mark.parametrize("boundary", BOUNDARIES)
@pytest.mark.parametrize("Nt", [1, 2])
def test_forward_bit_exact(cuda_lib, filter_mode, boundary, Nt):
    from diffrp_gb300 import nvdr as dr
    H, W, C = 37, 53, 3
    tex, uv, da = _case(Nt, 2, H, W, C, 19, 23, seed=Nt)
    mipped = filter_mode.startswith("linear-mipmap")
    got = dr.texture(_t(tex), _t(uv), _t(da) if mipped else None, filter_mode=filter_mode, boundary_mode=boundary)
    L = O.tex_levels(H, W) if mipped else 1
    ref = O.tex_fwd(tex, O.tex_mip_build(tex, L), L, uv, da if mipped else None, filter_mode, boundary)
    np.testing.assert_array_equal(got.cpu().numpy(), ref)


# (textures, H, W, C): four channels take the float4 path; odd sizes, a
# size-1 axis and per-view textures the per-channel one; 3 x 4099 has 13
# levels (the pyramid gradient's longest chain variant)
GRAD_SHAPES = [(1, 32, 24, 4), (2, 37, 53, 3), (1, 1, 9, 2), (2, 20, 44, 4), (1, 3, 4099, 2)]


@pytest.mark.parametrize("shape", GRAD_SHAPES)
@pytest.mark.parametrize("filter_mode", FILTERS)
@pytest.mark.parametrize("boundary", BOUNDARIES)
def test_gradients_match_oracle(cuda_lib, filter_mode, boundary, shape):
    from diffrp_gb300 import nvdr as dr
    Nt, H, W, C = shape
    tex, uv, da = _case(Nt, 2, H, W, C, 17, 13, seed=5)
    mipped = filter_mode.startswith("linear-mipmap")
    gout = np.random.default_rng(9).normal(size=(2, 17, 13, C)).astype(np.float32)
    tex_t, uv_t = _t(tex).requires_grad_(True), _t(uv).requires_grad_(True)
    da_t = _t(da).requires_grad_(True) if mipped else None
    out = dr.texture(tex_t, uv_t, da_t, filter_mode=filter_mode, boundary_mode=boundary)
    out.backward(_t(gout))
    L = O.tex_levels(H, W) if mipped else 1
    pyr = O.tex_mip_build(tex, L)
    g0, gpyr, guv, gda = O.tex_bwd(tex, pyr, L, uv, da if mipped else None, gout, filter_mode, boundary)
    gtex = O.tex_mip_bwd(g0, gpyr, L)
    for got, ref, what in [(tex_t.grad, gtex, "tex"), (uv_t.grad, guv, "uv")] + \
            ([(da_t.grad, gda, "uv_da")] if mipped else []):
        got = got.cpu().numpy()
        scale = max(float(np.abs(ref).max()), 1e-30)
        assert float(np.abs(got - ref).max()) <= 1e-5 * scale, what
    if filter_mode == "linear-mipmap-linear":
        assert np.abs(gda).max() > 0  # the level of detail carries a gradient


def test_interpolated_derivatives_drive_the_level(cuda_lib):
    """rasterize -> interpolate(uv, diff_attrs) -> texture on a plane seen at
    a grazing angle: the trilinear result equals the oracle's on the same
    uv / uv_da, and far pixels sample coarser levels than near ones."""
    from diffrp_gb300 import nvdr as dr
    H = W = 128
    # a quad receding in depth, uv tiled 8 times
    pos = np.array([[-1, -1, 0.2, 1], [1, -1, 0.2, 1], [-4, 6, 0.9, 6], [4, 6, 0.9, 6]], np.float32)
    tri = np.array([[0, 1, 2], [1, 3, 2]], np.int32)
    uvs = np.array([[0, 0], [8, 0], [0, 8], [8, 8]], np.float32)
    ctx = dr.RasterizeCudaContext()
    rast, db = dr.rasterize(ctx, _t(pos), _t(tri), (H, W))
    uv, uv_da = dr.interpolate(_t(uvs), rast, _t(tri), rast_db=db, diff_attrs="all")
    rng = np.random.default_rng(2)
    tex = rng.uniform(0, 1, (1, 64, 64, 3)).astype(np.float32)
    got = dr.texture(_t(tex), uv, uv_da, filter_mode="linear-mipmap-linear", boundary_mode="wrap").cpu().numpy()
    L = O.tex_levels(64, 64)
    ref = O.tex_fwd(tex, O.tex_mip_build(tex, L), L, uv.cpu().numpy(), uv_da.cpu().numpy(), "linear-mipmap-linear",
                    "wrap")
    np.testing.assert_array_equal(got, ref)
    # far rows (top) average more texels: their values vary less than near rows
    cov = rast[0, ..., 3].cpu().numpy() > 0
    near, far = got[0, 4:20][cov[4:20]], got[0, -40:-20][cov[-40:-20]]
    assert near.size and far.size and far.std() < near.std()


def test_argument_errors(cuda_lib):
    from diffrp_gb300 import nvdr as dr
    tex, uv, da = _case(1, 1, 8, 8, 1, 4, 4)
    with pytest.raises(RuntimeError):  # the bias takes uv's shape without its last dimension
        dr.texture(_t(tex), _t(uv), _t(da), mip_level_bias=_t(da[..., :2]))
    with pytest.raises(ValueError):  # mip-mapped without uv_da or a bias
        dr.texture(_t(tex), _t(uv), filter_mode="linear-mipmap-linear")
    with pytest.raises(NotImplementedError):
        dr.texture(_t(tex), _t(uv), boundary_mode="cube")
    with pytest.raises(RuntimeError):
        dr.texture(_t(np.concatenate([tex, tex, tex])), _t(np.concatenate([uv, uv])))
    mip = dr.texture_construct_mip(_t(tex), max_mip_level=1)
    with pytest.raises(RuntimeError):
        dr.texture(_t(tex), _t(uv), _t(da), mip=mip)  # built for a different max_mip_level
    out = dr.texture(_t(tex), _t(uv), _t(da), mip=mip, max_mip_level=1)
    assert out.shape == (1, 4, 4, 1)


def test_sample_texture_keeps_sample2d_orientation(cuda_lib):
    """materials.sample_texture without derivatives is diffrp's sample2d
    (grid_sample with v flipped, border padding; diffrp/utils/shader_ops.py:
    199-255) restated: uv (0, 0) at the bottom-left image corner."""
    from diffrp_gb300.materials import sample_texture
    rng = np.random.default_rng(4)
    image = _t(rng.uniform(0, 1, (24, 40, 4)).astype(np.float32))
    uv = _t(rng.uniform(-0.2, 1.2, (300, 2)).astype(np.float32))
    got = sample_texture(image, uv, wrap="clamp")
    grid = ((uv * 2 - 1) * torch.tensor([1.0, -1.0], device="cuda")).reshape(1, 1, -1, 2)
    ref = torch.nn.functional.grid_sample(image[None].permute(0, 3, 1, 2), grid, mode="bilinear",
                                          padding_mode="border", align_corners=False).view(4, -1).T
    torch.testing.assert_close(got, ref, rtol=0, atol=2e-6)


def _ground_scene(material):
    from diffrp_gb300 import scene
    # a plane below the default camera (at z = 3.2, looking down -z),
    # receding to z = -8: uv tiled 8 x 40 across it
    verts = torch.tensor([[-2, -0.6, 2.0], [2, -0.6, 2.0], [-2, -0.6, -8.0], [2, -0.6, -8.0]], device="cuda")
    tris = torch.tensor([[0, 1, 2], [1, 3, 2]], dtype=torch.int32, device="cuda")
    uv = torch.tensor([[0, 0], [8, 0], [0, 40], [8, 40]], dtype=torch.float32, device="cuda")
    sc = scene.Scene()
    sc.add_mesh_object(scene.MeshObject(material, verts, tris, uv=uv))
    return sc


def test_session_textured_material_uses_derivatives(cuda_lib):
    """A textured ground plane through the session API: with derivatives the
    material samples mip-mapped, so the far, minified part of the plane is
    filtered (its albedo varies much less than with plain bilinear
    sampling); both interpolator implementations give the same images."""
    from diffrp_gb300.materials import TexturedMaterial
    from diffrp_gb300.rendering import camera
    from diffrp_gb300.rendering.surface_deferred import (SurfaceDeferredRenderSession,
                                                         SurfaceDeferredRenderSessionOptions)
    checker = ((np.indices((32, 32)).sum(0) % 2) * np.ones((4, 1, 1))).transpose(1, 2, 0).astype(np.float32)
    cam = camera.PerspectiveCamera(fov=40, h=96, w=128)
    images = {}
    for impl in ["full_screen", "stencil_masked"]:
        for deriv in [False, True]:
            sc = _ground_scene(TexturedMaterial(_t(checker)))
            opts = SurfaceDeferredRenderSessionOptions(interpolator_impl=impl, derivatives=deriv)
            s = SurfaceDeferredRenderSession(sc, cam, opaque_only=True, options=opts)
            images[impl, deriv] = s.albedo_layered()[0].cpu().numpy()[0]
    for deriv in [False, True]:
        np.testing.assert_allclose(images["full_screen", deriv], images["stencil_masked", deriv], rtol=0, atol=1e-6)
    plain, mipped = images["full_screen", False], images["full_screen", True]
    # the plane spans image rows 0 (near, bottom) to about 40 (far clip at
    # distance 10); rows 25-38 see 10-60 texels per pixel
    far_plain, far_mip = plain[25:38, 30:98, 0], mipped[25:38, 30:98, 0]
    assert far_mip.std() < 0.5 * far_plain.std()
    near = slice(0, 8)
    np.testing.assert_allclose(mipped[near].mean(), plain[near].mean(), atol=0.1)


def test_peeling_reads_emptiness_per_chunk(cuda_lib):
    """Unlimited layers over a stack of 6 parallel quads: 6 layers (the
    seventh is empty and dropped); a cap of 2 keeps 2, a cap of 9 keeps 6,
    and a cap of 7 keeps its last layer although it is empty (the reference
    loop, surface_deferred.py:258-266, drops an empty layer only before the
    last one)."""
    from diffrp_gb300 import scene, materials
    from diffrp_gb300.rendering import camera
    from diffrp_gb300.rendering.surface_deferred import (SurfaceDeferredRenderSession,
                                                         SurfaceDeferredRenderSessionOptions)
    cam = camera.PerspectiveCamera(fov=40, h=32, w=32)
    for cap, want in [(0, 6), (2, 2), (9, 6), (6, 6), (7, 7)]:
        sc = scene.Scene()
        for k in range(6):
            z = -0.5 * k
            verts = torch.tensor([[-1, -1, z], [1, -1, z], [-1, 1, z], [1, 1, z]], device="cuda")
            tris = torch.tensor([[0, 1, 2], [1, 3, 2]], dtype=torch.int32, device="cuda")
            sc.add_mesh_object(scene.MeshObject(materials.DefaultMaterial(), verts, tris))
        s = SurfaceDeferredRenderSession(sc, cam, opaque_only=False,
                                         options=SurfaceDeferredRenderSessionOptions(max_layers=cap))
        assert len(s.rasterize()) == want, (cap, len(s.rasterize()))


def test_full_size_receding_plane(cuda_lib):
    """The benchmark's texture workload at its full size: a 1024x1024 RGBA
    texture sampled trilinearly with wrap at the 1024x1024 pixels of a ground
    plane at a grazing angle (uv tiled 16 x 64, so most samples are minified
    onto the coarse levels, where the warp-aggregated atomics collide most).
    The forward is bit-exact against the oracle.  The texture's gradient
    (through the pyramid) agrees with the oracle's float64 backward within
    1e-4 of its largest component (float atomics against exact sums; it is
    continuous where a pixel's level changes).  The uv and uv_da gradients
    (per pixel, and uv_da's jumps where the level pair changes) agree with
    the float32 backward, whose level choices are the kernel's, within 1e-5."""
    from diffrp_gb300 import nvdr as dr
    n = 1024
    pos = np.array([[-1, -1, 0.2, 1], [1, -1, 0.2, 1], [-12, 16, 0.99, 16], [12, 16, 0.99, 16]], np.float32)
    tri = np.array([[0, 1, 2], [1, 3, 2]], np.int32)
    uvs = np.array([[0, 0], [16, 0], [0, 64], [16, 64]], np.float32)
    rast, db = dr.rasterize(dr.RasterizeCudaContext(), _t(pos), _t(tri), (n, n))
    uv, uv_da = dr.interpolate(_t(uvs), rast, _t(tri), rast_db=db, diff_attrs="all")
    rng = np.random.default_rng(11)
    tex = rng.uniform(0, 1, (1, n, n, 4)).astype(np.float32)
    gout = rng.uniform(0, 1, (1, n, n, 4)).astype(np.float32)
    tex_t = _t(tex).requires_grad_(True)
    uv_t = uv.detach().clone().requires_grad_(True)
    da_t = uv_da.detach().clone().requires_grad_(True)
    out = dr.texture(tex_t, uv_t, da_t, filter_mode="linear-mipmap-linear", boundary_mode="wrap")
    out.backward(_t(gout))
    uv_np, da_np = uv.cpu().numpy(), uv_da.cpu().numpy()
    L = O.tex_levels(n, n)
    ref = O.tex_fwd(tex, O.tex_mip_build(tex, L), L, uv_np, da_np, "linear-mipmap-linear", "wrap")
    np.testing.assert_array_equal(out.detach().cpu().numpy(), ref)
    pyr = O.tex_mip_build(tex, L, "f64")
    g0, gpyr, _, _ = O.tex_bwd(tex, pyr, L, uv_np, da_np, gout, "linear-mipmap-linear", "wrap", "f64")
    gtex = O.tex_mip_bwd(g0, gpyr, L, "f64")
    _, _, guv, gda = O.tex_bwd(tex, O.tex_mip_build(tex, L), L, uv_np, da_np, gout, "linear-mipmap-linear", "wrap")
    for got, want, what, tol in [(tex_t.grad, gtex, "tex", 1e-4), (uv_t.grad, guv, "uv", 1e-5),
                                 (da_t.grad, gda, "uv_da", 1e-5)]:
        got = got.cpu().numpy().astype(np.float64)
        scale = float(np.abs(want).max())
        assert scale > 0, what
        assert float(np.abs(got - want).max()) <= tol * scale, what


def _sample2d(image, uv, padding, mode):
    """diffrp's sample2d (diffrp/utils/shader_ops.py:199-255) restated:
    grid_sample with v flipped, align_corners=False."""
    C = image.shape[-1]
    grid = ((uv.reshape(-1, 2) * 2 - 1) * torch.tensor([1.0, -1.0], device=uv.device)).reshape(1, 1, -1, 2)
    out = torch.nn.functional.grid_sample(image[None].permute(0, 3, 1, 2), grid, mode=mode, padding_mode=padding,
                                          align_corners=False).view(C, -1).T
    return out.reshape(*uv.shape[:-1], C)


@pytest.mark.parametrize("wrap_mode", ["repeat", "clamp", "mirror"])
@pytest.mark.parametrize("interpolation", ["linear", "point"])
def test_gltf_sampler_matches_reference_without_derivatives(cuda_lib, wrap_mode, interpolation):
    """GLTFSampler.sample without derivatives is the reference's
    GLTFSampler.sample (diffrp/materials/gltf_material.py:15-22): 'repeat'
    takes uv modulo 1 and pads by reflection, 'clamp' pads by border,
    'mirror' by reflection; 'point' is grid_sample's nearest.  Samples keep
    away from exact nearest-texel ties (grid_sample rounds half to even).
    Tolerance 1e-5: grid_sample reflects the continuous coordinate in float
    arithmetic (up to 92 texels here, an ulp of 7.6e-6), the kernel mirrors
    integer texel indices, so bilinear weights differ by an ulp of x."""
    from diffrp_gb300.materials import GLTFSampler
    rng = np.random.default_rng(21)
    image = _t(rng.uniform(0, 1, (24, 40, 3)).astype(np.float32))
    uv = _t(rng.uniform(-1.3, 2.3, (50, 7, 2)).astype(np.float32))
    got = GLTFSampler(image, wrap_mode, interpolation).sample(uv)
    ref_uv = uv.remainder(1.0) if wrap_mode == "repeat" else uv
    ref = _sample2d(image, ref_uv, "border" if wrap_mode == "clamp" else "reflection",
                    "bilinear" if interpolation == "linear" else "nearest")
    torch.testing.assert_close(got, ref, rtol=0, atol=1e-5)


class _Fragments:
    """A SurfaceInput stand-in: uv, vertex colour and (optionally) uv_da."""

    def __init__(self, uv, color, uv_da=None):
        self.uv, self.color, self._da = uv, color, uv_da

    @property
    def uv_da(self):
        if self._da is None:
            raise RuntimeError("no derivatives")
        return self._da


def _gltf(rng, alpha_mode):
    from diffrp_gb300.materials import GLTFMaterial, GLTFSampler

    def img(c):
        return _t(rng.uniform(0, 1, (16, 24, c)).astype(np.float32))
    return GLTFMaterial(
        base_color_factor=_t(np.array([0.9, 0.8, 0.7, 0.6], np.float32)),
        base_color_texture=GLTFSampler(img(4), "repeat"),
        metallic_factor=0.7, roughness_factor=0.4,
        metallic_roughness_texture=GLTFSampler(img(3), "mirror"),
        normal_texture=GLTFSampler(img(3), "clamp"),
        occlusion_texture=GLTFSampler(img(1), "repeat", "point"),
        emissive_factor=_t(np.array([0.5, 0.25, 1.0], np.float32)),
        emissive_texture=GLTFSampler(img(3), "clamp"),
        alpha_cutoff=0.3, alpha_mode=alpha_mode)


@pytest.mark.parametrize("alpha_mode", ["OPAQUE", "MASK", "BLEND"])
def test_gltf_material_shade_matches_reference(cuda_lib, alpha_mode):
    """GLTFMaterial.shade without derivatives against the reference's shade
    (diffrp/materials/gltf_material.py:44-67) restated on sample2d; with
    derivatives every 'linear' texture is sampled trilinearly, equal to the
    oracle on the same (remaindered, mirrored) coordinates."""
    rng = np.random.default_rng(22)
    m = _gltf(rng, alpha_mode)
    n = 500
    uv = _t(rng.uniform(-0.5, 1.5, (n, 2)).astype(np.float32))
    color = _t(rng.uniform(0.5, 1, (n, 4)).astype(np.float32))
    out = m.shade(None, _Fragments(uv, color))

    def ref_sample(s, uv_):
        u2 = uv_.remainder(1.0) if s.wrap_mode == "repeat" else uv_
        return _sample2d(s.image, u2, "border" if s.wrap_mode == "clamp" else "reflection",
                         "bilinear" if s.interpolation == "linear" else "nearest")
    rgba = m.base_color_factor * color * ref_sample(m.base_color_texture, uv)
    mr = ref_sample(m.metallic_roughness_texture, uv)
    want = {"albedo": rgba[..., :3], "normal": 2 * ref_sample(m.normal_texture, uv) - 1,
            "emission": m.emissive_factor * ref_sample(m.emissive_texture, uv),
            "metallic": m.metallic_factor * mr[..., 2:3], "smoothness": 1.0 - m.roughness_factor * mr[..., 1:2],
            "occlusion": ref_sample(m.occlusion_texture, uv)[..., :1]}
    if alpha_mode == "MASK":
        want["alpha"] = (rgba[..., 3:4] > m.alpha_cutoff).float()
    elif alpha_mode == "BLEND":
        want["alpha"] = rgba[..., 3:4]
    else:
        assert out.alpha is None
    for k, v in want.items():
        torch.testing.assert_close(getattr(out, k), v, rtol=0, atol=1e-5, msg=k)
    # with derivatives: trilinear, against the oracle
    da = _t((rng.uniform(-1, 1, (n, 4)) * 2.0 ** rng.uniform(-2, 5, (n, 1)) / 24).astype(np.float32))
    out_d = m.shade(None, _Fragments(uv, color, da))
    s = m.emissive_texture  # clamp, linear
    img = s.image.cpu().numpy()[None]
    L = O.tex_levels(16, 24)
    uv_t = torch.stack([uv[:, 0], 1 - uv[:, 1]], -1).cpu().numpy().reshape(1, 1, n, 2)
    da_t = (da * _t(np.array([1, 1, -1, -1], np.float32))).cpu().numpy().reshape(1, 1, n, 4)
    ref = O.tex_fwd(img, O.tex_mip_build(img, L), L, uv_t, da_t, "linear-mipmap-linear", "clamp").reshape(n, 3)
    np.testing.assert_allclose(out_d.emission.cpu().numpy(), m.emissive_factor.cpu().numpy() * ref, rtol=0,
                               atol=1e-6)


def test_session_gltf_material_with_derivatives(cuda_lib):
    """A glTF-textured ground plane through the session: trained base colour
    texture (requires_grad) gets gradients through the mip pyramid; the
    minified far part is filtered with derivatives."""
    from diffrp_gb300.materials import GLTFMaterial, GLTFSampler
    from diffrp_gb300.rendering import camera
    from diffrp_gb300.rendering.surface_deferred import (SurfaceDeferredRenderSession,
                                                         SurfaceDeferredRenderSessionOptions)
    checker = ((np.indices((32, 32)).sum(0) % 2) * np.ones((4, 1, 1))).transpose(1, 2, 0).astype(np.float32)
    cam = camera.PerspectiveCamera(fov=40, h=96, w=128)
    images = {}
    for deriv in [False, True]:
        base = _t(checker).requires_grad_(True)
        white = _t(np.ones((4, 4, 3), np.float32))
        m = GLTFMaterial(_t(np.ones(4, np.float32)), GLTFSampler(base, "repeat"), 0.0, 1.0, GLTFSampler(white),
                         None, None, None, GLTFSampler(white), 0.5, "OPAQUE")
        s = SurfaceDeferredRenderSession(_ground_scene(m), cam, opaque_only=True,
                                         options=SurfaceDeferredRenderSessionOptions(derivatives=deriv))
        img = s.albedo_layered()[0]
        img.sum().backward()
        assert base.grad is not None and float(base.grad.abs().sum()) > 0
        images[deriv] = img.detach().cpu().numpy()[0]
    far_plain, far_mip = images[False][25:38, 30:98, 0], images[True][25:38, 30:98, 0]
    assert far_mip.std() < 0.5 * far_plain.std()


@pytest.mark.parametrize("with_da", [False, True])
@pytest.mark.parametrize("filter_mode", ["linear-mipmap-nearest", "linear-mipmap-linear"])
def test_mip_level_bias(cuda_lib, with_da, filter_mode):
    """nvdiffrast's mip_level_bias: added to the level of detail from uv_da
    (alone, it sets it).  Forward bit-exact against the oracle; gradients to
    the texture, uv, uv_da and the bias within 1e-5 of the largest."""
    from diffrp_gb300 import nvdr as dr
    H, W, C = 32, 24, 4
    tex, uv, da = _case(1, 2, H, W, C, 17, 13, seed=6)
    rng = np.random.default_rng(10)
    bias = rng.uniform(-1.5, 5.5, (2, 17, 13)).astype(np.float32)
    gout = rng.normal(size=(2, 17, 13, C)).astype(np.float32)
    tex_t, uv_t, b_t = _t(tex).requires_grad_(True), _t(uv).requires_grad_(True), _t(bias).requires_grad_(True)
    da_t = _t(da).requires_grad_(True) if with_da else None
    out = dr.texture(tex_t, uv_t, da_t, mip_level_bias=b_t, filter_mode=filter_mode, boundary_mode="wrap")
    L = O.tex_levels(H, W)
    pyr = O.tex_mip_build(tex, L)
    da_np = da if with_da else None
    ref = O.tex_fwd(tex, pyr, L, uv, da_np, filter_mode, "wrap", bias=bias)
    np.testing.assert_array_equal(out.detach().cpu().numpy(), ref)
    out.backward(_t(gout))
    g0, gpyr, guv, gda, gb = O.tex_bwd(tex, pyr, L, uv, da_np, gout, filter_mode, "wrap", bias=bias)
    gtex = O.tex_mip_bwd(g0, gpyr, L)
    pairs = [(tex_t.grad, gtex, "tex"), (uv_t.grad, guv, "uv"), (b_t.grad, gb, "bias")]
    if with_da:
        pairs.append((da_t.grad, gda, "uv_da"))
    for got, want, what in pairs:
        got = got.cpu().numpy()
        scale = max(float(np.abs(want).max()), 1e-30)
        assert float(np.abs(got - want).max()) <= 1e-5 * scale, what
    if filter_mode == "linear-mipmap-linear":
        assert np.abs(gb).max() > 0


def test_material_pyramid_follows_the_image(cuda_lib):
    """A sampler's cached pyramid is rebuilt when its image is modified in
    place or replaced, so trilinear samples always see the current image."""
    from diffrp_gb300.materials import GLTFSampler
    rng = np.random.default_rng(12)
    image = _t(rng.uniform(0, 1, (16, 16, 3)).astype(np.float32))
    uv = _t(rng.uniform(0, 1, (64, 2)).astype(np.float32))
    da = _t(np.full((64, 4), 0.2, np.float32))  # minified: coarse levels
    s = GLTFSampler(image, "repeat")
    first = s.sample(uv, da)
    with torch.no_grad():
        image.mul_(0.5)
    torch.testing.assert_close(s.sample(uv, da), 0.5 * first, rtol=1e-6, atol=1e-6)
    s.image = torch.zeros_like(image)
    assert float(s.sample(uv, da).abs().max()) == 0.0
