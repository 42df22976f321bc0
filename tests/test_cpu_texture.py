"""The texture-sampling oracle (oracle/drp_oracle_tex.c) against independent
references, on the CPU.

* bilinear sampling with clamp / zero / mirror boundaries against
  torch.nn.functional.grid_sample (align_corners=False, border / zeros /
  reflection padding): the same texel-centre convention, computed by other
  code (mirrored repeat of the bilinear taps equals reflecting the
  coordinate about the texture's edges);
* wrap against clamp on a texture tiled three times;
* the mip pyramid against a numpy 2x2 reshape-mean (even sizes) and the
  size-1 rule (odd and degenerate sizes);
* the level-of-detail log2 against math.log2;
* every gradient (texture through the pyramid, uv, uv_da) against float64
  central differences of the float64 build.
"""
import math

import numpy as np
import pytest
import torch

import oracle as O


def _tex(N, H, W, C, seed=0):
    return np.random.default_rng(seed).uniform(-1, 1, (N, H, W, C)).astype(np.float32)


def _uv(N, h, w, lo=-0.2, hi=1.2, seed=1):
    return np.random.default_rng(seed).uniform(lo, hi, (N, h, w, 2)).astype(np.float32)


@pytest.mark.parametrize("boundary,padding", [("clamp", "border"), ("zero", "zeros"), ("mirror", "reflection")])
def test_bilinear_matches_grid_sample(boundary, padding):
    tex = _tex(2, 13, 17, 3)
    uv = _uv(2, 9, 11)
    got = O.tex_fwd(tex, O.tex_mip_build(tex, 1), 1, uv, None, "linear", boundary)
    grid = torch.from_numpy(uv * 2 - 1).double()
    ref = torch.nn.functional.grid_sample(torch.from_numpy(tex).double().permute(0, 3, 1, 2), grid, mode="bilinear",
                                          padding_mode=padding, align_corners=False).permute(0, 2, 3, 1).numpy()
    np.testing.assert_allclose(got, ref, rtol=0, atol=2e-6)


def test_wrap_is_clamp_on_a_tiled_texture():
    tex = _tex(1, 8, 6, 2)
    tiled = np.tile(tex, (1, 3, 3, 1))
    uv = _uv(1, 7, 7, lo=-0.9, hi=1.9)
    wrap = O.tex_fwd(tex, O.tex_mip_build(tex, 1), 1, uv, None, "linear", "wrap")
    clamp = O.tex_fwd(tiled, O.tex_mip_build(tiled, 1), 1, (uv + 1) / 3, None, "linear", "clamp")
    np.testing.assert_allclose(wrap, clamp, rtol=0, atol=2e-5)


def test_nearest_picks_the_texel_containing_uv():
    tex = _tex(1, 4, 5, 1)
    uv = np.array([[[[0.05, 0.05], [0.95, 0.95], [0.39, 0.51]]]], np.float32)
    got = O.tex_fwd(tex, O.tex_mip_build(tex, 1), 1, uv, None, "nearest", "clamp")[0, 0, :, 0]
    np.testing.assert_array_equal(got, [tex[0, 0, 0, 0], tex[0, 3, 4, 0], tex[0, 2, 1, 0]])


def test_mip_pyramid_levels():
    tex = _tex(1, 16, 8, 2)
    L = O.tex_levels(16, 8)
    assert L == 5  # 16x8, 8x4, 4x2, 2x1, 1x1
    pyr = O.tex_mip_build(tex, L, precision="f64")
    off, h, w, lvl = 0, 16, 8, tex[0].astype(np.float64)
    for k in range(L):
        if k > 0:  # level 0 is the texture itself
            got = pyr[off:off + h * w * 2].reshape(h, w, 2)
            np.testing.assert_allclose(got, lvl, rtol=0, atol=1e-12)
            off += h * w * 2
        if k + 1 < L:
            if w == 1:
                lvl = np.concatenate([lvl, lvl], axis=1)
            lvl = lvl.reshape(h // 2, 2, max(w // 2, 1), 2, 2).mean(axis=(1, 3))
            h, w = max(h // 2, 1), max(w // 2, 1)
    assert O.tex_levels(1024, 1024) == 11 and O.tex_levels(1024, 1024, 3) == 4 and O.tex_levels(5, 7) == 3


def test_level_of_detail_log2():
    # the pyramid level chosen from uv_da follows 0.5 log2(footprint^2)
    H = W = 64
    L = O.tex_levels(H, W)
    tex = np.zeros((1, H, W, 1), np.float32)
    pyr = O.tex_mip_build(tex, L)
    # a constant level index image: level k holds the value k
    off = 0
    for k in range(1, L):
        n = max(H >> k, 1) * max(W >> k, 1)
        pyr[off:off + n] = k
        off += n
    rng = np.random.default_rng(3)
    lam = rng.uniform(0.0, L - 1.0, 200)
    scale = 2.0 ** lam / W
    uv = np.full((1, 1, 200, 2), 0.5, np.float32)
    da = np.zeros((1, 1, 200, 4), np.float32)
    da[0, 0, :, 0] = scale
    got = O.tex_fwd(tex, pyr, L, uv, da, "linear-mipmap-linear", "clamp")[0, 0, :, 0]
    ref = np.array([0.5 * math.log2(float(np.float32(s) * W) ** 2) for s in scale])
    np.testing.assert_allclose(got, ref, rtol=0, atol=3e-6)


def _central(fn, x, idx, eps):
    xp, xm = x.copy(), x.copy()
    xp[idx] += eps
    xm[idx] -= eps
    return (fn(xp) - fn(xm)) / (2 * eps)


@pytest.mark.parametrize("filter_mode", ["linear", "linear-mipmap-nearest", "linear-mipmap-linear"])
@pytest.mark.parametrize("boundary", ["wrap", "clamp", "zero", "mirror"])
def test_gradients_match_central_differences(filter_mode, boundary):
    H, W, C = 12, 10, 3
    L = O.tex_levels(H, W)
    rng = np.random.default_rng(7)
    tex = rng.uniform(-1, 1, (1, H, W, C))
    uv = rng.uniform(-0.3, 1.3, (2, 3, 4, 2))
    da = rng.uniform(-0.3, 0.3, (2, 3, 4, 4)) / W * 2.0 ** rng.uniform(0.3, 2.7, (2, 3, 4, 1))
    gout = rng.normal(size=(2, 3, 4, C))

    def loss(tex_, uv_, da_):
        pyr = O.tex_mip_build(tex_, L, "f64")
        return float((O.tex_fwd(tex_, pyr, L, uv_, da_, filter_mode, boundary, "f64") * gout).sum())

    pyr = O.tex_mip_build(tex, L, "f64")
    g0, gpyr, guv, gda = O.tex_bwd(tex, pyr, L, uv, da, gout, filter_mode, boundary, "f64")
    gtex = O.tex_mip_bwd(g0, gpyr, L, "f64")
    eps = 1e-6
    for idx in [(0, 0, 0, 0), (0, 5, 3, 1), (0, 11, 9, 2), (0, 6, 0, 0)]:
        fd = _central(lambda t: loss(t, uv, da), tex, idx, eps)
        assert abs(gtex[idx] - fd) <= 1e-6 + 1e-6 * abs(fd), ("tex", idx, gtex[idx], fd)
    for idx in [(0, 0, 0, 0), (1, 2, 3, 1), (1, 1, 2, 0)]:
        fd = _central(lambda x: loss(tex, x, da), uv, idx, eps)
        assert abs(guv[idx] - fd) <= 1e-5 * max(1.0, abs(fd)), ("uv", idx, guv[idx], fd)
    for idx in [(0, 0, 1, 0), (1, 2, 2, 1), (0, 2, 3, 2), (1, 0, 0, 3)]:
        fd = _central(lambda d: loss(tex, uv, d), da, idx, 1e-8)
        assert abs(gda[idx] - fd) <= 1e-4 * max(1.0, abs(fd)), ("uv_da", idx, gda[idx], fd)


def test_mip_level_bias_shifts_the_level():
    """The per-pixel mip level bias adds to the level of detail (alone it
    sets it), clamped to the pyramid: a level-index pyramid (level k holds
    k) returns lambda itself under trilinear filtering."""
    H = W = 64
    L = O.tex_levels(H, W)
    tex = np.zeros((1, H, W, 1), np.float32)
    pyr = O.tex_mip_build(tex, L)
    off = 0
    for k in range(1, L):
        n = max(H >> k, 1) * max(W >> k, 1)
        pyr[off:off + n] = k
        off += n
    rng = np.random.default_rng(5)
    n = 200
    uv = np.full((1, 1, n, 2), 0.5, np.float32)
    bias = rng.uniform(-2.0, L + 1.0, (1, 1, n)).astype(np.float32)
    got = O.tex_fwd(tex, pyr, L, uv, None, "linear-mipmap-linear", "clamp", bias=bias)[0, 0, :, 0]
    np.testing.assert_allclose(got, np.clip(bias[0, 0], 0, L - 1), rtol=0, atol=2e-6)
    lam = rng.uniform(0.0, 3.0, n)
    da = np.zeros((1, 1, n, 4), np.float32)
    da[0, 0, :, 0] = 2.0 ** lam / W
    bias = rng.uniform(-1.0, 2.0, (1, 1, n)).astype(np.float32)
    got = O.tex_fwd(tex, pyr, L, uv, da, "linear-mipmap-linear", "clamp", bias=bias)[0, 0, :, 0]
    ref = np.array([0.5 * math.log2(float(np.float32(s) * W) ** 2) for s in da[0, 0, :, 0]]) + bias[0, 0]
    np.testing.assert_allclose(got, np.clip(ref, 0, L - 1), rtol=0, atol=3e-6)


@pytest.mark.parametrize("with_da", [False, True])
def test_mip_level_bias_gradient_matches_central_differences(with_da):
    H, W, C = 12, 10, 3
    L = O.tex_levels(H, W)
    rng = np.random.default_rng(8)
    tex = rng.uniform(-1, 1, (1, H, W, C))
    uv = rng.uniform(-0.3, 1.3, (2, 3, 4, 2))
    da = (rng.uniform(-0.3, 0.3, (2, 3, 4, 4)) / W * 2.0 ** rng.uniform(0.3, 1.5, (2, 3, 4, 1))) if with_da else None
    bias = rng.uniform(0.2, 2.3, (2, 3, 4))
    gout = rng.normal(size=(2, 3, 4, C))

    def loss(b):
        pyr = O.tex_mip_build(tex, L, "f64")
        return float((O.tex_fwd(tex, pyr, L, uv, da, "linear-mipmap-linear", "wrap", "f64", bias=b) * gout).sum())

    pyr = O.tex_mip_build(tex, L, "f64")
    res = O.tex_bwd(tex, pyr, L, uv, da, gout, "linear-mipmap-linear", "wrap", "f64", bias=bias)
    gb = res[4]
    for idx in [(0, 0, 0), (1, 2, 3), (0, 1, 2), (1, 0, 1)]:
        fd = _central(loss, bias, idx, 1e-7)
        assert abs(gb[idx] - fd) <= 1e-5 * max(1.0, abs(fd)), (idx, gb[idx], fd)
    if with_da:  # uv_da's gradient with the bias in lambda
        def loss_da(d):
            return float((O.tex_fwd(tex, pyr, L, uv, d, "linear-mipmap-linear", "wrap", "f64", bias=bias)
                          * gout).sum())
        for idx in [(0, 0, 1, 0), (1, 2, 2, 1)]:
            fd = _central(loss_da, da, idx, 1e-8)
            assert abs(res[3][idx] - fd) <= 1e-4 * max(1.0, abs(fd)), ("uv_da", idx, res[3][idx], fd)
