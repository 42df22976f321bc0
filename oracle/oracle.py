"""numpy front-end of the C oracle (``drp_oracle.c``).

TEST INFRASTRUCTURE ONLY -- the checker for the CUDA path and the timed CPU
baseline.  The product package never imports this module.

Argument conventions follow the nvdiffrast-style boundary that diffrp calls
(diffrp/rendering/surface_deferred.py:260-262, :775 and
diffrp/rendering/interpolator.py:83):

* ``pos``  -- (V, 4) clip-space positions shared by all views (range mode,
  ``ranges`` gives ``[first, count]`` per view) or (B, V, 4) (instanced mode);
* ``tri``  -- (F, 3) int32;
* ``rast`` -- (B, H, W, 4) = (u, v, z/w, tri_id + 1), row 0 at NDC y = -1;
* ``rast_db`` -- (B, H, W, 4) = (du/dX, du/dY, dv/dX, dv/dY).

``precision='f32'`` uses the bit-exact float build, ``'f64'`` the double build
(coverage is identical in both: snapping is always float).
"""
import ctypes
import os

import numpy as np

from . import build as _build

__all__ = [
    "load", "triidx_to_float", "float_to_triidx", "raster_ids", "rasterize", "raster_bwd",
    "interpolate", "interpolate_bwd", "interpolate_sparse", "topology", "antialias", "antialias_bwd",
    "key_tri", "default_threads", "aa_plan", "l1_fixed_visibility",
    "TEX_FILTERS", "TEX_BOUNDARIES", "tex_levels", "tex_mip_build", "tex_mip_bwd", "tex_fwd", "tex_bwd",
]

_LIBS = {}
_c_int = ctypes.c_int
_c_long = ctypes.c_long
_p = ctypes.c_void_p


def default_threads():
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1


def load(precision="f32"):
    if precision not in _LIBS:
        out = _build.build()
        lib = ctypes.CDLL(os.path.join(out, "liborc_%s.so" % precision))
        lib.orc_triidx_to_float.restype = ctypes.c_float
        lib.orc_triidx_to_float.argtypes = [ctypes.c_int32]
        lib.orc_float_to_triidx.restype = ctypes.c_int32
        lib.orc_float_to_triidx.argtypes = [ctypes.c_float]
        lib.orc_raster_ids.argtypes = [_p, _c_long, _c_long, _p, _c_long, _p, _p, _c_int, _c_int, _c_int, _p, _p, _c_int]
        lib.orc_shade.argtypes = [_p, _c_long, _c_long, _p, _c_long, _p, _c_int, _c_int, _c_int, _p, _p, _c_int]
        lib.orc_raster_bwd.argtypes = [_p, _c_long, _c_long, _p, _c_long, _p, _p, _p, _c_int, _c_int, _c_int, _p, _c_int]
        lib.orc_interp_fwd.argtypes = [_p, _c_long, _c_long, _c_int, _p, _p, _p, _c_long, _c_int, _c_int, _c_int,
                                       _p, _c_int, _p, _p, _c_int]
        lib.orc_interp_bwd.argtypes = [_p, _c_long, _c_long, _c_int, _p, _p, _p, _c_long, _c_int, _c_int, _c_int,
                                       _p, _c_int, _p, _p, _p, _p, _p, _c_int]
        lib.orc_interp_sparse_fwd.argtypes = [_p, _c_long, _c_int, _p, _p, _c_long, _p]
        lib.orc_topology.argtypes = [_p, _c_long, _p]
        real = ctypes.c_double if precision == "f64" else ctypes.c_float
        lib.orc_aa_fwd.argtypes = [_p, _c_int, _p, _p, _c_long, _c_long, _p, _c_long, _p, _c_int, _c_int, _c_int,
                                   _p, _c_int]
        lib.orc_aa_bwd.argtypes = [_p, _c_int, _p, _p, _c_long, _c_long, _p, _c_long, _p, _c_int, _c_int, _c_int,
                                   _p, real, _p, _p, _c_int]
        lib.orc_aa_plan.argtypes = [_p, _p, _c_long, _p, _c_long, _p, _c_int, _c_int, _p, _c_long]
        lib.orc_aa_plan.restype = _c_long
        lib.orc_l1_fixed_visibility.argtypes = [_p, _p, _p, _c_int, _c_int, _c_int, _p, _p, _p, _c_long, _p, _p,
                                                _c_int]
        lib.orc_l1_fixed_visibility.restype = _c_int
        lib.orc_tex_levels.argtypes = [_c_int, _c_int, _c_int]
        lib.orc_tex_levels.restype = _c_int
        lib.orc_tex_pyramid_texels.argtypes = [_c_int, _c_int, _c_int]
        lib.orc_tex_pyramid_texels.restype = _c_long
        lib.orc_tex_mip_build.argtypes = [_p, _c_int, _c_int, _c_int, _c_int, _c_int, _p]
        lib.orc_tex_mip_build.restype = None
        lib.orc_tex_mip_bwd.argtypes = [_p, _c_int, _c_int, _c_int, _c_int, _c_int, _p]
        lib.orc_tex_mip_bwd.restype = None
        lib.orc_tex_fwd.argtypes = [_p, _p, _c_int, _c_int, _c_int, _c_int, _c_int, _p, _p, _p, _c_int, _c_int,
                                    _c_int, _c_int, _c_int, _p]
        lib.orc_tex_fwd.restype = None
        lib.orc_tex_bwd.argtypes = [_p, _p, _c_int, _c_int, _c_int, _c_int, _c_int, _p, _p, _p, _c_int, _c_int,
                                    _c_int, _c_int, _c_int, _p, _p, _p, _p, _p, _p]
        lib.orc_tex_bwd.restype = None
        for name in ["orc_raster_ids", "orc_shade", "orc_raster_bwd", "orc_interp_fwd", "orc_interp_bwd",
                     "orc_interp_sparse_fwd", "orc_topology", "orc_aa_fwd", "orc_aa_bwd"]:
            getattr(lib, name).restype = _c_int
        _LIBS[precision] = lib
    return _LIBS[precision]


def _dt(precision):
    return np.float64 if precision == "f64" else np.float32


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("oracle %s failed with status %d" % (what, rc))


def triidx_to_float(x):
    x = np.asarray(x, dtype=np.int64)
    lib = load()
    return np.array([lib.orc_triidx_to_float(int(v)) for v in x.ravel()], dtype=np.float32).reshape(x.shape)


def float_to_triidx(x):
    x = np.asarray(x, dtype=np.float32)
    lib = load()
    return np.array([lib.orc_float_to_triidx(float(v)) for v in x.ravel()], dtype=np.int32).reshape(x.shape)


def _views(pos, tri, ranges):
    """Return (pos contiguous, view stride, V, B, tri_first, tri_count)."""
    F = tri.shape[0]
    if pos.ndim == 3:
        B, V = pos.shape[0], pos.shape[1]
        stride = V * 4
        first = np.zeros(B, np.int32)
        count = np.full(B, F, np.int32)
        if ranges is not None:
            raise ValueError("ranges only valid with 2-D pos")
    else:
        V = pos.shape[0]
        stride = 0
        if ranges is None:
            ranges = np.array([[0, F]], np.int32)
        ranges = np.ascontiguousarray(ranges, dtype=np.int32)
        B = ranges.shape[0]
        first = np.ascontiguousarray(ranges[:, 0])
        count = np.ascontiguousarray(ranges[:, 1])
    return stride, V, B, first, count


def key_tri(key):
    """Triangle index (or -1) from a visibility key array."""
    k = np.asarray(key, dtype=np.uint64)
    t = (k & np.uint64(0xFFFFFFFF)).astype(np.int64)
    t[k == np.uint64(0xFFFFFFFFFFFFFFFF)] = -1
    return t


def raster_ids(pos, tri, resolution, ranges=None, prev_key=None, nthreads=None):
    pos32 = np.ascontiguousarray(pos, dtype=np.float32)
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    H, W = resolution
    stride, V, B, first, count = _views(pos32, tri, ranges)
    key = np.empty((B, H, W), np.uint64)
    if prev_key is not None:
        prev_key = np.ascontiguousarray(prev_key, dtype=np.uint64)
    lib = load()
    _check(lib.orc_raster_ids(_ptr(pos32), stride, V, _ptr(tri), tri.shape[0], _ptr(first), _ptr(count), B, H, W,
                              _ptr(prev_key), _ptr(key), nthreads or default_threads()), "raster_ids")
    return key


def rasterize(pos, tri, resolution, ranges=None, prev_key=None, grad_db=True, precision="f32", nthreads=None,
              key=None):
    """Returns (rast, rast_db or None, key)."""
    dt = _dt(precision)
    if key is None:
        key = raster_ids(pos, tri, resolution, ranges, prev_key, nthreads)
    posr = np.ascontiguousarray(pos, dtype=dt)
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    H, W = resolution
    stride, V, B, first, count = _views(posr, tri, ranges)
    rast = np.empty((B, H, W, 4), dt)
    db = np.empty((B, H, W, 4), dt) if grad_db else None
    lib = load(precision)
    _check(lib.orc_shade(_ptr(posr), stride, V, _ptr(tri), tri.shape[0], _ptr(key), B, H, W, _ptr(rast), _ptr(db),
                         nthreads or default_threads()), "shade")
    return rast, db, key


def raster_bwd(pos, tri, rast, grad_rast, grad_db=None, nthreads=None, precision="f64"):
    """dL/dpos in float64 (same layout as pos).  precision "f32" evaluates
    every per-pixel term in float32 (the arithmetic of the CUDA path, so the
    same branch at near-ties) and still accumulates in float64."""
    dt = _dt(precision)
    posr = np.ascontiguousarray(pos, dtype=dt)
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    rast = np.ascontiguousarray(rast, dtype=dt)
    B, H, W = rast.shape[:3]
    stride = posr.shape[1] * 4 if posr.ndim == 3 else 0
    V = posr.shape[-2]
    gp = np.zeros(posr.shape, np.float64)
    gr = np.ascontiguousarray(grad_rast, dtype=dt)
    gd = None if grad_db is None else np.ascontiguousarray(grad_db, dtype=dt)
    lib = load(precision)
    _check(lib.orc_raster_bwd(_ptr(posr), stride, V, _ptr(tri), tri.shape[0], _ptr(rast), _ptr(gr), _ptr(gd), B, H, W,
                              _ptr(gp), nthreads or default_threads()), "raster_bwd")
    return gp


def _diff_idx(diff_attrs, C):
    if diff_attrs is None:
        return np.zeros(0, np.int32)
    if isinstance(diff_attrs, str) and diff_attrs == "all":
        return np.arange(C, dtype=np.int32)
    return np.ascontiguousarray(diff_attrs, dtype=np.int32)


def interpolate(attr, rast, tri, rast_db=None, diff_attrs=None, precision="f32", nthreads=None):
    dt = _dt(precision)
    attr = np.ascontiguousarray(attr, dtype=dt)
    rast = np.ascontiguousarray(rast, dtype=dt)
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    B, H, W = rast.shape[:3]
    C = attr.shape[-1]
    V = attr.shape[-2]
    stride = V * C if attr.ndim == 3 else 0
    didx = _diff_idx(diff_attrs, C)
    nd = len(didx)
    out = np.empty((B, H, W, C), dt)
    da = np.empty((B, H, W, 2 * nd), dt) if nd else None
    db = None if rast_db is None else np.ascontiguousarray(rast_db, dtype=dt)
    if nd and db is None:
        raise ValueError("diff_attrs requires rast_db")
    lib = load(precision)
    _check(lib.orc_interp_fwd(_ptr(attr), stride, V, C, _ptr(rast), _ptr(db), _ptr(tri), tri.shape[0], B, H, W,
                              _ptr(didx), nd, _ptr(out), _ptr(da), nthreads or default_threads()), "interp_fwd")
    return out, da


def interpolate_bwd(attr, rast, tri, grad_out, rast_db=None, diff_attrs=None, grad_da=None, nthreads=None,
                    precision="f64"):
    """Returns (grad_attr f64, grad_rast, grad_db or None); grad_rast /
    grad_db in the evaluation precision ("f32": float32 terms, see
    raster_bwd)."""
    dt = _dt(precision)
    attr = np.ascontiguousarray(attr, dtype=dt)
    rast = np.ascontiguousarray(rast, dtype=dt)
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    B, H, W = rast.shape[:3]
    C = attr.shape[-1]
    V = attr.shape[-2]
    stride = V * C if attr.ndim == 3 else 0
    didx = _diff_idx(diff_attrs, C)
    nd = len(didx)
    go = np.ascontiguousarray(grad_out, dtype=dt)
    gda = None if (grad_da is None or nd == 0) else np.ascontiguousarray(grad_da, dtype=dt)
    db = None if rast_db is None else np.ascontiguousarray(rast_db, dtype=dt)
    ga = np.zeros(attr.shape, np.float64)
    gr = np.empty((B, H, W, 4), dt)
    gdb = np.empty((B, H, W, 4), dt) if db is not None else None
    lib = load(precision)
    _check(lib.orc_interp_bwd(_ptr(attr), stride, V, C, _ptr(rast), _ptr(db), _ptr(tri), tri.shape[0], B, H, W,
                              _ptr(didx), nd, _ptr(go), _ptr(gda), _ptr(ga), _ptr(gr), _ptr(gdb),
                              nthreads or default_threads()), "interp_bwd")
    return ga, gr, gdb


def interpolate_sparse(vertex_buffer, vi_data, tri_idx, precision="f32"):
    dt = _dt(precision)
    vb = np.ascontiguousarray(vertex_buffer, dtype=dt)
    vi = np.ascontiguousarray(vi_data, dtype=dt)
    ti = np.ascontiguousarray(tri_idx, dtype=np.int64)
    N = vi.shape[0]
    out = np.empty((N, vb.shape[1]), dt)
    lib = load(precision)
    _check(lib.orc_interp_sparse_fwd(_ptr(vb), vb.shape[0], vb.shape[1], _ptr(vi), _ptr(ti), N, _ptr(out)),
           "interp_sparse")
    return out


def topology(tri):
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    nbr = np.empty(tri.shape, np.int32)
    _check(load().orc_topology(_ptr(tri), tri.shape[0], _ptr(nbr)), "topology")
    return nbr


def antialias(color, rast, pos, tri, nbr=None, precision="f32", nthreads=None):
    dt = _dt(precision)
    color = np.ascontiguousarray(color, dtype=dt)
    rast = np.ascontiguousarray(rast, dtype=dt)
    posr = np.ascontiguousarray(pos, dtype=dt)
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    if nbr is None:
        nbr = topology(tri)
    B, H, W, C = color.shape
    stride = posr.shape[1] * 4 if posr.ndim == 3 else 0
    out = np.empty_like(color)
    lib = load(precision)
    _check(lib.orc_aa_fwd(_ptr(color), C, _ptr(rast), _ptr(posr), stride, posr.shape[-2], _ptr(tri), tri.shape[0],
                          _ptr(nbr), B, H, W, _ptr(out), nthreads or default_threads()), "aa_fwd")
    return out


def antialias_bwd(color, rast, pos, tri, grad_out, nbr=None, pos_gradient_boost=1.0, nthreads=None,
                  precision="f64"):
    """Returns (grad_color, grad_pos f64); grad_color in the evaluation
    precision ("f32": float32 terms, see raster_bwd)."""
    dt = _dt(precision)
    color = np.ascontiguousarray(color, dtype=dt)
    rast = np.ascontiguousarray(rast, dtype=dt)
    posr = np.ascontiguousarray(pos, dtype=dt)
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    if nbr is None:
        nbr = topology(tri)
    go = np.ascontiguousarray(grad_out, dtype=dt)
    B, H, W, C = color.shape
    stride = posr.shape[1] * 4 if posr.ndim == 3 else 0
    gc = np.empty_like(color)
    gp = np.zeros(posr.shape, np.float64)
    lib = load(precision)
    _check(lib.orc_aa_bwd(_ptr(color), C, _ptr(rast), _ptr(posr), stride, posr.shape[-2], _ptr(tri), tri.shape[0],
                          _ptr(nbr), B, H, W, _ptr(go), float(pos_gradient_boost), _ptr(gc), _ptr(gp),
                          nthreads or default_threads()), "aa_bwd")
    return gc, gp



def aa_plan(rast, pos, tri, nbr=None):
    """The decisions of one view's antialias forward, evaluated in float (the
    CUDA forward's decisions): an (n, 8) int32 array of (target pixel, source
    pixel, front pixel, other pixel, front triangle, crossing edge, branch,
    orientation sign); see orc_aa_plan.  rast: (H, W, 4) or (1, H, W, 4)."""
    rast = np.asarray(rast, dtype=np.float32)
    H, W = rast.shape[-3], rast.shape[-2]
    rast = np.ascontiguousarray(rast.reshape(-1, 4))
    posr = np.ascontiguousarray(pos, dtype=np.float32)
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    nbr = np.ascontiguousarray(topology(tri) if nbr is None else nbr, dtype=np.int32)
    lib = load("f32")
    cap = max(1024, H * W // 8)
    while True:
        plan = np.empty((cap, 8), np.int32)
        n = lib.orc_aa_plan(_ptr(rast), _ptr(posr), posr.shape[0], _ptr(tri), tri.shape[0], _ptr(nbr), H, W,
                            _ptr(plan), cap)
        if n <= cap:
            return plan[:n].copy()
        cap = n


def l1_fixed_visibility(pos, tri, attr, ids, sign, plan, resolution, tri_flag=None, nthreads=None):
    """Sum over pixels and channels of sign * antialiased colour, in float64,
    with every discrete decision of the forward held fixed: ids (H*W
    triangle indices, -1 background), plan (aa_plan) and sign (H*W*C values
    in {-1, 0, 1}).  tri_flag (one byte per triangle) restricts the sum to
    the terms that involve a flagged triangle (see orc_l1_fixed_visibility)."""
    H, W = resolution
    posr = np.ascontiguousarray(pos, dtype=np.float64)
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    attr = np.ascontiguousarray(attr, dtype=np.float64)
    ids = np.ascontiguousarray(ids, dtype=np.int32).reshape(-1)
    sign = np.ascontiguousarray(sign, dtype=np.int8).reshape(-1)
    plan = np.ascontiguousarray(plan, dtype=np.int32)
    C = attr.shape[-1]
    if ids.size != H * W or sign.size != H * W * C:
        raise ValueError("ids / sign do not match the resolution")
    flag = None if tri_flag is None else np.ascontiguousarray(tri_flag, dtype=np.uint8)
    out = np.zeros(1, np.float64)
    _check(load("f64").orc_l1_fixed_visibility(_ptr(posr), _ptr(tri), _ptr(attr), C, H, W, _ptr(ids), _ptr(sign),
                                               _ptr(plan), plan.shape[0], _ptr(flag), _ptr(out),
                                               nthreads or default_threads()), "l1_fixed_visibility")
    return float(out[0])


# ---------------------------------------------------------------------------
# Texture sampling (drp_oracle_tex.c): the mip-mapped sampler the CUDA
# texture kernels restate.  tex (Nt, H, W, C), uv (N, h, w, 2), uv_da
# (N, h, w, 4) = (du/dX, du/dY, dv/dX, dv/dY) or None.
# ---------------------------------------------------------------------------
TEX_FILTERS = {"nearest": 0, "linear": 1, "linear-mipmap-nearest": 2, "linear-mipmap-linear": 3}
TEX_BOUNDARIES = {"wrap": 0, "clamp": 1, "zero": 2, "mirror": 3}


def tex_levels(H, W, max_level=-1):
    return load("f32").orc_tex_levels(H, W, -1 if max_level is None else max_level)


def tex_mip_build(tex, levels, precision="f32"):
    """Levels 1 .. levels-1 of the pyramid, level-major: a flat array of
    Nt * C * texels(levels 1 ..) values (level 0 is tex itself)."""
    lib, dt = load(precision), _dt(precision)
    tex = np.ascontiguousarray(tex, dt)
    N, H, W, C = tex.shape
    n = lib.orc_tex_pyramid_texels(H, W, levels)
    pyr = np.zeros(max(1, N * n * C), dt)
    lib.orc_tex_mip_build(_ptr(tex), N, H, W, C, levels, _ptr(pyr))
    return pyr


def tex_mip_bwd(grad_tex, grad_pyr, levels, precision="f32"):
    """grad_tex (Nt, H, W, C) plus the pyramid gradient carried down to it
    (returns a new array; grad_pyr is not modified)."""
    lib, dt = load(precision), _dt(precision)
    out = np.ascontiguousarray(grad_tex, dt).copy()
    g = np.ascontiguousarray(grad_pyr, dt).copy()
    N, H, W, C = out.shape
    lib.orc_tex_mip_bwd(_ptr(g), N, H, W, C, levels, _ptr(out))
    return out


def tex_fwd(tex, pyr, levels, uv, uv_da=None, filter_mode="linear", boundary_mode="wrap", precision="f32",
            bias=None):
    """(N, h, w, C) samples; bias: the per-pixel mip level bias (N, h, w)
    added to the level of detail, or None."""
    lib, dt = load(precision), _dt(precision)
    tex = np.ascontiguousarray(tex, dt)
    pyr = np.ascontiguousarray(pyr, dt)
    uv = np.ascontiguousarray(uv, dt)
    Nt, H, W, C = tex.shape
    N, h, w, _ = uv.shape
    da = None if uv_da is None else np.ascontiguousarray(uv_da, dt)
    b = None if bias is None else np.ascontiguousarray(bias, dt)
    out = np.zeros((N, h, w, C), dt)
    lib.orc_tex_fwd(_ptr(tex), _ptr(pyr), Nt, H, W, C, levels, _ptr(uv), None if da is None else _ptr(da),
                    None if b is None else _ptr(b), N, h, w, TEX_FILTERS[filter_mode], TEX_BOUNDARIES[boundary_mode],
                    _ptr(out))
    return out


def tex_bwd(tex, pyr, levels, uv, uv_da, grad_out, filter_mode="linear", boundary_mode="wrap", precision="f32",
            bias=None):
    """(grad_tex, grad_pyr, grad_uv, grad_uv_da or None), plus grad_bias when
    ``bias`` is given; grad_tex holds the level-0 share only (tex_mip_bwd
    adds the pyramid's)."""
    lib, dt = load(precision), _dt(precision)
    tex = np.ascontiguousarray(tex, dt)
    pyr = np.ascontiguousarray(pyr, dt)
    uv = np.ascontiguousarray(uv, dt)
    g = np.ascontiguousarray(grad_out, dt)
    Nt, H, W, C = tex.shape
    N, h, w, _ = uv.shape
    da = None if uv_da is None else np.ascontiguousarray(uv_da, dt)
    b = None if bias is None else np.ascontiguousarray(bias, dt)
    gtex = np.zeros_like(tex)
    gpyr = np.zeros_like(pyr)
    guv = np.zeros_like(uv)
    gda = None if da is None else np.zeros_like(da)
    gb = None if b is None else np.zeros_like(b)
    lib.orc_tex_bwd(_ptr(tex), _ptr(pyr), Nt, H, W, C, levels, _ptr(uv), None if da is None else _ptr(da),
                    None if b is None else _ptr(b), N, h, w, TEX_FILTERS[filter_mode], TEX_BOUNDARIES[boundary_mode],
                    _ptr(g), _ptr(gtex), _ptr(gpyr), _ptr(guv), None if gda is None else _ptr(gda),
                    None if gb is None else _ptr(gb))
    if b is not None:
        return gtex, gpyr, guv, gda, gb
    return gtex, gpyr, guv, gda
