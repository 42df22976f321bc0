/*
 * drp_oracle_tex.c -- CPU restatement of mip-mapped texture sampling (test
 * infrastructure only: the parity tests and the benchmark's CPU baseline
 * call it; the library never does).
 *
 * The semantics are those fixed for diffrp_gb300.nvdr.texture, the drop-in
 * for nvdiffrast's dr.texture: the sampler that consumes the screen-space
 * derivatives interpolate() produces (uv_da), for the texture lookups of
 * diffrp's materials (diffrp/materials/gltf_material.py:47-48 through
 * diffrp/utils/shader_ops.py:224 sample2d, which samples without mipmaps).
 * nvdiffrast itself is not in the reference tree, so these rules are this
 * project's, stated once here and in the CUDA kernels (texture.cu).  The
 * restatement is pinned by tests/test_cpu_texture.py against independent
 * code -- torch's grid_sample for bilinear clamp / zero / mirror sampling, a
 * numpy reshape-mean for the pyramid, math.log2 for the level of detail --
 * and against float64 central differences for every gradient; parity with
 * nvdiffrast's own outputs is unpinned (absent here).
 *
 *  - Texture (N, H, W, C), texel (x, y) centred at ((x + 0.5) / W,
 *    (y + 0.5) / H) in uv; row y = 0 at v = 0.
 *  - Mip level k + 1 halves level k (floor, at least 1) and is the 2x2 box
 *    average ((a + b) + c) + d times 0.25 of the texels (2x, 2y), (2x+1, 2y),
 *    (2x, 2y+1), (2x+1, 2y+1), indices clamped to level k (a level of width
 *    1 repeats its column).
 *  - Bilinear at level k: x = u W_k - 0.5, y = v H_k - 0.5, x0 = floor(x),
 *    fx = x - x0 (likewise y); r0 = fma(fx, t10 - t00, t00), r1 = fma(fx,
 *    t11 - t01, t01), value = fma(fy, r1 - r0, r0).  Boundary: wrap (index
 *    modulo the size), clamp (index clamped), zero (texels outside read 0),
 *    mirror (index modulo twice the size, the second half reversed).
 *  - Nearest: the texel of level 0 whose centre is nearest, (floor(x + 0.5),
 *    floor(y + 0.5)) with x, y as for bilinear, same boundaries.
 *  - Storage: level 0 is the texture; levels 1 .. L-1 form one level-major
 *    array (level k: (N, H_k, W_k, C)), the layout of texture.cu's pyramid.
 *  - Level of detail from uv_da = (du/dX, du/dY, dv/dX, dv/dY):
 *    lx = (du/dX W)^2 + (dv/dX H)^2, ly = (du/dY W)^2 + (dv/dY H)^2,
 *    lambda = 0.5 log2(max(lx, ly)) (0 when the footprint is zero or not
 *    finite, or without uv_da) plus the pixel's mip level bias when given,
 *    clamped to [0, levels - 1].  log2 is evaluated as e + 2 t p(t^2)
 *    / ln 2 with x = m 2^e, m in [sqrt(1/2), sqrt(2)), t = (m - 1) / (m + 1)
 *    and the atanh series p = 1 + t^2/3 + t^4/5 + t^6/7 + t^8/9 (relative
 *    error below 2e-8), so that the CPU and the GPU round it identically.
 *  - linear-mipmap-nearest: bilinear at level floor(lambda + 0.5);
 *    linear-mipmap-linear: s0, s1 bilinear at levels l0 = floor(lambda) and
 *    min(l0 + 1, levels - 1), value = fma(f, s1 - s0, s0) with f = lambda -
 *    l0 (s0 alone when f = 0).
 *  - Gradients: to the texels (bilinear weights times the level weight, then
 *    down the pyramid through the box filter), to uv (the bilinear
 *    derivative times W_k, H_k), and to uv_da through lambda for
 *    linear-mipmap-linear where lambda is not clamped.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef REAL
#define REAL float
#endif
typedef REAL real;

#if defined(__GNUC__)
#define ORC_EXPORT __attribute__((visibility("default")))
#else
#define ORC_EXPORT
#endif

enum { TEX_NEAREST = 0, TEX_LINEAR = 1, TEX_MIP_NEAREST = 2, TEX_MIP_LINEAR = 3 };
enum { TEX_WRAP = 0, TEX_CLAMP = 1, TEX_ZERO = 2, TEX_MIRROR = 3 };

static inline real r_fma(real a, real b, real c) {
#ifdef REAL_IS_DOUBLE
    return fma(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

/* Level sizes: levels = 1 + halvings until both sizes are 1, at most
 * max_level + 1 (max_level < 0: no cap). */
ORC_EXPORT int orc_tex_levels(int H, int W, int max_level) {
    int n = 1, h = H, w = W;
    while ((h > 1 || w > 1) && (max_level < 0 || n <= max_level)) {
        h = h > 1 ? h >> 1 : 1;
        w = w > 1 ? w >> 1 : 1;
        ++n;
    }
    return n;
}

static void level_dims(int H, int W, int k, int* hk, int* wk) {
    int h = H, w = W;
    for (int i = 0; i < k; ++i) {
        h = h > 1 ? h >> 1 : 1;
        w = w > 1 ? w >> 1 : 1;
    }
    *hk = h;
    *wk = w;
}

/* Layout: level 0 is the texture itself (Nt, H, W, C); levels 1 .. L-1 are
 * one level-major array, level k holding (Nt, H_k, W_k, C) at float offset
 * Nt C (texels of levels 1 .. k-1).  lvl_base gives level k's first float
 * for texture n (k = 0: in tex). */
static long level_texels_from1(int H, int W, int k) {
    long off = 0;
    for (int i = 1; i < k; ++i) {
        int h, w;
        level_dims(H, W, i, &h, &w);
        off += (long)h * w;
    }
    return off;
}

ORC_EXPORT long orc_tex_pyramid_texels(int H, int W, int levels) { return level_texels_from1(H, W, levels); }

static inline const real* lvl_base(const real* tex, const real* pyr, int Nt, int H, int W, int C, int k, int n) {
    int h, w;
    level_dims(H, W, k, &h, &w);
    if (k == 0) return tex + (long)n * H * W * C;
    return pyr + (long)Nt * level_texels_from1(H, W, k) * C + (long)n * h * w * C;
}

static inline real* lvl_base_w(real* tex, real* pyr, int Nt, int H, int W, int C, int k, int n) {
    return (real*)lvl_base(tex, pyr, Nt, H, W, C, k, n);
}

ORC_EXPORT void orc_tex_mip_build(const real* tex, int N, int H, int W, int C, int levels, real* pyr) {
    for (int n = 0; n < N; ++n) {
        for (int k = 1; k < levels; ++k) {
            int hp, wp, hk, wk;
            level_dims(H, W, k - 1, &hp, &wp);
            level_dims(H, W, k, &hk, &wk);
            const real* src = lvl_base(tex, pyr, N, H, W, C, k - 1, n);
            real* dst = lvl_base_w(NULL, pyr, N, H, W, C, k, n);
            for (int y = 0; y < hk; ++y)
                for (int x = 0; x < wk; ++x) {
                    const int x0 = 2 * x < wp - 1 ? 2 * x : wp - 1, x1 = 2 * x + 1 < wp - 1 ? 2 * x + 1 : wp - 1;
                    const int y0 = 2 * y < hp - 1 ? 2 * y : hp - 1, y1 = 2 * y + 1 < hp - 1 ? 2 * y + 1 : hp - 1;
                    for (int c = 0; c < C; ++c) {
                        const real a = src[((long)y0 * wp + x0) * C + c], b = src[((long)y0 * wp + x1) * C + c];
                        const real d0 = src[((long)y1 * wp + x0) * C + c], d1 = src[((long)y1 * wp + x1) * C + c];
                        dst[((long)y * wk + x) * C + c] = (((a + b) + d0) + d1) * (real)0.25;
                    }
                }
        }
    }
}

/* Backward of the pyramid: level-k gradients flow down to level 0 (a gather:
 * texel i of level k - 1 receives from texel i >> 1 of level k, twice along
 * an axis where level k - 1 has size 1).  grad_pyr (levels 1 ..) is
 * consumed; level 0's share is added into grad_tex. */
ORC_EXPORT void orc_tex_mip_bwd(real* grad_pyr, int N, int H, int W, int C, int levels, real* grad_tex) {
    for (int n = 0; n < N; ++n) {
        for (int k = levels - 1; k >= 1; --k) {
            int hp, wp, hk, wk;
            level_dims(H, W, k - 1, &hp, &wp);
            level_dims(H, W, k, &hk, &wk);
            const real* src = lvl_base(NULL, grad_pyr, N, H, W, C, k, n);
            real* dst = lvl_base_w(grad_tex, grad_pyr, N, H, W, C, k - 1, n);
            const real mx = wp == 1 ? (real)2 : (real)1, my = hp == 1 ? (real)2 : (real)1;
            for (int y = 0; y < hp; ++y)
                for (int x = 0; x < wp; ++x) {
                    const int cx = x >> 1, cy = y >> 1;
                    if (cx >= wk || cy >= hk) continue;
                    for (int c = 0; c < C; ++c)
                        dst[((long)y * wp + x) * C + c] += ((real)0.25 * mx) * my * src[((long)cy * wk + cx) * C + c];
                }
        }
    }
}

/* log2 for the level of detail (see the header comment). */
static inline real tex_log2(real x) {
    int e;
#ifdef REAL_IS_DOUBLE
    real m = frexp(x, &e);
#else
    real m = frexpf(x, &e);
#endif
    if (m < (real)0.70710678f) {
        m = m * (real)2;
        e = e - 1;
    }
    const real t = (m - (real)1) / (m + (real)1);
    const real t2 = t * t;
    real p = (real)(1.0f / 9.0f);
    p = p * t2 + (real)(1.0f / 7.0f);
    p = p * t2 + (real)(1.0f / 5.0f);
    p = p * t2 + (real)(1.0f / 3.0f);
    p = p * t2 + (real)1;
    return (real)e + t * p * (real)2.88539008f;
}

typedef struct {
    int l0, l1;
    real f;           /* weight of l1 */
    int interior;     /* lambda strictly inside (0, levels - 1): lambda's gradient flows */
    int da_active;    /* lambda has the footprint term (uv_da given, footprint > 0) */
    real r2;
    int use_x;        /* the X footprint is the larger */
    real ax, ay, bx, by;
} lod_t;

/* bias: the pixel's mip level bias, added to lambda (NULL: none). */
static void tex_lod(const real* da, const real* bias, int H, int W, int levels, int filter, lod_t* L) {
    memset(L, 0, sizeof(*L));
    if ((!da && !bias) || levels <= 1 || filter < TEX_MIP_NEAREST) return;
    real lam = 0;
    if (da) {
        L->ax = da[0] * (real)W;
        L->bx = da[1] * (real)W;
        L->ay = da[2] * (real)H;
        L->by = da[3] * (real)H;
        const real lx = L->ax * L->ax + L->ay * L->ay;
        const real ly = L->bx * L->bx + L->by * L->by;
        L->use_x = lx >= ly;
        const real r2 = L->use_x ? lx : ly;
        L->r2 = r2;
        L->da_active = r2 > 0 && isfinite(r2);
        if (L->da_active) lam = (real)0.5 * tex_log2(r2);
    }
    if (bias) lam = lam + *bias;
    const real top = (real)(levels - 1);
    L->interior = lam > 0 && lam < top;
    if (!(lam > 0)) lam = 0;
    if (lam > top) lam = top;
    if (filter == TEX_MIP_NEAREST) {
#ifdef REAL_IS_DOUBLE
        int l = (int)floor(lam + (real)0.5);
#else
        int l = (int)floorf(lam + (real)0.5);
#endif
        if (l > levels - 1) l = levels - 1;
        L->l0 = L->l1 = l;
        L->f = 0;
        L->interior = 0;
        return;
    }
#ifdef REAL_IS_DOUBLE
    const int l0 = (int)floor(lam);
#else
    const int l0 = (int)floorf(lam);
#endif
    L->l0 = l0;
    L->l1 = l0 + 1 < levels ? l0 + 1 : levels - 1;
    L->f = L->l1 > l0 ? lam - (real)l0 : (real)0;
}

static inline int wrap_index(int i, int n) {
    int r = i % n;
    return r < 0 ? r + n : r;
}

/* Mirrored repeat: period 2n, the second half reversed. */
static inline int mirror_index(int i, int n) {
    const int m = wrap_index(i, 2 * n);
    return m < n ? m : 2 * n - 1 - m;
}

/* Texel index for boundary mode; -1 outside (zero mode). */
static inline long texel_index(int x, int y, int w, int h, int boundary) {
    if (boundary == TEX_WRAP) {
        x = wrap_index(x, w);
        y = wrap_index(y, h);
    } else if (boundary == TEX_CLAMP) {
        x = x < 0 ? 0 : (x > w - 1 ? w - 1 : x);
        y = y < 0 ? 0 : (y > h - 1 ? h - 1 : y);
    } else if (boundary == TEX_MIRROR) {
        x = mirror_index(x, w);
        y = mirror_index(y, h);
    } else if (x < 0 || x >= w || y < 0 || y >= h) {
        return -1;
    }
    return (long)y * w + x;
}

/* uv -> texel coordinate, bounded so that the integer conversions below stay
 * in range for any finite input (2^24 texels of slack). */
static inline real tex_coord(real u, int size) {
    real x = u * (real)size - (real)0.5;
    const real lim = (real)16777216.0f;
    if (!(x > -lim)) x = -lim;
    if (x > lim) x = lim;
    return x;
}

typedef struct {
    long i00, i10, i01, i11;
    real fx, fy;
} bilin_t;

static inline void bilin_setup(real u, real v, int w, int h, int boundary, bilin_t* B) {
    const real x = tex_coord(u, w), y = tex_coord(v, h);
#ifdef REAL_IS_DOUBLE
    const real x0 = floor(x), y0 = floor(y);
#else
    const real x0 = floorf(x), y0 = floorf(y);
#endif
    B->fx = x - x0;
    B->fy = y - y0;
    const int ix = (int)x0, iy = (int)y0;
    B->i00 = texel_index(ix, iy, w, h, boundary);
    B->i10 = texel_index(ix + 1, iy, w, h, boundary);
    B->i01 = texel_index(ix, iy + 1, w, h, boundary);
    B->i11 = texel_index(ix + 1, iy + 1, w, h, boundary);
}

static inline real fetch(const real* lvl, long i, int C, int c) { return i < 0 ? (real)0 : lvl[i * C + c]; }

static inline real bilin_value(const real* lvl, const bilin_t* B, int C, int c) {
    const real t00 = fetch(lvl, B->i00, C, c), t10 = fetch(lvl, B->i10, C, c);
    const real t01 = fetch(lvl, B->i01, C, c), t11 = fetch(lvl, B->i11, C, c);
    const real r0 = r_fma(B->fx, t10 - t00, t00), r1 = r_fma(B->fx, t11 - t01, t01);
    return r_fma(B->fy, r1 - r0, r0);
}

/* out (N, h, w, C).  tex pyramid per texture (Nt = 1 or N). */
ORC_EXPORT void orc_tex_fwd(const real* tex, const real* pyr, int Nt, int H, int W, int C, int levels,
                            const real* uv, const real* uv_da, const real* bias, int N, int h, int w, int filter,
                            int boundary, real* out) {
    const long npix = (long)h * w;
#pragma omp parallel for schedule(static)
    for (long p = 0; p < (long)N * npix; ++p) {
        const int n = (int)(p / npix), tn = Nt == 1 ? 0 : n;
        const real* P = lvl_base(tex, pyr, Nt, H, W, C, 0, tn);
        const real u = uv[2 * p], v = uv[2 * p + 1];
        real* o = out + p * C;
        if (filter == TEX_NEAREST) {
#ifdef REAL_IS_DOUBLE
            const int ix = (int)floor(tex_coord(u, W) + (real)0.5), iy = (int)floor(tex_coord(v, H) + (real)0.5);
#else
            const int ix = (int)floorf(tex_coord(u, W) + (real)0.5), iy = (int)floorf(tex_coord(v, H) + (real)0.5);
#endif
            const long i = texel_index(ix, iy, W, H, boundary);
            for (int c = 0; c < C; ++c) o[c] = fetch(P, i, C, c);
            continue;
        }
        lod_t L;
        tex_lod(uv_da ? uv_da + 4 * p : NULL, bias ? bias + p : NULL, H, W, levels, filter, &L);
        int h0, w0, h1, w1;
        level_dims(H, W, L.l0, &h0, &w0);
        level_dims(H, W, L.l1, &h1, &w1);
        bilin_t B0, B1;
        bilin_setup(u, v, w0, h0, boundary, &B0);
        bilin_setup(u, v, w1, h1, boundary, &B1);
        const real* lv0 = lvl_base(tex, pyr, Nt, H, W, C, L.l0, tn);
        const real* lv1 = lvl_base(tex, pyr, Nt, H, W, C, L.l1, tn);
        for (int c = 0; c < C; ++c) {
            const real s0 = bilin_value(lv0, &B0, C, c);
            if (L.f > 0) {
                const real s1 = bilin_value(lv1, &B1, C, c);
                o[c] = r_fma(L.f, s1 - s0, s0);
            } else {
                o[c] = s0;
            }
        }
    }
}

static void bilin_bwd(const real* lvl, real* glvl, const bilin_t* B, int w, int h, int C, const real* g, real wl,
                      real* gu, real* gv) {
    const real fx = B->fx, fy = B->fy;
    const real w00 = ((real)1 - fx) * ((real)1 - fy), w10 = fx * ((real)1 - fy);
    const real w01 = ((real)1 - fx) * fy, w11 = fx * fy;
    real dx = 0, dy = 0;
    for (int c = 0; c < C; ++c) {
        const real gc = g[c] * wl;
        const real t00 = fetch(lvl, B->i00, C, c), t10 = fetch(lvl, B->i10, C, c);
        const real t01 = fetch(lvl, B->i01, C, c), t11 = fetch(lvl, B->i11, C, c);
        dx += gc * (((real)1 - fy) * (t10 - t00) + fy * (t11 - t01));
        dy += gc * ((r_fma(fx, t11 - t01, t01)) - (r_fma(fx, t10 - t00, t00)));
        if (B->i00 >= 0) glvl[B->i00 * C + c] += gc * w00;
        if (B->i10 >= 0) glvl[B->i10 * C + c] += gc * w10;
        if (B->i01 >= 0) glvl[B->i01 * C + c] += gc * w01;
        if (B->i11 >= 0) glvl[B->i11 * C + c] += gc * w11;
    }
    *gu += dx * (real)w;
    *gv += dy * (real)h;
}

/* grad_tex (level 0) and grad_pyr (levels 1 .., zeroed by the caller)
 * accumulate; grad_uv (N, h, w, 2), grad_uv_da and grad_bias (may be null)
 * are written.  Single-threaded (texel gradients are shared). */
ORC_EXPORT void orc_tex_bwd(const real* tex, const real* pyr, int Nt, int H, int W, int C, int levels,
                            const real* uv, const real* uv_da, const real* bias, int N, int h, int w, int filter,
                            int boundary, const real* grad_out, real* grad_tex, real* grad_pyr, real* grad_uv,
                            real* grad_uv_da, real* grad_bias) {
    const long npix = (long)h * w;
    for (long p = 0; p < (long)N * npix; ++p) {
        const int n = (int)(p / npix), tn = Nt == 1 ? 0 : n;
        const real* P = lvl_base(tex, pyr, Nt, H, W, C, 0, tn);
        real* G = lvl_base_w(grad_tex, grad_pyr, Nt, H, W, C, 0, tn);
        const real u = uv[2 * p], v = uv[2 * p + 1];
        const real* g = grad_out + p * C;
        real gu = 0, gv = 0;
        if (grad_uv_da) memset(grad_uv_da + 4 * p, 0, 4 * sizeof(real));
        if (grad_bias) grad_bias[p] = 0;
        if (filter == TEX_NEAREST) {
#ifdef REAL_IS_DOUBLE
            const int ix = (int)floor(tex_coord(u, W) + (real)0.5), iy = (int)floor(tex_coord(v, H) + (real)0.5);
#else
            const int ix = (int)floorf(tex_coord(u, W) + (real)0.5), iy = (int)floorf(tex_coord(v, H) + (real)0.5);
#endif
            const long i = texel_index(ix, iy, W, H, boundary);
            if (i >= 0)
                for (int c = 0; c < C; ++c) G[i * C + c] += g[c];
            grad_uv[2 * p] = 0;
            grad_uv[2 * p + 1] = 0;
            continue;
        }
        lod_t L;
        const real* da = uv_da ? uv_da + 4 * p : NULL;
        tex_lod(da, bias ? bias + p : NULL, H, W, levels, filter, &L);
        int h0, w0, h1, w1;
        level_dims(H, W, L.l0, &h0, &w0);
        level_dims(H, W, L.l1, &h1, &w1);
        bilin_t B0, B1;
        bilin_setup(u, v, w0, h0, boundary, &B0);
        bilin_setup(u, v, w1, h1, boundary, &B1);
        const real* P0 = lvl_base(tex, pyr, Nt, H, W, C, L.l0, tn);
        const real* P1 = lvl_base(tex, pyr, Nt, H, W, C, L.l1, tn);
        real* G0 = lvl_base_w(grad_tex, grad_pyr, Nt, H, W, C, L.l0, tn);
        real* G1 = lvl_base_w(grad_tex, grad_pyr, Nt, H, W, C, L.l1, tn);
        const real f = L.f;
        bilin_bwd(P0, G0, &B0, w0, h0, C, g, f > 0 ? (real)1 - f : (real)1, &gu, &gv);
        if (f > 0) {
            bilin_bwd(P1, G1, &B1, w1, h1, C, g, f, &gu, &gv);
            if ((grad_uv_da || grad_bias) && L.interior) {
                real dl = 0; /* d out / d lambda . grad_out */
                for (int c = 0; c < C; ++c) dl += g[c] * (bilin_value(P1, &B1, C, c) - bilin_value(P0, &B0, C, c));
                if (grad_bias) grad_bias[p] = dl;
                if (grad_uv_da && L.da_active) {
                    /* lambda = 0.5 log2(r2) + bias: d lambda / d r2 = 0.5 / (r2 ln 2) */
                    const real dr2 = dl * ((real)0.72134752f / L.r2);
                    real* gd = grad_uv_da + 4 * p;
                    if (L.use_x) {
                        gd[0] = dr2 * (real)2 * L.ax * (real)W;
                        gd[2] = dr2 * (real)2 * L.ay * (real)H;
                    } else {
                        gd[1] = dr2 * (real)2 * L.bx * (real)W;
                        gd[3] = dr2 * (real)2 * L.by * (real)H;
                    }
                }
            }
        }
        grad_uv[2 * p] = gu;
        grad_uv[2 * p + 1] = gv;
    }
}
