// texture.cu -- mip-mapped texture sampling, the consumer of the
// screen-space derivatives interpolate() produces: nvdiffrast's dr.texture
// semantics as this project fixes them (nearest, bilinear, bilinear in the
// nearest mip level, trilinear; wrap / clamp / zero boundaries; level of
// detail from uv_da), for the texture lookups of diffrp's materials
// (diffrp/materials/gltf_material.py:47-48, which sample through
// diffrp/utils/shader_ops.py:224 sample2d without mipmaps).  Every
// expression mirrors the oracle (oracle/drp_oracle_tex.c) in source order
// under --fmad=false, so the forward is bit-exact against it.
//
// Storage: level 0 is the caller's texture (Nt, H, W, C); levels 1 .. L-1
// are one level-major array (level k: (Nt, H_k, W_k, C)), built here.
// Sampling: one thread per output pixel.  Backward: the texel gradients of
// a pixel go to its level (float atomics), then the pyramid backward
// gathers each level's gradient into the one below (no atomics).
#include <cstdio>

#include "../../include/diffrp_gb300.h"
#include "drp_common.cuh"
#include "drp_internal.h"

namespace drp {

constexpr int kTexNearest = 0, kTexMipNearest = 2, kTexMipLinear = 3;  // 1: linear (bilinear, level 0)
constexpr int kTexWrap = 0, kTexClamp = 1, kTexZero = 2;
constexpr int kTexMaxLevels = 32;

struct TexArgs {
    const float* tex;
    const float* pyr;
    int Nt, H, W, C, levels;
    int lh[kTexMaxLevels], lw[kTexMaxLevels];
    long long lofs[kTexMaxLevels];  // float offset of level k (k >= 1) in pyr; level k's texture n at + n H_k W_k C
    const float* uv;                // (N, h, w, 2)
    const float4* uv_da;            // (N, h, w) of (du/dX, du/dY, dv/dX, dv/dY), or null
    long long npix, view_pix;       // N h w, h w
    int filter, boundary;
    float* out;
    // backward
    const float* grad_out;
    float* grad_tex;
    float* grad_pyr;
    float* grad_uv;
    float4* grad_uv_da;
    int vec4;  // C == 4 with 16-byte aligned gradient levels: one float4 atomic per texel
};

__device__ __forceinline__ const float* tex_level(const TexArgs& a, const float* base0, const float* pyr, int k,
                                                  int n) {
    if (k == 0) return base0 + (long long)n * a.H * a.W * a.C;
    return pyr + a.lofs[k] + (long long)n * a.lh[k] * a.lw[k] * a.C;
}

// log2 of the level of detail: x = m 2^e, m in [sqrt(1/2), sqrt(2)), and
// the atanh series log(m) = 2 (t + t^3/3 + t^5/5 + t^7/7 + t^9/9), t =
// (m - 1) / (m + 1) (|t| <= 0.172, relative error below 2e-8).
__device__ __forceinline__ float tex_log2(float x) {
    int e;
    float m = frexpf(x, &e);
    if (m < 0.70710678f) {
        m = m * 2.0f;
        e = e - 1;
    }
    const float t = (m - 1.0f) / (m + 1.0f);
    const float t2 = t * t;
    float p = 1.0f / 9.0f;
    p = p * t2 + 1.0f / 7.0f;
    p = p * t2 + 1.0f / 5.0f;
    p = p * t2 + 1.0f / 3.0f;
    p = p * t2 + 1.0f;
    return (float)e + t * p * 2.88539008f;
}

struct TexLod {
    int l0, l1;
    float f;
    bool interior;
    float r2;
    bool use_x;
    float ax, ay, bx, by;
};

__device__ __forceinline__ TexLod tex_lod(const TexArgs& a, long long p) {
    TexLod L;
    L.l0 = L.l1 = 0;
    L.f = 0.f;
    L.interior = false;
    L.r2 = 0.f;
    L.use_x = true;
    L.ax = L.ay = L.bx = L.by = 0.f;
    if (!a.uv_da || a.levels <= 1 || a.filter < kTexMipNearest) return L;
    const float4 da = a.uv_da[p];
    L.ax = da.x * (float)a.W;
    L.bx = da.y * (float)a.W;
    L.ay = da.z * (float)a.H;
    L.by = da.w * (float)a.H;
    const float lx = L.ax * L.ax + L.ay * L.ay;
    const float ly = L.bx * L.bx + L.by * L.by;
    L.use_x = lx >= ly;
    const float r2 = L.use_x ? lx : ly;
    L.r2 = r2;
    float lam = 0.f;
    if (r2 > 0.f && isfinite(r2)) lam = 0.5f * tex_log2(r2);
    const float top = (float)(a.levels - 1);
    L.interior = lam > 0.f && lam < top;
    if (!(lam > 0.f)) lam = 0.f;
    if (lam > top) lam = top;
    if (a.filter == kTexMipNearest) {
        int l = (int)floorf(lam + 0.5f);
        if (l > a.levels - 1) l = a.levels - 1;
        L.l0 = L.l1 = l;
        L.interior = false;
        return L;
    }
    const int l0 = (int)floorf(lam);
    L.l0 = l0;
    L.l1 = l0 + 1 < a.levels ? l0 + 1 : a.levels - 1;
    L.f = L.l1 > l0 ? lam - (float)l0 : 0.f;
    return L;
}

__device__ __forceinline__ int wrap_index(int i, int n) {
    const int r = i % n;
    return r < 0 ? r + n : r;
}

__device__ __forceinline__ long long texel_index(int x, int y, int w, int h, int boundary) {
    if (boundary == kTexWrap) {
        x = wrap_index(x, w);
        y = wrap_index(y, h);
    } else if (boundary == kTexClamp) {
        x = x < 0 ? 0 : (x > w - 1 ? w - 1 : x);
        y = y < 0 ? 0 : (y > h - 1 ? h - 1 : y);
    } else if (x < 0 || x >= w || y < 0 || y >= h) {
        return -1;
    }
    return (long long)y * w + x;
}

__device__ __forceinline__ float tex_coord(float u, int size) {
    float x = u * (float)size - 0.5f;
    const float lim = 16777216.0f;
    if (!(x > -lim)) x = -lim;
    if (x > lim) x = lim;
    return x;
}

struct Bilin {
    long long i00, i10, i01, i11;
    float fx, fy;
};

__device__ __forceinline__ Bilin bilin_setup(float u, float v, int w, int h, int boundary) {
    Bilin B;
    const float x = tex_coord(u, w), y = tex_coord(v, h);
    const float x0 = floorf(x), y0 = floorf(y);
    B.fx = x - x0;
    B.fy = y - y0;
    const int ix = (int)x0, iy = (int)y0;
    B.i00 = texel_index(ix, iy, w, h, boundary);
    B.i10 = texel_index(ix + 1, iy, w, h, boundary);
    B.i01 = texel_index(ix, iy + 1, w, h, boundary);
    B.i11 = texel_index(ix + 1, iy + 1, w, h, boundary);
    return B;
}

__device__ __forceinline__ float fetch(const float* lvl, long long i, int C, int c) {
    return i < 0 ? 0.f : __ldg(lvl + i * C + c);
}

__device__ __forceinline__ float bilin_value(const float* lvl, const Bilin& B, int C, int c) {
    const float t00 = fetch(lvl, B.i00, C, c), t10 = fetch(lvl, B.i10, C, c);
    const float t01 = fetch(lvl, B.i01, C, c), t11 = fetch(lvl, B.i11, C, c);
    const float r0 = fmaf(B.fx, t10 - t00, t00), r1 = fmaf(B.fx, t11 - t01, t01);
    return fmaf(B.fy, r1 - r0, r0);
}

__device__ __forceinline__ long long nearest_index(const TexArgs& a, float u, float v) {
    const int ix = (int)floorf(tex_coord(u, a.W) + 0.5f), iy = (int)floorf(tex_coord(v, a.H) + 0.5f);
    return texel_index(ix, iy, a.W, a.H, a.boundary);
}

// Level k of every texture from level k - 1: the 2x2 box average, indices
// clamped to level k - 1.
__global__ void __launch_bounds__(256) tex_mip_level_kernel(const float* __restrict__ src, float* __restrict__ dst,
                                                            int Nt, int hp, int wp, int hk, int wk, int C) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)hk * wk;
    if (i >= (long long)Nt * per) return;
    const int n = (int)(i / per);
    const int r = (int)(i - (long long)n * per);
    const int y = r / wk, x = r - y * wk;
    const int x0 = 2 * x < wp - 1 ? 2 * x : wp - 1, x1 = 2 * x + 1 < wp - 1 ? 2 * x + 1 : wp - 1;
    const int y0 = 2 * y < hp - 1 ? 2 * y : hp - 1, y1 = 2 * y + 1 < hp - 1 ? 2 * y + 1 : hp - 1;
    const float* s = src + (long long)n * hp * wp * C;
    float* d = dst + (long long)n * per * C + (long long)r * C;
    for (int c = 0; c < C; ++c) {
        const float pa = s[((long long)y0 * wp + x0) * C + c], pb = s[((long long)y0 * wp + x1) * C + c];
        const float pc = s[((long long)y1 * wp + x0) * C + c], pd = s[((long long)y1 * wp + x1) * C + c];
        d[c] = (((pa + pb) + pc) + pd) * 0.25f;
    }
}

// Pyramid backward, level k into level k - 1 (gather): texel (x, y) of level
// k - 1 receives 0.25 of texel (x >> 1, y >> 1) of level k, twice along an
// axis of size 1.
__global__ void __launch_bounds__(256) tex_mip_bwd_kernel(const float* __restrict__ src, float* __restrict__ dst,
                                                          int Nt, int hp, int wp, int hk, int wk, int C) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)hp * wp;
    if (i >= (long long)Nt * per) return;
    const int n = (int)(i / per);
    const int r = (int)(i - (long long)n * per);
    const int y = r / wp, x = r - y * wp;
    const int cx = x >> 1, cy = y >> 1;
    if (cx >= wk || cy >= hk) return;
    const float mx = wp == 1 ? 2.f : 1.f, my = hp == 1 ? 2.f : 1.f;
    const float* s = src + (long long)n * hk * wk * C + ((long long)cy * wk + cx) * C;
    float* d = dst + (long long)n * per * C + (long long)r * C;
    for (int c = 0; c < C; ++c) d[c] += (0.25f * mx) * my * s[c];
}

__global__ void __launch_bounds__(256) tex_fwd_kernel(TexArgs a) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.npix) return;
    const int n = (int)(p / a.view_pix), tn = a.Nt == 1 ? 0 : n;
    const float u = a.uv[2 * p], v = a.uv[2 * p + 1];
    const int C = a.C;
    float* o = a.out + p * C;
    if (a.filter == kTexNearest) {
        const float* l0 = tex_level(a, a.tex, a.pyr, 0, tn);
        const long long i = nearest_index(a, u, v);
        for (int c = 0; c < C; ++c) o[c] = fetch(l0, i, C, c);
        return;
    }
    const TexLod L = tex_lod(a, p);
    const Bilin B0 = bilin_setup(u, v, a.lw[L.l0], a.lh[L.l0], a.boundary);
    const float* v0 = tex_level(a, a.tex, a.pyr, L.l0, tn);
    if (L.f > 0.f) {
        const Bilin B1 = bilin_setup(u, v, a.lw[L.l1], a.lh[L.l1], a.boundary);
        const float* v1 = tex_level(a, a.tex, a.pyr, L.l1, tn);
        for (int c = 0; c < C; ++c) {
            const float s0 = bilin_value(v0, B0, C, c), s1 = bilin_value(v1, B1, C, c);
            o[c] = fmaf(L.f, s1 - s0, s0);
        }
    } else {
        for (int c = 0; c < C; ++c) o[c] = bilin_value(v0, B0, C, c);
    }
}

// Adds v into *dst from every lane of the warp whose dst is the same
// address: the lanes of one address (found with __match_any_sync) sum their
// values by shuffles and one of them issues the atomic.  Under
// minification thousands of pixels land on the same few texels of the
// coarse levels; contended float atomics there serialise in L2.  dst ==
// nullptr: nothing to add (the lane still takes part).
__device__ __forceinline__ void warp_add(float* dst, float v, unsigned peers) {
    float sum = 0.f;
    unsigned rem = peers;
    while (rem) {  // the group's lanes step through it together
        const int src = __ffs(rem) - 1;
        rem &= rem - 1;
        sum += __shfl_sync(peers, v, src);
    }
    if (dst && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(dst, sum);
}

__device__ __forceinline__ void warp_add4(float4* dst, float4 v, unsigned peers) {
    float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
    unsigned rem = peers;
    while (rem) {
        const int src = __ffs(rem) - 1;
        rem &= rem - 1;
        sum.x += __shfl_sync(peers, v.x, src);
        sum.y += __shfl_sync(peers, v.y, src);
        sum.z += __shfl_sync(peers, v.z, src);
        sum.w += __shfl_sync(peers, v.w, src);
    }
    if (dst && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(dst, sum);
}

__device__ __forceinline__ void bilin_bwd(const float* lvl, float* glvl, const Bilin& B, int w, int h, int C,
                                          bool vec4, const float* g, float wl, float& gu, float& gv) {
    const float fx = B.fx, fy = B.fy;
    const float wt[4] = {(1.f - fx) * (1.f - fy), fx * (1.f - fy), (1.f - fx) * fy, fx * fy};
    const long long idx[4] = {B.i00, B.i10, B.i01, B.i11};
    float* row[4];
    unsigned peers[4];
    const unsigned active = __activemask();
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        row[t] = idx[t] >= 0 ? glvl + idx[t] * C : nullptr;
        peers[t] = __match_any_sync(active, reinterpret_cast<unsigned long long>(row[t]));
    }
    float dx = 0.f, dy = 0.f;
    for (int c = 0; c < C; ++c) {
        const float gc = g[c] * wl;
        const float t00 = fetch(lvl, B.i00, C, c), t10 = fetch(lvl, B.i10, C, c);
        const float t01 = fetch(lvl, B.i01, C, c), t11 = fetch(lvl, B.i11, C, c);
        dx = fmaf(gc, fmaf(1.f - fy, t10 - t00, fy * (t11 - t01)), dx);
        dy = fmaf(gc, fmaf(fx, t11 - t01, t01) - fmaf(fx, t10 - t00, t00), dy);
        if (vec4) continue;
#pragma unroll
        for (int t = 0; t < 4; ++t) warp_add(row[t] ? row[t] + c : nullptr, gc * wt[t], peers[t]);
    }
    if (vec4) {
        const float4 gc = make_float4(g[0] * wl, g[1] * wl, g[2] * wl, g[3] * wl);
#pragma unroll
        for (int t = 0; t < 4; ++t)
            warp_add4(reinterpret_cast<float4*>(row[t]),
                      make_float4(gc.x * wt[t], gc.y * wt[t], gc.z * wt[t], gc.w * wt[t]), peers[t]);
    }
    gu = fmaf(dx, (float)w, gu);
    gv = fmaf(dy, (float)h, gv);
}

__global__ void __launch_bounds__(256) tex_bwd_kernel(TexArgs a) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.npix) return;
    const int n = (int)(p / a.view_pix), tn = a.Nt == 1 ? 0 : n;
    const float u = a.uv[2 * p], v = a.uv[2 * p + 1];
    const int C = a.C;
    const float* g = a.grad_out + p * C;
    float gu = 0.f, gv = 0.f;
    float4 gda = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.filter == kTexNearest) {
        float* G0 = const_cast<float*>(tex_level(a, a.grad_tex, a.grad_pyr, 0, tn));
        const long long i = nearest_index(a, u, v);
        float* row = i >= 0 ? G0 + i * C : nullptr;
        const unsigned peers = __match_any_sync(__activemask(), reinterpret_cast<unsigned long long>(row));
        for (int c = 0; c < C; ++c) warp_add(row ? row + c : nullptr, g[c], peers);
    } else {
        const TexLod L = tex_lod(a, p);
        const Bilin B0 = bilin_setup(u, v, a.lw[L.l0], a.lh[L.l0], a.boundary);
        const float* P0 = tex_level(a, a.tex, a.pyr, L.l0, tn);
        float* G0 = const_cast<float*>(tex_level(a, a.grad_tex, a.grad_pyr, L.l0, tn));
        const float f = L.f;
        bilin_bwd(P0, G0, B0, a.lw[L.l0], a.lh[L.l0], C, a.vec4, g, f > 0.f ? 1.f - f : 1.f, gu, gv);
        if (f > 0.f) {
            const Bilin B1 = bilin_setup(u, v, a.lw[L.l1], a.lh[L.l1], a.boundary);
            const float* P1 = tex_level(a, a.tex, a.pyr, L.l1, tn);
            float* G1 = const_cast<float*>(tex_level(a, a.grad_tex, a.grad_pyr, L.l1, tn));
            bilin_bwd(P1, G1, B1, a.lw[L.l1], a.lh[L.l1], C, a.vec4, g, f, gu, gv);
            if (a.grad_uv_da && L.interior) {
                float dl = 0.f;
                for (int c = 0; c < C; ++c) dl = fmaf(g[c], bilin_value(P1, B1, C, c) - bilin_value(P0, B0, C, c), dl);
                // lambda = 0.5 log2(r2): d lambda / d r2 = 0.5 / (r2 ln 2)
                const float dr2 = dl * (0.72134752f / L.r2);
                if (L.use_x) {
                    gda.x = dr2 * 2.f * L.ax * (float)a.W;
                    gda.z = dr2 * 2.f * L.ay * (float)a.H;
                } else {
                    gda.y = dr2 * 2.f * L.bx * (float)a.W;
                    gda.w = dr2 * 2.f * L.by * (float)a.H;
                }
            }
        }
    }
    a.grad_uv[2 * p] = gu;
    a.grad_uv[2 * p + 1] = gv;
    if (a.grad_uv_da) a.grad_uv_da[p] = gda;
}

// The texture's level table (sizes, pyramid offsets) after checking its
// arguments.
static int tex_levels_setup(TexArgs& a, const char* who, const float* tex, const float* pyr, int num_tex,
                            int height, int width, int channels, int levels) {
    char msg[160];
    if (!tex || num_tex < 1 || height < 1 || width < 1 || height > (1 << 15) || width > (1 << 15) || channels < 1 ||
        levels < 1 || (levels > 1 && !pyr)) {
        snprintf(msg, sizeof(msg), "%s: bad texture arguments", who);
        drp_set_last_error(msg);
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    int maxl = 0;
    if (drp_texture_levels(height, width, -1, &maxl) || levels > maxl || levels > kTexMaxLevels) {
        snprintf(msg, sizeof(msg), "%s: levels above the texture's pyramid", who);
        drp_set_last_error(msg);
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    a = TexArgs{};
    a.tex = tex;
    a.pyr = pyr;
    a.Nt = num_tex;
    a.H = height;
    a.W = width;
    a.C = channels;
    a.levels = levels;
    long long texels = 0;  // of levels 1 .. k-1
    int h = height, w = width;
    for (int k = 0; k < levels; ++k) {
        a.lh[k] = h;
        a.lw[k] = w;
        a.lofs[k] = k == 0 ? 0 : (long long)num_tex * texels * channels;
        if (k >= 1) texels += (long long)h * w;
        h = h > 1 ? h >> 1 : 1;
        w = w > 1 ? w >> 1 : 1;
    }
    return DRP_STATUS_OK;
}

static int tex_setup(TexArgs& a, const char* who, const float* tex, const float* pyr, int num_tex, int height,
                     int width, int channels, int levels, const float* uv, const float* uv_da, int num_views,
                     int out_height, int out_width, int filter_mode, int boundary_mode) {
    const int st = tex_levels_setup(a, who, tex, pyr, num_tex, height, width, channels, levels);
    if (st) return st;
    if (!uv || num_views < 1 || (num_tex != 1 && num_tex != num_views) || out_height < 0 || out_width < 0 ||
        filter_mode < kTexNearest || filter_mode > kTexMipLinear || boundary_mode < kTexWrap ||
        boundary_mode > kTexZero || (reinterpret_cast<uintptr_t>(uv) & 7) ||
        (reinterpret_cast<uintptr_t>(uv_da) & 15)) {
        char msg[160];
        snprintf(msg, sizeof(msg), "%s: bad sampling arguments", who);
        drp_set_last_error(msg);
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    a.uv = uv;
    a.uv_da = reinterpret_cast<const float4*>(uv_da);
    a.view_pix = (long long)out_height * out_width;
    a.npix = a.view_pix * num_views;
    a.filter = filter_mode;
    a.boundary = boundary_mode;
    return DRP_STATUS_OK;
}

}  // namespace drp

#define DRP_API extern "C" __attribute__((visibility("default")))

DRP_API int drp_texture_levels(int height, int width, int max_mip_level, int* levels) {
    if (!levels || height < 1 || width < 1) {
        drp_set_last_error("drp_texture_levels: bad arguments");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    int n = 1, h = height, w = width;
    while ((h > 1 || w > 1) && (max_mip_level < 0 || n <= max_mip_level)) {
        h = h > 1 ? h >> 1 : 1;
        w = w > 1 ? w >> 1 : 1;
        ++n;
    }
    *levels = n;
    return DRP_STATUS_OK;
}

DRP_API int drp_texture_pyramid_floats(int num_tex, int height, int width, int channels, int levels,
                                       long long* floats) {
    if (!floats || num_tex < 1 || height < 1 || width < 1 || channels < 1 || levels < 1) {
        drp_set_last_error("drp_texture_pyramid_floats: bad arguments");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    long long texels = 0;
    int h = height, w = width;
    for (int k = 1; k < levels; ++k) {
        h = h > 1 ? h >> 1 : 1;
        w = w > 1 ? w >> 1 : 1;
        texels += (long long)h * w;
    }
    *floats = texels * num_tex * channels;
    return DRP_STATUS_OK;
}

DRP_API int drp_texture_mip_build(const float* tex, int num_tex, int height, int width, int channels, int levels,
                                  float* pyr, void* stream) {
    drp::TexArgs a;
    int st = drp::tex_levels_setup(a, "drp_texture_mip_build", tex, pyr, num_tex, height, width, channels, levels);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    for (int k = 1; k < levels; ++k) {
        const float* src = k == 1 ? tex : pyr + a.lofs[k - 1];
        const long long n = (long long)num_tex * a.lh[k] * a.lw[k];
        drp::tex_mip_level_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
            src, pyr + a.lofs[k], num_tex, a.lh[k - 1], a.lw[k - 1], a.lh[k], a.lw[k], channels);
        drp_note_launch();
    }
    return drp_check_launch("drp_texture_mip_build");
}

DRP_API int drp_texture_fwd(const float* tex, const float* pyr, int num_tex, int height, int width, int channels,
                            int levels, const float* uv, const float* uv_da, int num_views, int out_height,
                            int out_width, int filter_mode, int boundary_mode, float* out, void* stream) {
    drp::TexArgs a;
    int st = drp::tex_setup(a, "drp_texture_fwd", tex, pyr, num_tex, height, width, channels, levels, uv, uv_da,
                            num_views, out_height, out_width, filter_mode, boundary_mode);
    if (st) return st;
    if (!out) {
        drp_set_last_error("drp_texture_fwd: null output");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    if (a.npix == 0) return DRP_STATUS_OK;
    a.out = out;
    drp::tex_fwd_kernel<<<(unsigned)((a.npix + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(a);
    drp_note_launch();
    return drp_check_launch("drp_texture_fwd");
}

DRP_API int drp_texture_bwd(const float* tex, const float* pyr, int num_tex, int height, int width, int channels,
                            int levels, const float* uv, const float* uv_da, int num_views, int out_height,
                            int out_width, int filter_mode, int boundary_mode, const float* grad_out,
                            float* grad_tex, float* grad_pyr, float* grad_uv, float* grad_uv_da, void* stream) {
    drp::TexArgs a;
    int st = drp::tex_setup(a, "drp_texture_bwd", tex, pyr, num_tex, height, width, channels, levels, uv, uv_da,
                            num_views, out_height, out_width, filter_mode, boundary_mode);
    if (st) return st;
    if (!grad_out || !grad_tex || !grad_uv || (levels > 1 && !grad_pyr) || (grad_uv_da && !uv_da) ||
        (reinterpret_cast<uintptr_t>(grad_uv) & 7) || (reinterpret_cast<uintptr_t>(grad_uv_da) & 15)) {
        drp_set_last_error("drp_texture_bwd: bad gradient buffers");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    long long pyr_floats = 0;
    drp_texture_pyramid_floats(num_tex, height, width, channels, levels, &pyr_floats);
    if (pyr_floats > 0) cudaMemsetAsync(grad_pyr, 0, sizeof(float) * (size_t)pyr_floats, s);
    a.grad_out = grad_out;
    a.grad_tex = grad_tex;
    a.grad_pyr = grad_pyr;
    a.vec4 = channels == 4 && (reinterpret_cast<uintptr_t>(grad_tex) & 15) == 0 &&
             (reinterpret_cast<uintptr_t>(grad_pyr) & 15) == 0;
    a.grad_uv = grad_uv;
    a.grad_uv_da = reinterpret_cast<float4*>(grad_uv_da);
    if (a.npix > 0) {
        drp::tex_bwd_kernel<<<(unsigned)((a.npix + 255) / 256), 256, 0, s>>>(a);
        drp_note_launch();
    }
    for (int k = levels - 1; k >= 1; --k) {
        float* dst = k == 1 ? grad_tex : grad_pyr + a.lofs[k - 1];
        const long long n = (long long)num_tex * a.lh[k - 1] * a.lw[k - 1];
        drp::tex_mip_bwd_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
            grad_pyr + a.lofs[k], dst, num_tex, a.lh[k - 1], a.lw[k - 1], a.lh[k], a.lw[k], channels);
        drp_note_launch();
    }
    return drp_check_launch("drp_texture_bwd");
}
