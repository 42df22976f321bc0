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
constexpr int kTexWrap = 0, kTexClamp = 1, kTexZero = 2, kTexMirror = 3;
constexpr int kTexMaxLevels = 32;

struct TexArgs {
    const float* tex;
    const float* pyr;
    int Nt, H, W, C, levels;
    int lh[kTexMaxLevels], lw[kTexMaxLevels];
    long long lofs[kTexMaxLevels];  // float offset of level k (k >= 1) in pyr; level k's texture n at + n H_k W_k C
    const float* uv;                // (N, h, w, 2)
    const float4* uv_da;            // (N, h, w) of (du/dX, du/dY, dv/dX, dv/dY), or null
    const float* bias;              // (N, h, w) mip level bias added to the level of detail, or null
    long long npix, view_pix;       // N h w, h w
    int filter, boundary;
    float* out;
    // backward
    const float* grad_out;
    float* grad_tex;
    float* grad_pyr;
    float* grad_uv;
    float4* grad_uv_da;
    float* grad_bias;  // (N, h, w), or null
    // C == 4 with every texel and pixel buffer of the call 16-byte aligned:
    // float4 loads, stores and atomics
    int vec4;
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
    bool interior;   // lambda strictly inside (0, levels - 1): its gradient flows
    bool da_active;  // lambda has the footprint term (uv_da given, footprint > 0)
    float r2;
    bool use_x;
    float ax, ay, bx, by;
};

// da: the pixel's (du/dX, du/dY, dv/dX, dv/dY) (zero without uv_da); b:
// its mip level bias (zero without one).  lambda = 0.5 log2 of the larger
// squared footprint (0 without uv_da or for a zero / non-finite footprint)
// plus the bias, clamped to the pyramid.
__device__ __forceinline__ TexLod tex_lod(const TexArgs& a, float4 da, float b) {
    TexLod L;
    L.l0 = L.l1 = 0;
    L.f = 0.f;
    L.interior = false;
    L.da_active = false;
    L.r2 = 0.f;
    L.use_x = true;
    L.ax = L.ay = L.bx = L.by = 0.f;
    if ((!a.uv_da && !a.bias) || a.levels <= 1 || a.filter < kTexMipNearest) return L;
    float lam = 0.f;
    if (a.uv_da) {
        L.ax = da.x * (float)a.W;
        L.bx = da.y * (float)a.W;
        L.ay = da.z * (float)a.H;
        L.by = da.w * (float)a.H;
        const float lx = L.ax * L.ax + L.ay * L.ay;
        const float ly = L.bx * L.bx + L.by * L.by;
        L.use_x = lx >= ly;
        const float r2 = L.use_x ? lx : ly;
        L.r2 = r2;
        L.da_active = r2 > 0.f && isfinite(r2);
        if (L.da_active) lam = 0.5f * tex_log2(r2);
    }
    if (a.bias) lam = lam + b;
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
    if ((n & (n - 1)) == 0) return i & (n - 1);  // a power of two (two's complement)
    const int r = i % n;
    return r < 0 ? r + n : r;
}

// Mirrored repeat: period 2n, the second half reversed (glTF
// MIRRORED_REPEAT; for bilinear taps the same as reflecting the coordinate
// about the texture's edges, grid_sample's 'reflection' padding).
__device__ __forceinline__ int mirror_index(int i, int n) {
    const int m = wrap_index(i, 2 * n);
    return m < n ? m : 2 * n - 1 - m;
}

// Texel columns (or rows) i and i + 1 of a bilinear tap after the boundary
// rule (texel_index's); -1: outside (zero boundary).
__device__ __forceinline__ void tap_pair(int i, int n, int boundary, int& a, int& b) {
    if (boundary == kTexWrap) {
        a = wrap_index(i, n);
        b = a + 1 == n ? 0 : a + 1;
    } else if (boundary == kTexClamp) {
        a = i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
        b = i + 1 < 0 ? 0 : (i + 1 > n - 1 ? n - 1 : i + 1);
    } else if (boundary == kTexMirror) {
        a = mirror_index(i, n);
        b = mirror_index(i + 1, n);
    } else {
        a = i >= 0 && i < n ? i : -1;
        b = i + 1 >= 0 && i + 1 < n ? i + 1 : -1;
    }
}

// Texel index within its level (textures are at most 2^15 texels a side), or -1.
__device__ __forceinline__ int texel_index(int x, int y, int w, int h, int boundary) {
    if (boundary == kTexWrap) {
        x = wrap_index(x, w);
        y = wrap_index(y, h);
    } else if (boundary == kTexClamp) {
        x = x < 0 ? 0 : (x > w - 1 ? w - 1 : x);
        y = y < 0 ? 0 : (y > h - 1 ? h - 1 : y);
    } else if (boundary == kTexMirror) {
        x = mirror_index(x, w);
        y = mirror_index(y, h);
    } else if (x < 0 || x >= w || y < 0 || y >= h) {
        return -1;
    }
    return y * w + x;
}

__device__ __forceinline__ float tex_coord(float u, int size) {
    float x = u * (float)size - 0.5f;
    const float lim = 16777216.0f;
    if (!(x > -lim)) x = -lim;
    if (x > lim) x = lim;
    return x;
}

struct Bilin {
    int i00, i10, i01, i11;
    float fx, fy;
    int ix, iy;  // the tap's first texel before the boundary rule
};

__device__ __forceinline__ Bilin bilin_setup(float u, float v, int w, int h, int boundary) {
    Bilin B;
    const float x = tex_coord(u, w), y = tex_coord(v, h);
    const float x0 = floorf(x), y0 = floorf(y);
    B.fx = x - x0;
    B.fy = y - y0;
    const int ix = (int)x0, iy = (int)y0;
    B.ix = ix;
    B.iy = iy;
    int xa, xb, ya, yb;
    tap_pair(ix, w, boundary, xa, xb);
    tap_pair(iy, h, boundary, ya, yb);
    B.i00 = xa < 0 || ya < 0 ? -1 : ya * w + xa;
    B.i10 = xb < 0 || ya < 0 ? -1 : ya * w + xb;
    B.i01 = xa < 0 || yb < 0 ? -1 : yb * w + xa;
    B.i11 = xb < 0 || yb < 0 ? -1 : yb * w + xb;
    return B;
}

__device__ __forceinline__ float fetch(const float* lvl, int i, int C, int c) {
    return i < 0 ? 0.f : __ldg(lvl + (long long)i * C + c);
}

__device__ __forceinline__ float4 fetch4(const float* lvl, int i) {
    return i < 0 ? make_float4(0.f, 0.f, 0.f, 0.f) : __ldg(reinterpret_cast<const float4*>(lvl) + i);
}

__device__ __forceinline__ float bilerp(const Bilin& B, float t00, float t10, float t01, float t11) {
    const float r0 = fmaf(B.fx, t10 - t00, t00), r1 = fmaf(B.fx, t11 - t01, t01);
    return fmaf(B.fy, r1 - r0, r0);
}

__device__ __forceinline__ float bilin_value(const float* lvl, const Bilin& B, int C, int c) {
    return bilerp(B, fetch(lvl, B.i00, C, c), fetch(lvl, B.i10, C, c), fetch(lvl, B.i01, C, c),
                  fetch(lvl, B.i11, C, c));
}

// The four texels of a bilinear tap, four channels each.
struct Quad {
    float4 t00, t10, t01, t11;
};

__device__ __forceinline__ Quad fetch_quad(const float* lvl, const Bilin& B) {
    return Quad{fetch4(lvl, B.i00), fetch4(lvl, B.i10), fetch4(lvl, B.i01), fetch4(lvl, B.i11)};
}

__device__ __forceinline__ float4 bilerp4(const Bilin& B, const Quad& q) {
    return make_float4(bilerp(B, q.t00.x, q.t10.x, q.t01.x, q.t11.x), bilerp(B, q.t00.y, q.t10.y, q.t01.y, q.t11.y),
                       bilerp(B, q.t00.z, q.t10.z, q.t01.z, q.t11.z), bilerp(B, q.t00.w, q.t10.w, q.t01.w, q.t11.w));
}

__device__ __forceinline__ int nearest_index(const TexArgs& a, float u, float v) {
    const int ix = (int)floorf(tex_coord(u, a.W) + 0.5f), iy = (int)floorf(tex_coord(v, a.H) + 0.5f);
    return texel_index(ix, iy, a.W, a.H, a.boundary);
}

// Levels base + 1 .. base + nl of every texture from level base.  Level k
// texel (x, y) is the 2x2 box average (((a + b) + c) + d) / 4 of level k - 1
// at x0 = 2x, x1 = 2x + 1, y0 = 2y, y1 = 2y + 1, indices clamped to level
// k - 1.  One CTA builds a side x side tile of level base + 1 and the tiles
// above it (side / 2, side / 4, ...), each level from the one below in shared
// memory (a tile's parents lie in the tile below it), writing every level to
// the pyramid: the same values as one pass per level, in one launch.
__global__ void __launch_bounds__(256) tex_mip_tile_kernel(TexArgs a, int base, int nl, int side, int tiles_x,
                                                           int tiles_y) {
    extern __shared__ float4 sm4[];
    float* sm = reinterpret_cast<float*>(sm4);
    const int C = a.C;
    const int per = tiles_x * tiles_y;
    const int n = blockIdx.x / per;
    const int rr = blockIdx.x - n * per;
    const int ty = rr / tiles_x, tx = rr - ty * tiles_x;
    const float* src = tex_level(a, a.tex, a.pyr, base, n);
    int pw = a.lw[base], ph = a.lh[base];
    int prev_off = 0, prev_side = 0, off = 0;
    for (int s = 0; s < nl; ++s) {
        const int k = base + 1 + s;
        const int T = side >> s, w = a.lw[k], h = a.lh[k];
        const int ox = tx * T, oy = ty * T;
        float* dst = const_cast<float*>(tex_level(a, a.pyr, a.pyr, k, n));
        for (int t = threadIdx.x; t < T * T; t += blockDim.x) {
            const int ly = t / T, lx = t - ly * T;
            const int x = ox + lx, y = oy + ly;
            if (x >= w || y >= h) continue;
            const int x0 = 2 * x < pw - 1 ? 2 * x : pw - 1, x1 = 2 * x + 1 < pw - 1 ? 2 * x + 1 : pw - 1;
            const int y0 = 2 * y < ph - 1 ? 2 * y : ph - 1, y1 = 2 * y + 1 < ph - 1 ? 2 * y + 1 : ph - 1;
            if (s == 0 && a.vec4) {  // four channels, one float4 load per texel (the same sums)
                const float4* q = reinterpret_cast<const float4*>(src);
                const float4 ta = __ldg(q + (long long)y0 * pw + x0), tb = __ldg(q + (long long)y0 * pw + x1);
                const float4 tc = __ldg(q + (long long)y1 * pw + x0), td = __ldg(q + (long long)y1 * pw + x1);
                const float4 r = make_float4((((ta.x + tb.x) + tc.x) + td.x) * 0.25f, (((ta.y + tb.y) + tc.y) + td.y) * 0.25f,
                                             (((ta.z + tb.z) + tc.z) + td.z) * 0.25f, (((ta.w + tb.w) + tc.w) + td.w) * 0.25f);
                reinterpret_cast<float4*>(dst)[(long long)y * w + x] = r;
                if (s + 1 < nl) reinterpret_cast<float4*>(sm + off)[ly * T + lx] = r;
                continue;
            }
            for (int c = 0; c < C; ++c) {
                float pa, pb, pc, pd;
                if (s == 0) {
                    pa = src[((long long)y0 * pw + x0) * C + c];
                    pb = src[((long long)y0 * pw + x1) * C + c];
                    pc = src[((long long)y1 * pw + x0) * C + c];
                    pd = src[((long long)y1 * pw + x1) * C + c];
                } else {  // the tile below starts at (2 ox, 2 oy)
                    const float* q = sm + prev_off;
                    pa = q[((y0 - 2 * oy) * prev_side + (x0 - 2 * ox)) * C + c];
                    pb = q[((y0 - 2 * oy) * prev_side + (x1 - 2 * ox)) * C + c];
                    pc = q[((y1 - 2 * oy) * prev_side + (x0 - 2 * ox)) * C + c];
                    pd = q[((y1 - 2 * oy) * prev_side + (x1 - 2 * ox)) * C + c];
                }
                const float v = (((pa + pb) + pc) + pd) * 0.25f;
                dst[((long long)y * w + x) * C + c] = v;
                if (s + 1 < nl) sm[off + (ly * T + lx) * C + c] = v;
            }
        }
        __syncthreads();
        prev_off = off;
        prev_side = T;
        off += T * T * C;
        pw = w;
        ph = h;
    }
}

// Pixels per thread of the sampling kernels: every pixel's uv and uv_da are
// loaded first, so that the later pixels' loads overlap the first's work.
constexpr int kTexPix = 2;

// The pixel's uv, uv_da and mip level bias (zero without them).
struct TexIn {
    float u, v, b;
    float4 da;
};

__device__ __forceinline__ TexIn tex_inputs(const TexArgs& a, long long p) {
    const float2 uv = reinterpret_cast<const float2*>(a.uv)[p];
    TexIn in;
    in.u = uv.x;
    in.v = uv.y;
    in.da = a.uv_da ? a.uv_da[p] : make_float4(0.f, 0.f, 0.f, 0.f);
    in.b = a.bias ? a.bias[p] : 0.f;
    return in;
}

__device__ __forceinline__ void tex_fwd_pixel(const TexArgs& a, long long p, const TexIn& in) {
    const float u = in.u, v = in.v;
    const int n = (int)(p / a.view_pix), tn = a.Nt == 1 ? 0 : n;
    const int C = a.C;
    float* o = a.out + p * C;
    if (a.filter == kTexNearest) {
        const float* l0 = tex_level(a, a.tex, a.pyr, 0, tn);
        const int i = nearest_index(a, u, v);
        for (int c = 0; c < C; ++c) o[c] = fetch(l0, i, C, c);
        return;
    }
    const TexLod L = tex_lod(a, in.da, in.b);
    const Bilin B0 = bilin_setup(u, v, a.lw[L.l0], a.lh[L.l0], a.boundary);
    const float* v0 = tex_level(a, a.tex, a.pyr, L.l0, tn);
    if (a.vec4) {  // the same arithmetic per channel, one load per texel
        float4 r = bilerp4(B0, fetch_quad(v0, B0));
        if (L.f > 0.f) {
            const Bilin B1 = bilin_setup(u, v, a.lw[L.l1], a.lh[L.l1], a.boundary);
            const float4 s1 = bilerp4(B1, fetch_quad(tex_level(a, a.tex, a.pyr, L.l1, tn), B1));
            r = make_float4(fmaf(L.f, s1.x - r.x, r.x), fmaf(L.f, s1.y - r.y, r.y), fmaf(L.f, s1.z - r.z, r.z),
                            fmaf(L.f, s1.w - r.w, r.w));
        }
        reinterpret_cast<float4*>(a.out)[p] = r;
        return;
    }
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

// kTexPix pixels per thread, blockDim.x apart.
__global__ void __launch_bounds__(256, 3) tex_fwd_kernel(TexArgs a) {
    const long long base = (long long)blockIdx.x * (kTexPix * blockDim.x) + threadIdx.x;
    TexIn in[kTexPix];
#pragma unroll
    for (int j = 0; j < kTexPix; ++j)
        if (base + j * blockDim.x < a.npix) in[j] = tex_inputs(a, base + j * blockDim.x);
#pragma unroll
    for (int j = 0; j < kTexPix; ++j)
        if (base + j * blockDim.x < a.npix) tex_fwd_pixel(a, base + j * blockDim.x, in[j]);
}

// Sum of v over this lane's group (the lanes of `peers`, all of `active`
// taking part), left in the group's lowest lane: pointer jumping along the
// group in lane order, ceil(log2(largest group)) rounds of shuffles instead of
// one per member.  Under minification thousands of pixels land on the same
// few texels of the coarse levels, so groups are large.
template <int N>
__device__ __forceinline__ void group_sum(float (&v)[N], unsigned peers, unsigned active) {
    const int lane = threadIdx.x & 31;
    const unsigned after = lane == 31 ? 0u : peers & (~0u << (lane + 1));
    int next = after ? __ffs(after) - 1 : -1;
    const int largest = __reduce_max_sync(active, (unsigned)__popc(peers));
    const int rounds = largest <= 1 ? 0 : 32 - __clz(largest - 1);
    for (int r = 0; r < rounds; ++r) {
        const int src = next >= 0 ? next : lane;
        float o[N];
#pragma unroll
        for (int c = 0; c < N; ++c) o[c] = __shfl_sync(active, v[c], src);
        const int nn = __shfl_sync(active, next, src);
        if (next >= 0) {
#pragma unroll
            for (int c = 0; c < N; ++c) v[c] += o[c];
            next = nn;
        }
    }
}

// Adds v (N consecutive floats; N == 4: a 16-byte aligned float4) into dst
// from every lane of the warp whose dst is the same address: one atomic per
// group, issued by its lowest lane.  nullptr: nothing to add (the lane still
// takes part).
template <int N>
__device__ __forceinline__ void warp_add(float* dst, float (&v)[N], unsigned active) {
    const unsigned peers = __match_any_sync(active, reinterpret_cast<unsigned long long>(dst));
    group_sum<N>(v, peers, active);
    if (!dst || (threadIdx.x & 31) != __ffs(peers) - 1) return;
    if constexpr (N == 4) {
        atomicAdd(reinterpret_cast<float4*>(dst), make_float4(v[0], v[1], v[2], v[3]));
    } else {
        atomicAdd(dst, v[0]);
    }
}

__device__ __forceinline__ float* grad_level(const TexArgs& a, int k, int n) {
    return const_cast<float*>(tex_level(a, a.grad_tex, a.grad_pyr, k, n));
}

__device__ __forceinline__ void bilin_bwd(const float* lvl, float* glvl, const Bilin& B, int w, int h, int C,
                                          const float* g, float wl, float& gu, float& gv) {
    const float fx = B.fx, fy = B.fy;
    const float wt[4] = {(1.f - fx) * (1.f - fy), fx * (1.f - fy), (1.f - fx) * fy, fx * fy};
    const int idx[4] = {B.i00, B.i10, B.i01, B.i11};
    const unsigned active = __activemask();
    float dx = 0.f, dy = 0.f;
    for (int c = 0; c < C; ++c) {
        const float gc = g[c] * wl;
        const float t00 = fetch(lvl, B.i00, C, c), t10 = fetch(lvl, B.i10, C, c);
        const float t01 = fetch(lvl, B.i01, C, c), t11 = fetch(lvl, B.i11, C, c);
        dx = fmaf(gc, fmaf(1.f - fy, t10 - t00, fy * (t11 - t01)), dx);
        dy = fmaf(gc, fmaf(fx, t11 - t01, t01) - fmaf(fx, t10 - t00, t00), dy);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            float val[1] = {gc * wt[t]};
            warp_add<1>(idx[t] >= 0 ? glvl + (long long)idx[t] * C + c : nullptr, val, active);
        }
    }
    gu = fmaf(dx, (float)w, gu);
    gv = fmaf(dy, (float)h, gv);
}

// bilin_bwd of four channels from one float4 load per texel (the same
// arithmetic per channel); q: the texels.  Lanes whose taps start at the same
// texel (ix, iy) of the same level and texture share all four texels: one
// match finds them, one group sum adds their 4 x 4 values and the group's
// lowest lane issues the four float4 atomics.
__device__ __forceinline__ void bilin_bwd4(const Quad& q, float* glvl, const Bilin& B, int level, int tn,
                                           bool per_view, int w, int h, float4 g4, float wl, float& gu,
                                           float& gv) {
    const float fx = B.fx, fy = B.fy;
    const float wt[4] = {(1.f - fx) * (1.f - fy), fx * (1.f - fy), (1.f - fx) * fy, fx * fy};
    const int idx[4] = {B.i00, B.i10, B.i01, B.i11};
    const unsigned active = __activemask();
    const float gc[4] = {g4.x * wl, g4.y * wl, g4.z * wl, g4.w * wl};
    const float a00[4] = {q.t00.x, q.t00.y, q.t00.z, q.t00.w}, a10[4] = {q.t10.x, q.t10.y, q.t10.z, q.t10.w};
    const float a01[4] = {q.t01.x, q.t01.y, q.t01.z, q.t01.w}, a11[4] = {q.t11.x, q.t11.y, q.t11.z, q.t11.w};
    float dx = 0.f, dy = 0.f;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const float t00 = a00[c], t10 = a10[c], t01 = a01[c], t11 = a11[c];
        dx = fmaf(gc[c], fmaf(1.f - fy, t10 - t00, fy * (t11 - t01)), dx);
        dy = fmaf(gc[c], fmaf(fx, t11 - t01, t01) - fmaf(fx, t10 - t00, t00), dy);
    }
    // ix, iy within +-2^24 + 1 (tex_coord's clamp): 26 bits each after the offset
    const unsigned long long key = ((unsigned long long)level << 56) |
                                   ((unsigned long long)((B.ix + (1 << 25)) & 0x3ffffff) << 26) |
                                   (unsigned long long)((B.iy + (1 << 25)) & 0x3ffffff);
    unsigned peers = __match_any_sync(active, key);
    if (per_view) peers &= __match_any_sync(active, (unsigned)tn);
    float val[16];
#pragma unroll
    for (int t = 0; t < 4; ++t)
#pragma unroll
        for (int c = 0; c < 4; ++c) val[4 * t + c] = gc[c] * wt[t];
    group_sum<16>(val, peers, active);
    if ((threadIdx.x & 31) == __ffs(peers) - 1) {
#pragma unroll
        for (int t = 0; t < 4; ++t)
            if (idx[t] >= 0)
                atomicAdd(reinterpret_cast<float4*>(glvl) + idx[t],
                          make_float4(val[4 * t], val[4 * t + 1], val[4 * t + 2], val[4 * t + 3]));
    }
    gu = fmaf(dx, (float)w, gu);
    gv = fmaf(dy, (float)h, gv);
}

// One pixel's gradients: texel gradients added into the levels, the uv and
// uv_da gradients written.
__device__ __forceinline__ void tex_bwd_pixel(const TexArgs& a, long long p, const TexIn& in) {
    const float u = in.u, v = in.v;
    const int n = (int)(p / a.view_pix), tn = a.Nt == 1 ? 0 : n;
    const int C = a.C;
    const float* g = a.grad_out + p * C;
    float gu = 0.f, gv = 0.f, gb = 0.f;
    float4 gda = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.filter == kTexNearest) {
        float* G0 = grad_level(a, 0, tn);
        const int i = nearest_index(a, u, v);
        const unsigned active = __activemask();
        for (int c = 0; c < C; ++c) {
            float val[1] = {g[c]};
            warp_add<1>(i >= 0 ? G0 + (long long)i * C + c : nullptr, val, active);
        }
    } else {
        const TexLod L = tex_lod(a, in.da, in.b);
        const Bilin B0 = bilin_setup(u, v, a.lw[L.l0], a.lh[L.l0], a.boundary);
        const float* P0 = tex_level(a, a.tex, a.pyr, L.l0, tn);
        const float f = L.f;
        const bool want_dl = (a.grad_uv_da || a.grad_bias) && L.interior;
        float dl = 0.f;  // d out / d lambda . grad_out
        if (a.vec4) {
            const float4 g4 = reinterpret_cast<const float4*>(a.grad_out)[p];
            const Quad q0 = fetch_quad(P0, B0);
            bilin_bwd4(q0, grad_level(a, L.l0, tn), B0, L.l0, tn, a.Nt > 1, a.lw[L.l0], a.lh[L.l0], g4,
                       f > 0.f ? 1.f - f : 1.f, gu, gv);
            if (f > 0.f) {
                const Bilin B1 = bilin_setup(u, v, a.lw[L.l1], a.lh[L.l1], a.boundary);
                const Quad q1 = fetch_quad(tex_level(a, a.tex, a.pyr, L.l1, tn), B1);
                bilin_bwd4(q1, grad_level(a, L.l1, tn), B1, L.l1, tn, a.Nt > 1, a.lw[L.l1], a.lh[L.l1], g4, f, gu,
                           gv);
                if (want_dl) {
                    const float4 s0 = bilerp4(B0, q0), s1 = bilerp4(B1, q1);
                    dl = fmaf(g4.x, s1.x - s0.x, dl);
                    dl = fmaf(g4.y, s1.y - s0.y, dl);
                    dl = fmaf(g4.z, s1.z - s0.z, dl);
                    dl = fmaf(g4.w, s1.w - s0.w, dl);
                }
            }
        } else {
            bilin_bwd(P0, grad_level(a, L.l0, tn), B0, a.lw[L.l0], a.lh[L.l0], C, g, f > 0.f ? 1.f - f : 1.f, gu,
                      gv);
            if (f > 0.f) {
                const Bilin B1 = bilin_setup(u, v, a.lw[L.l1], a.lh[L.l1], a.boundary);
                const float* P1 = tex_level(a, a.tex, a.pyr, L.l1, tn);
                bilin_bwd(P1, grad_level(a, L.l1, tn), B1, a.lw[L.l1], a.lh[L.l1], C, g, f, gu, gv);
                if (want_dl)
                    for (int c = 0; c < C; ++c)
                        dl = fmaf(g[c], bilin_value(P1, B1, C, c) - bilin_value(P0, B0, C, c), dl);
            }
        }
        if (f > 0.f && want_dl) gb = dl;
        if (f > 0.f && want_dl && a.grad_uv_da && L.da_active) {
            // lambda = 0.5 log2(r2) + bias: d lambda / d r2 = 0.5 / (r2 ln 2)
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
    reinterpret_cast<float2*>(a.grad_uv)[p] = make_float2(gu, gv);
    if (a.grad_uv_da) a.grad_uv_da[p] = gda;
    if (a.grad_bias) a.grad_bias[p] = gb;
}

// kTexPix pixels per thread, blockDim.x apart (the warp's lanes take each
// pixel together: its atomics are aggregated over the warp).
__global__ void __launch_bounds__(256, 3) tex_bwd_kernel(TexArgs a) {
    const long long base = (long long)blockIdx.x * (kTexPix * blockDim.x) + threadIdx.x;
    TexIn in[kTexPix];
#pragma unroll
    for (int j = 0; j < kTexPix; ++j)
        if (base + j * blockDim.x < a.npix) in[j] = tex_inputs(a, base + j * blockDim.x);
#pragma unroll
    for (int j = 0; j < kTexPix; ++j)
        if (base + j * blockDim.x < a.npix) tex_bwd_pixel(a, base + j * blockDim.x, in[j]);
}

__device__ __forceinline__ float vadd(float a, float b) { return a + b; }
__device__ __forceinline__ float vscale(float m, float t) { return m * t; }
__device__ __forceinline__ float4 vadd(float4 a, float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ float4 vscale(float m, float4 t) { return make_float4(m * t.x, m * t.y, m * t.z, m * t.w); }

constexpr int kTexMaxChain = 15;  // pyramid levels above level 0 of a texture of at most 2^15 texels a side

// The cascade of one channel group (V: float or float4) of level-1 texel
// (x1, y1): every level's load issued first (levels above the top read the
// top again; registers only), then the evaluation from the top.  MAXC: the
// longest chain the launch holds (top <= MAXC), so that a pyramid of few
// levels keeps few registers.
template <typename V, int MAXC>
__device__ __forceinline__ V mip_chain(const TexArgs& a, int n, int x1, int y1, int top, int c) {
    V g[MAXC];
#pragma unroll
    for (int k = 1; k <= MAXC; ++k) {  // level k holds (x1, y1)'s ancestor (x1 >> (k - 1), y1 >> (k - 1))
        const int j = k < top ? k : top;
        const float* G = a.grad_pyr + a.lofs[j] + (long long)n * a.lh[j] * a.lw[j] * a.C;
        g[k - 1] = *reinterpret_cast<const V*>(G + ((long long)(y1 >> (j - 1)) * a.lw[j] + (x1 >> (j - 1))) * a.C + c);
    }
    V t = g[0];
#pragma unroll
    for (int k = MAXC; k >= 1; --k) {
        if (k > top) continue;
        if (k == top) {
            t = g[k - 1];
        } else {
            const float m = (0.25f * (a.lw[k] == 1 ? 2.f : 1.f)) * (a.lh[k] == 1 ? 2.f : 1.f);
            t = vadd(g[k - 1], vscale(m, t));
        }
    }
    return t;
}

// Pyramid backward in one pass: texel (x, y) of level k - 1 receives 0.25 of
// texel (x >> 1, y >> 1) of level k (twice along an axis of size 1; nothing
// beyond twice level k's size), after level k has received its own share
// from level k + 1.  One thread per level-1 texel follows its chain of
// parents and evaluates that cascade from the top (t_{k-1} = G_{k-1} +
// c_{k-1} t_k, the operations of one pass per level in the same order), then
// adds c_0 t_1 into the gradients of its (up to) four level-0 texels.
template <int MAXC>
__global__ void __launch_bounds__(256) tex_mip_chain_kernel(TexArgs a) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int w1 = a.lw[1], h1 = a.lh[1];
    const long long per = (long long)h1 * w1;
    if (i >= (long long)a.Nt * per) return;
    const int n = (int)(i / per);
    const int r = (int)(i - (long long)n * per);
    const int y1 = r / w1, x1 = r - y1 * w1;
    int top = 1;  // the highest level of the chain
    while (top + 1 < a.levels && (x1 >> top) < a.lw[top + 1] && (y1 >> top) < a.lh[top + 1]) ++top;
    const float m = (0.25f * (a.W == 1 ? 2.f : 1.f)) * (a.H == 1 ? 2.f : 1.f);
    const int C = a.C;
    float* g0 = a.grad_tex + (long long)n * a.H * a.W * C;
    if (a.vec4) {
        const float4 t = vscale(m, mip_chain<float4, MAXC>(a, n, x1, y1, top, 0));
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                const int x = 2 * x1 + dx, y = 2 * y1 + dy;
                if (x >= a.W || y >= a.H) continue;
                float4* d = reinterpret_cast<float4*>(g0) + (long long)y * a.W + x;
                *d = vadd(*d, t);
            }
    } else {
        for (int c = 0; c < C; ++c) {
            const float t = m * mip_chain<float, MAXC>(a, n, x1, y1, top, c);
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) {
                    const int x = 2 * x1 + dx, y = 2 * y1 + dy;
                    if (x >= a.W || y >= a.H) continue;
                    float* d = g0 + ((long long)y * a.W + x) * C + c;
                    *d = *d + t;
                }
        }
    }
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
                     int width, int channels, int levels, const float* uv, const float* uv_da, const float* bias,
                     int num_views, int out_height, int out_width, int filter_mode, int boundary_mode) {
    const int st = tex_levels_setup(a, who, tex, pyr, num_tex, height, width, channels, levels);
    if (st) return st;
    if (!uv || num_views < 1 || (num_tex != 1 && num_tex != num_views) || out_height < 0 || out_width < 0 ||
        filter_mode < kTexNearest || filter_mode > kTexMipLinear || boundary_mode < kTexWrap ||
        boundary_mode > kTexMirror || (reinterpret_cast<uintptr_t>(uv) & 7) ||
        (reinterpret_cast<uintptr_t>(uv_da) & 15) || (reinterpret_cast<uintptr_t>(bias) & 3)) {
        char msg[160];
        snprintf(msg, sizeof(msg), "%s: bad sampling arguments", who);
        drp_set_last_error(msg);
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    a.uv = uv;
    a.uv_da = reinterpret_cast<const float4*>(uv_da);
    a.bias = bias;
    a.view_pix = (long long)out_height * out_width;
    a.npix = a.view_pix * num_views;
    a.filter = filter_mode;
    a.boundary = boundary_mode;
    return DRP_STATUS_OK;
}

}  // namespace drp

#define DRP_API extern "C" __attribute__((visibility("default")))

static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

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
    // tile side: 16 texels, less where the tiles of C channels exceed 48 KB
    int side = 16, per_launch = 5;
    while (side > 1 && (size_t)side * side * 2 * channels * sizeof(float) > (48u << 10)) {
        side >>= 1;
        --per_launch;
    }
    if ((size_t)side * side * 2 * channels * sizeof(float) > (48u << 10)) {
        drp_set_last_error("drp_texture_mip_build: more than 6144 channels");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    a.vec4 = channels == 4 && aligned16(tex) && aligned16(pyr);
    for (int base = 0; base + 1 < levels; base += per_launch) {
        const int nl = levels - 1 - base < per_launch ? levels - 1 - base : per_launch;
        const int tiles_x = (a.lw[base + 1] + side - 1) / side, tiles_y = (a.lh[base + 1] + side - 1) / side;
        const long long blocks = (long long)num_tex * tiles_x * tiles_y;
        if (blocks > 0x7fffffff) {
            drp_set_last_error("drp_texture_mip_build: too many textures");
            return DRP_STATUS_INVALID_ARGUMENT;
        }
        const size_t smem = (size_t)side * side * 2 * channels * sizeof(float);  // the tiles above the first
        drp::tex_mip_tile_kernel<<<(unsigned)blocks, 256, smem, s>>>(a, base, nl, side, tiles_x, tiles_y);
        drp_note_launch();
    }
    return drp_check_launch("drp_texture_mip_build");
}

DRP_API int drp_texture_fwd(const float* tex, const float* pyr, int num_tex, int height, int width, int channels,
                            int levels, const float* uv, const float* uv_da, const float* mip_level_bias,
                            int num_views, int out_height, int out_width, int filter_mode, int boundary_mode,
                            float* out, void* stream) {
    drp::TexArgs a;
    int st = drp::tex_setup(a, "drp_texture_fwd", tex, pyr, num_tex, height, width, channels, levels, uv, uv_da,
                            mip_level_bias, num_views, out_height, out_width, filter_mode, boundary_mode);
    if (st) return st;
    if (!out) {
        drp_set_last_error("drp_texture_fwd: null output");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    if (a.npix == 0) return DRP_STATUS_OK;
    a.out = out;
    a.vec4 = channels == 4 && aligned16(tex) && aligned16(pyr) && aligned16(out);
    const long long per_block = 256 * drp::kTexPix;
    drp::tex_fwd_kernel<<<(unsigned)((a.npix + per_block - 1) / per_block), 256, 0,
                          static_cast<cudaStream_t>(stream)>>>(a);
    drp_note_launch();
    return drp_check_launch("drp_texture_fwd");
}

DRP_API int drp_texture_bwd(const float* tex, const float* pyr, int num_tex, int height, int width, int channels,
                            int levels, const float* uv, const float* uv_da, const float* mip_level_bias,
                            int num_views, int out_height, int out_width, int filter_mode, int boundary_mode,
                            const float* grad_out, float* grad_tex, float* grad_pyr, float* grad_uv,
                            float* grad_uv_da, float* grad_mip_level_bias, void* stream) {
    drp::TexArgs a;
    int st = drp::tex_setup(a, "drp_texture_bwd", tex, pyr, num_tex, height, width, channels, levels, uv, uv_da,
                            mip_level_bias, num_views, out_height, out_width, filter_mode, boundary_mode);
    if (st) return st;
    if (!grad_out || !grad_tex || !grad_uv || (levels > 1 && !grad_pyr) || (grad_uv_da && !uv_da) ||
        (grad_mip_level_bias && !mip_level_bias) || (reinterpret_cast<uintptr_t>(grad_uv) & 7) ||
        (reinterpret_cast<uintptr_t>(grad_uv_da) & 15) || (reinterpret_cast<uintptr_t>(grad_mip_level_bias) & 3)) {
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
    a.vec4 = channels == 4 && aligned16(tex) && aligned16(pyr) && aligned16(grad_out) && aligned16(grad_tex) &&
             aligned16(grad_pyr);
    a.grad_uv = grad_uv;
    a.grad_uv_da = reinterpret_cast<float4*>(grad_uv_da);
    a.grad_bias = grad_mip_level_bias;
    if (a.npix > 0) {
        const long long per_block = 256 * drp::kTexPix;
        drp::tex_bwd_kernel<<<(unsigned)((a.npix + per_block - 1) / per_block), 256, 0, s>>>(a);
        drp_note_launch();
    }
    if (levels > 1 && a.filter >= drp::kTexMipNearest) {
        const long long n = (long long)num_tex * a.lh[1] * a.lw[1];
        const unsigned grid = (unsigned)((n + 255) / 256);
        if (levels - 1 <= 7)
            drp::tex_mip_chain_kernel<7><<<grid, 256, 0, s>>>(a);
        else if (levels - 1 <= 11)
            drp::tex_mip_chain_kernel<11><<<grid, 256, 0, s>>>(a);
        else
            drp::tex_mip_chain_kernel<drp::kTexMaxChain><<<grid, 256, 0, s>>>(a);
        drp_note_launch();
    }
    return drp_check_launch("drp_texture_bwd");
}
