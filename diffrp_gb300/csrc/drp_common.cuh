// drp_common.cuh -- device helpers shared by the diffrp_gb300 kernels.
//
// Floating-point contract: every translation unit is compiled with
// --fmad=false, so float expressions round once per operation in source order
// and the only fused multiply-adds are explicit fmaf() calls.  Visibility,
// rast, rast_db and the forward images are therefore bit-identical to a CPU
// evaluation of the same expressions.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define DRP_SUBPIX_BITS 8
#define DRP_SUBPIX 256
#define DRP_HALF_SUBPIX 128
#define DRP_GUARD 64.0f
#define DRP_MAX_POLY 8
#define DRP_MAX_RES 16384

// Device-side error bits (stats word 2).
#define DRP_DEVERR_BAD_INDEX 1u
#define DRP_DEVERR_LIST_OVERFLOW 2u
#define DRP_DEVERR_CHANNELS 4u

namespace drp {

// Programmatic dependent launch (Hopper and later).  A kernel launched with
// launch_pdl() (drp_internal.h) may be scheduled before the kernel ahead of
// it in the stream has finished, which hides the launch gap between the
// dependent kernels of one pass.  pdl_wait() (griddepcontrol.wait) blocks
// until the kernel ahead has completed and its memory writes are visible:
// every kernel launched with launch_pdl() calls it before its first global
// memory access.  pdl_launch_dependents() (griddepcontrol.launch_dependents)
// lets the next kernel's CTAs be scheduled once every CTA of this grid has
// issued it or exited.  Both are no-ops in a kernel launched without the
// attribute.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" :::); }


// ---------------------------------------------------------------------------
// Triangle id <-> float encoding of the rast w channel
// (diffrp/rendering/interpolator.py:24-29): ids up to 2^24 are stored as exact
// floats, larger ids as the float whose bit pattern is 0x4a800000 + id.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float enc_triid(int32_t id1) {
    if (id1 <= 0x01000000) return (float)id1;
    return __uint_as_float(0x4a800000u + (uint32_t)id1);
}

__device__ __forceinline__ int32_t dec_triid(float f) {
    if (f <= 16777216.0f) return (int32_t)f;
    return (int32_t)(__float_as_uint(f) - 0x4a800000u);
}

// Triangle index (0-based) from a rast w value, -1 for background.
__device__ __forceinline__ int32_t rast_tri(float w) {
    if (!(w > 0.0f)) return -1;
    return dec_triid(w) - 1;
}

// Triangle of a caller-supplied rast row, validated: -1 unless the id is in
// [0, F) and its three vertex indices are in [0, V).
__device__ __forceinline__ int32_t checked_tri(float w, const int* tri, long long F, long long V, int& i0, int& i1,
                                               int& i2) {
    const int32_t t = rast_tri(w);
    if (t < 0 || t >= F) return -1;
    i0 = tri[3 * (long long)t];
    i1 = tri[3 * (long long)t + 1];
    i2 = tri[3 * (long long)t + 2];
    if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= V || i1 >= V || i2 >= V) return -1;
    return t;
}

__device__ __forceinline__ uint32_t depth_order(float z) {
    uint32_t b = __float_as_uint(z);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ __forceinline__ int64_t floor_shift(int64_t a) { return a >> DRP_SUBPIX_BITS; }
__device__ __forceinline__ int64_t ceil_shift(int64_t a) { return -((-a) >> DRP_SUBPIX_BITS); }

// ---------------------------------------------------------------------------
// Setup: trivial reject, near-plane / guard-band clipping, projection, snap.
// ---------------------------------------------------------------------------
struct Poly {
    int n;
    int32_t X[DRP_MAX_POLY], Y[DRP_MAX_POLY];
    float Z[DRP_MAX_POLY];
};

__device__ __forceinline__ float plane_dist(const float4& p, int plane) {
    switch (plane) {
    case 0: return p.z + p.w;
    case 1: return DRP_GUARD * p.w - p.x;
    case 2: return p.x + DRP_GUARD * p.w;
    case 3: return DRP_GUARD * p.w - p.y;
    default: return p.y + DRP_GUARD * p.w;
    }
}

__device__ __forceinline__ float frustum_dist(const float4& p, int plane) {
    switch (plane) {
    case 0: return p.w + p.x;
    case 1: return p.w - p.x;
    case 2: return p.w + p.y;
    case 3: return p.w - p.y;
    case 4: return p.w + p.z;
    default: return p.w - p.z;
    }
}

__device__ __forceinline__ bool finite4(const float4& p) {
    return isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(p.w);
}

__device__ __forceinline__ int32_t snap_coord(float c, float w, int res) {
    float q = c / w;
    float s = (q + 1.0f) * (float)(res * DRP_HALF_SUBPIX);
    return __float2int_rn(s);
}

// 0 = culled, 1 = simple triangle (no clipping), 2 = clipped polygon.
__device__ __forceinline__ int needs_clip_or_cull(const float4& p0, const float4& p1, const float4& p2) {
    if (!finite4(p0) || !finite4(p1) || !finite4(p2)) return 0;
#pragma unroll
    for (int pl = 0; pl < 6; ++pl)
        if (frustum_dist(p0, pl) < 0.0f && frustum_dist(p1, pl) < 0.0f && frustum_dist(p2, pl) < 0.0f) return 0;
    bool need = !(p0.w > 0.0f) || !(p1.w > 0.0f) || !(p2.w > 0.0f);
#pragma unroll
    for (int pl = 0; pl < 5; ++pl)
        need = need || plane_dist(p0, pl) < 0.0f || plane_dist(p1, pl) < 0.0f || plane_dist(p2, pl) < 0.0f;
    return need ? 2 : 1;
}

// Sutherland-Hodgman against near + 4 guard planes, then project and snap.
static __device__ __noinline__ void setup_clipped(float4 p0, float4 p1, float4 p2, int W, int H, Poly& out) {
    float4 poly[DRP_MAX_POLY], tmp[DRP_MAX_POLY];
    int n = 3;
    poly[0] = p0;
    poly[1] = p1;
    poly[2] = p2;
    out.n = 0;
    for (int pl = 0; pl < 5 && n >= 3; ++pl) {
        int m = 0;
        for (int i = 0; i < n; ++i) {
            float4 p = poly[i];
            float4 q = poly[(i + 1) % n];
            float dp = plane_dist(p, pl), dq = plane_dist(q, pl);
            bool pin = dp >= 0.0f, qin = dq >= 0.0f;
            if (pin) tmp[m++] = p;
            if (pin != qin) {
                float t = dp / (dp - dq);
                float4 r;
                r.x = p.x + t * (q.x - p.x);
                r.y = p.y + t * (q.y - p.y);
                r.z = p.z + t * (q.z - p.z);
                r.w = p.w + t * (q.w - p.w);
                tmp[m++] = r;
            }
        }
        n = m;
        for (int i = 0; i < n; ++i) poly[i] = tmp[i];
    }
    if (n < 3) return;
    for (int i = 0; i < n; ++i)
        if (!(poly[i].w > 0.0f)) return;
    for (int i = 0; i < n; ++i) {
        out.X[i] = snap_coord(poly[i].x, poly[i].w, W);
        out.Y[i] = snap_coord(poly[i].y, poly[i].w, H);
        out.Z[i] = poly[i].z / poly[i].w;
    }
    out.n = n;
}

// Depth plane of a (fan) sub-triangle in fixed-point units, fan order.
struct Plane {
    float Z0, A, B;
};

__device__ __forceinline__ Plane depth_plane(int64_t X0, int64_t Y0, float Z0, int64_t X1, int64_t Y1, float Z1,
                                             int64_t X2, int64_t Y2, float Z2, int64_t area2) {
    float dx1 = (float)(X1 - X0), dy1 = (float)(Y1 - Y0);
    float dx2 = (float)(X2 - X0), dy2 = (float)(Y2 - Y0);
    float dz1 = Z1 - Z0, dz2 = Z2 - Z0;
    float det = (float)area2;
    Plane P;
    P.Z0 = Z0;
    P.A = (dz1 * dy2 - dy1 * dz2) / det;
    P.B = (dx1 * dz2 - dz1 * dx2) / det;
    return P;
}

__device__ __forceinline__ bool edge_inside(int64_t ax, int64_t ay, int64_t bx, int64_t by, int64_t cx, int64_t cy) {
    int64_t dx = bx - ax, dy = by - ay;
    int64_t e = dx * (cy - ay) - dy * (cx - ax);
    if (e > 0) return true;
    if (e < 0) return false;
    return (dy < 0) || (dy == 0 && dx < 0);
}

// ---------------------------------------------------------------------------
// Perspective-correct barycentrics (2D homogeneous), z/w and screen
// derivatives at a pixel centre.
// ---------------------------------------------------------------------------
struct Shade {
    float a[3], c[3], n[3], s;
    float u, v, nz, nw, zw;
    float Dx[3], Dy[3], Sx, Sy;
    float X, Y, kx, ky;
};

// NDC coordinate of the centre of pixel column / row `p` at resolution `res`.
__device__ __forceinline__ float pixel_ndc(int p, int res) { return (float)(2 * p + 1) / (float)res - 1.0f; }

__device__ __forceinline__ void shade_eval_xy(const float4& p0, const float4& p1, const float4& p2, float X, float Y,
                                              int W, int H, Shade& S);

__device__ __forceinline__ void shade_eval(const float4& p0, const float4& p1, const float4& p2, int px, int py,
                                           int W, int H, Shade& S) {
    shade_eval_xy(p0, p1, p2, pixel_ndc(px, W), pixel_ndc(py, H), W, H, S);
}

__device__ __forceinline__ void shade_eval_xy(const float4& p0, const float4& p1, const float4& p2, float X, float Y,
                                              int W, int H, Shade& S) {
    S.X = X;
    S.Y = Y;
    S.a[0] = p0.x - S.X * p0.w;
    S.a[1] = p1.x - S.X * p1.w;
    S.a[2] = p2.x - S.X * p2.w;
    S.c[0] = p0.y - S.Y * p0.w;
    S.c[1] = p1.y - S.Y * p1.w;
    S.c[2] = p2.y - S.Y * p2.w;
    const float* a = S.a;
    const float* c = S.c;
    S.n[0] = a[1] * c[2] - a[2] * c[1];
    S.n[1] = a[2] * c[0] - a[0] * c[2];
    S.n[2] = a[0] * c[1] - a[1] * c[0];
    S.s = (S.n[0] + S.n[1]) + S.n[2];
    S.u = S.n[0] / S.s;
    S.v = S.n[1] / S.s;
    S.nz = (S.n[0] * p0.z + S.n[1] * p1.z) + S.n[2] * p2.z;
    S.nw = (S.n[0] * p0.w + S.n[1] * p1.w) + S.n[2] * p2.w;
    S.zw = S.nz / S.nw;
    float w0 = p0.w, w1 = p1.w, w2 = p2.w;
    S.Dx[0] = c[1] * w2 - c[2] * w1;
    S.Dx[1] = c[2] * w0 - c[0] * w2;
    S.Dx[2] = c[0] * w1 - c[1] * w0;
    S.Dy[0] = w1 * a[2] - w2 * a[1];
    S.Dy[1] = w2 * a[0] - w0 * a[2];
    S.Dy[2] = w0 * a[1] - w1 * a[0];
    S.Sx = (S.Dx[0] + S.Dx[1]) + S.Dx[2];
    S.Sy = (S.Dy[0] + S.Dy[1]) + S.Dy[2];
    S.kx = 2.0f / (float)W;
    S.ky = 2.0f / (float)H;
}

__device__ __forceinline__ float4 shade_db(const Shade& S) {
    float4 d;
    d.x = ((S.Dx[0] - S.u * S.Sx) / S.s) * S.kx;
    d.y = ((S.Dy[0] - S.u * S.Sy) / S.s) * S.ky;
    d.z = ((S.Dx[1] - S.v * S.Sx) / S.s) * S.kx;
    d.w = ((S.Dy[1] - S.v * S.Sy) / S.s) * S.ky;
    return d;
}

__device__ __forceinline__ void cross3(const float* x, const float* y, float* o) {
    o[0] = fmaf(x[1], y[2], -x[2] * y[1]);
    o[1] = fmaf(x[2], y[0], -x[0] * y[2]);
    o[2] = fmaf(x[0], y[1], -x[1] * y[0]);
}

// dL/d(p_i) for L depending on (u, v, z/w) with gradient g and optionally on
// rast_db with gradient gdb.  out[i] receives the gradient of vertex i.
__device__ __forceinline__ void shade_grad(const float4& p0, const float4& p1, const float4& p2, const Shade& S,
                                           float gu, float gv, float gz, const float4* gdb, float4 out[3]) {
    float pz[3] = {p0.z, p1.z, p2.z};
    float wv[3] = {p0.w, p1.w, p2.w};
    float b[3] = {S.u, S.v, S.n[2] / S.s};
    float gb[3] = {gu, gv, 0.0f};
    float beta = fmaf(gb[0], b[0], gb[1] * b[1]);
    float inv_s = 1.0f / S.s, inv_nw = 1.0f / S.nw;
    float d = S.zw;
    float gn[3], gzc[3], gwd[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        gn[i] = (gb[i] - beta) * inv_s + gz * (pz[i] - d * wv[i]) * inv_nw;
        gzc[i] = gz * S.n[i] * inv_nw;
        gwd[i] = -gz * d * S.n[i] * inv_nw;
    }
    float qX[3] = {0.f, 0.f, 0.f}, qY[3] = {0.f, 0.f, 0.f};
    if (gdb) {
        float GX[3] = {gdb->x * S.kx, gdb->z * S.kx, 0.0f};
        float GY[3] = {gdb->y * S.ky, gdb->w * S.ky, 0.0f};
        float gamX = fmaf(GX[0], b[0], GX[1] * b[1]);
        float gamY = fmaf(GY[0], b[0], GY[1] * b[1]);
        float LX = (GX[0] * (S.Dx[0] - b[0] * S.Sx) + GX[1] * (S.Dx[1] - b[1] * S.Sx)) * inv_s;
        float LY = (GY[0] * (S.Dy[0] - b[0] * S.Sy) + GY[1] * (S.Dy[1] - b[1] * S.Sy)) * inv_s;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            qX[j] = (GX[j] - gamX) * inv_s;
            qY[j] = (GY[j] - gamY) * inv_s;
            gn[j] += -(S.Sx * inv_s) * qX[j] - LX * inv_s;
            gn[j] += -(S.Sy * inv_s) * qY[j] - LY * inv_s;
        }
    }
    float t1[3], t2[3], ga[3], gc[3], gw[3];
    cross3(S.c, gn, t1);
    cross3(qY, wv, t2);
#pragma unroll
    for (int i = 0; i < 3; ++i) ga[i] = t1[i] + t2[i];
    cross3(gn, S.a, t1);
    cross3(wv, qX, t2);
#pragma unroll
    for (int i = 0; i < 3; ++i) gc[i] = t1[i] + t2[i];
    cross3(qX, S.c, t1);
    cross3(S.a, qY, t2);
#pragma unroll
    for (int i = 0; i < 3; ++i) gw[i] = t1[i] + t2[i];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        out[i].x = ga[i];
        out[i].y = gc[i];
        out[i].z = gzc[i];
        out[i].w = -S.X * ga[i] - S.Y * gc[i] + gw[i] + gwd[i];
    }
}

// Gradient of (u, v) alone w.r.t. the three clip vertices at NDC (X, Y),
// for backward passes (no bit-exactness needed: reciprocals replace IEEE
// divisions).  out[i] receives dL/d p_i.
__device__ __forceinline__ void uv_grad_fast(const float4& p0, const float4& p1, const float4& p2, float X, float Y,
                                             float gu, float gv, float4 out[3]) {
    const float a[3] = {p0.x - X * p0.w, p1.x - X * p1.w, p2.x - X * p2.w};
    const float c[3] = {p0.y - Y * p0.w, p1.y - Y * p1.w, p2.y - Y * p2.w};
    const float n0 = fmaf(a[1], c[2], -a[2] * c[1]);
    const float n1 = fmaf(a[2], c[0], -a[0] * c[2]);
    const float n2 = fmaf(a[0], c[1], -a[1] * c[0]);
    const float inv_s = __frcp_rn((n0 + n1) + n2);
    const float beta = fmaf(gu, n0, gv * n1) * inv_s;  // sum gb_i b_i
    const float gn[3] = {(gu - beta) * inv_s, (gv - beta) * inv_s, -beta * inv_s};
    float ga[3], gc[3];
    cross3(c, gn, ga);
    cross3(gn, a, gc);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        out[i].x = ga[i];
        out[i].y = gc[i];
        out[i].z = 0.0f;
        out[i].w = -X * ga[i] - Y * gc[i];
    }
}

// ---------------------------------------------------------------------------
// Warp-level helpers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// Segmented warp reduction over runs of equal `key` in lane order.  seg_setup
// returns the last lane of this lane's run and whether the lane heads its run;
// seg_reduce leaves each run's total in its head lane.  Inactive lanes must
// pass a unique key (e.g. -1 - lane) and zero values.  All 32 lanes must call.
struct Seg {
    int run_end;
    bool head;
    int steps;  // shuffle steps needed by the longest run of the warp
};

__device__ __forceinline__ Seg seg_setup(long long key) {
    const unsigned FULL = 0xffffffffu;
    const int lane = lane_id();
    const long long prev = __shfl_up_sync(FULL, key, 1);
    Seg s;
    s.head = (lane == 0) || (prev != key);
    const unsigned heads = __ballot_sync(FULL, s.head);
    const unsigned after = (lane == 31) ? 0u : (heads & ~((2u << lane) - 1u));
    s.run_end = after ? (__ffs(after) - 2) : 31;
    const unsigned len = s.head ? (unsigned)(s.run_end - lane + 1) : 1u;
    const unsigned longest = __reduce_max_sync(FULL, len);
    s.steps = longest <= 1 ? 0 : 32 - __clz(longest - 1);  // ceil(log2(longest))
    return s;
}

template <int N>
__device__ __forceinline__ void seg_reduce(const Seg& s, float (&v)[N]) {
    const unsigned FULL = 0xffffffffu;
    const int lane = lane_id();
    for (int k = 0; k < s.steps; ++k) {  // warp-uniform trip count
        const int off = 1 << k;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            const float o = __shfl_down_sync(FULL, v[i], off);
            if (lane + off <= s.run_end) v[i] += o;
        }
    }
}

template <int N>
__device__ __forceinline__ bool segmented_sum(long long key, float (&v)[N]) {
    const Seg s = seg_setup(key);
    seg_reduce<N>(s, v);
    return s.head;
}

__device__ __forceinline__ void atomic_add4(float4* dst, const float4& v) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
    atomicAdd(dst, v);
#else
    atomicAdd(&dst->x, v.x);
    atomicAdd(&dst->y, v.y);
    atomicAdd(&dst->z, v.z);
    atomicAdd(&dst->w, v.w);
#endif
}

// s + x exactly as a float pair: s' = fl(s + x), err = (s + x) - s' (Knuth's
// TwoSum, no branch).  Sums of pairs carry their rounding errors in c.
__device__ __forceinline__ void two_sum(float& s, float& c, float x) {
    const float t = s + x;
    const float bp = t - s;
    const float err = (s - (t - bp)) + (x - bp);
    s = t;
    c += err;
}

// Threads of the block that forms a loss from its per-block partials.
constexpr int kFinalThreads = 256;

// *loss = scale * (sum of nblocks partials), by one whole block of NT
// threads: every thread adds its strided elements (eight loads in flight)
// in index order as a (sum, error) float pair, then the pairs are combined
// by a fixed shuffle tree within warps and across them -- a fixed order, so
// the loss is reproducible from run to run.  Float pairs instead of doubles:
// FP64 issues at a small fraction of the FP32 rate on this part, and this
// block sits on the step's critical path.  Every thread of the block calls
// it (it has a barrier).
template <int NT>
__device__ __forceinline__ void l1_final_block(const float* partial, long long nblocks, float scale, float* loss) {
    static_assert(NT % 32 == 0 && NT <= 1024, "l1_final_block: whole warps, at most 1024 threads");
    __shared__ float warp_s[NT / 32], warp_c[NT / 32];
    float s = 0.0f, c = 0.0f;
    for (long long i = threadIdx.x; i < nblocks; i += 8 * NT) {
        float v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = i + k * NT < nblocks ? partial[i + k * NT] : 0.0f;
#pragma unroll
        for (int k = 0; k < 8; ++k) two_sum(s, c, v[k]);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float os = __shfl_xor_sync(0xffffffffu, s, off), oc = __shfl_xor_sync(0xffffffffu, c, off);
        c += oc;
        two_sum(s, c, os);
    }
    if ((threadIdx.x & 31) == 0) {
        warp_s[threadIdx.x >> 5] = s;
        warp_c[threadIdx.x >> 5] = c;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const bool have = threadIdx.x < NT / 32;
        float v = have ? warp_s[threadIdx.x] : 0.0f, w = have ? warp_c[threadIdx.x] : 0.0f;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, v, off), ow = __shfl_xor_sync(0xffffffffu, w, off);
            w += ow;
            two_sum(v, w, ov);
        }
        if (threadIdx.x == 0) *loss = (v + w) * scale;
    }
}

}  // namespace drp
