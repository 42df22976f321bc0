// antialias.cu -- edge topology and analytic silhouette antialiasing
// (forward and backward).  Replaces dr.antialias and
// dr.antialias_construct_topology_hash as called at
// diffrp/rendering/surface_deferred.py:775.
//
// For each 4-neighbour pixel pair (A, B) with different triangle ids the
// front surface F (nearer z/w, or the only non-background pixel) is found; the
// segment between the two pixel centres leaves F's triangle through edge k at
// parameter t.  If edge k is a silhouette (no neighbour triangle across it, or
// the neighbour folds onto the same side in screen space) the colour of the
// pixel whose square the edge crosses is blended toward the other pixel with
// weight |t - 1/2|.  Every pixel gathers the pairs it belongs to, so the
// forward needs no atomics and is deterministic; the backward gathers colour
// gradients the same way and scatters edge-vertex gradients with float4
// atomics, one pair per owner pixel.
#include "drp_common.cuh"
#include "drp_internal.h"

namespace drp {

// ---------------------------------------------------------------------------
// Topology: open-addressing hash of undirected edges -> the (at most two)
// triangle edges that use it.  nbr[3t + k] = triangle across edge k (the edge
// between vertices k+1 and k+2) when exactly two distinct triangles share it.
// ---------------------------------------------------------------------------
static inline unsigned long long topo_capacity(long long F) {
    unsigned long long need = (unsigned long long)max(1ll, 6 * F);
    unsigned long long cap = 1024;
    while (cap < need) cap <<= 1;
    return cap;
}

size_t topology_ws_bytes(long long F) {
    const unsigned long long cap = topo_capacity(F);
    return cap * (sizeof(unsigned long long) + sizeof(unsigned) + 2 * sizeof(int)) + 256;
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

__device__ __forceinline__ bool edge_key(const int* tri, long long t, int k, unsigned long long& key) {
    const unsigned a = (unsigned)tri[3 * t + (k + 1) % 3], b = (unsigned)tri[3 * t + (k + 2) % 3];
    if (a == b) return false;
    const unsigned lo = min(a, b), hi = max(a, b);
    key = ((unsigned long long)lo << 32) | hi;
    return true;
}

__global__ void topo_insert_kernel(const int* tri, long long F, unsigned long long* keys, unsigned* cnt, int* slots,
                                   unsigned long long mask) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 3 * F) return;
    const long long t = e / 3;
    const int k = (int)(e % 3);
    unsigned long long key;
    if (!edge_key(tri, t, k, key)) return;
    unsigned long long h = mix64(key) & mask;
    for (unsigned long long probe = 0; probe <= mask; ++probe) {
        const unsigned long long prev = atomicCAS(keys + h, ~0ull, key);
        if (prev == ~0ull || prev == key) {
            const unsigned idx = atomicAdd(cnt + h, 1u);
            if (idx < 2) slots[2 * h + idx] = (int)e;
            return;
        }
        h = (h + 1) & mask;
    }
}

__global__ void topo_resolve_kernel(const int* tri, long long F, const unsigned long long* keys, const unsigned* cnt,
                                    const int* slots, unsigned long long mask, int* nbr) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 3 * F) return;
    const long long t = e / 3;
    const int k = (int)(e % 3);
    int out = -1;
    unsigned long long key;
    if (edge_key(tri, t, k, key)) {
        unsigned long long h = mix64(key) & mask;
        for (unsigned long long probe = 0; probe <= mask; ++probe) {
            const unsigned long long kk = keys[h];
            if (kk == key) {
                if (cnt[h] == 2) {
                    const int s0 = slots[2 * h], s1 = slots[2 * h + 1];
                    const int other = (s0 == (int)e) ? s1 : s0;
                    if (other / 3 != (int)t) out = other / 3;
                }
                break;
            }
            if (kk == ~0ull) break;
            h = (h + 1) & mask;
        }
    }
    nbr[e] = out;
}

int launch_topology(const int* tri, long long F, void* ws, size_t ws_bytes, int* nbr, cudaStream_t s) {
    if (F <= 0) return 0;
    const unsigned long long cap = topo_capacity(F);
    if (ws_bytes < topology_ws_bytes(F)) return 1;
    char* p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    unsigned long long* keys = reinterpret_cast<unsigned long long*>(p);
    unsigned* cnt = reinterpret_cast<unsigned*>(keys + cap);
    int* slots = reinterpret_cast<int*>(cnt + cap);
    cudaMemsetAsync(keys, 0xff, cap * sizeof(unsigned long long), s);
    cudaMemsetAsync(cnt, 0, cap * sizeof(unsigned), s);
    const long long n = 3 * F;
    topo_insert_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(tri, F, keys, cnt, slots, cap - 1);
    topo_resolve_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(tri, F, keys, cnt, slots, cap - 1, nbr);
    return 0;
}

// ---------------------------------------------------------------------------
// Pair evaluation.
// ---------------------------------------------------------------------------
struct AAPair {
    bool valid, clamped;
    long long target, src;  // pixel indices within the view
    float w, sign, sgn, eF, eO;
    int T, k;
    float2 s[3];
    float2 cF, cO;
};

__device__ __forceinline__ bool project_vertex(const float4& p, int W, int H, float2& s) {
    if (!(p.w > 0.0f)) return false;
    s.x = (p.x / p.w + 1.0f) * ((float)W * 0.5f);
    s.y = (p.y / p.w + 1.0f) * ((float)H * 0.5f);
    return true;
}

__device__ __forceinline__ float edge_fn(const float2& a, const float2& b, const float2& p) {
    return (b.x - a.x) * (p.y - a.y) - (b.y - a.y) * (p.x - a.x);
}

// rA, rB: rast rows of the two pixels; A is the left/lower pixel of the pair.
__device__ __forceinline__ void aa_pair(const AAArgs& a, const float4* P, long long A, long long Bp, const float4& rA,
                                        const float4& rB, AAPair& R) {
    R.valid = false;
    int d0, d1, d2;
    const int tA = checked_tri(rA.w, a.tri, a.num_triangles, a.num_vertices, d0, d1, d2);
    const int tB = checked_tri(rB.w, a.tri, a.num_triangles, a.num_vertices, d0, d1, d2);
    if (tA == tB) return;
    long long Fp;
    if (tA < 0) Fp = Bp;
    else if (tB < 0) Fp = A;
    else if (rA.z < rB.z) Fp = A;
    else if (rB.z < rA.z) Fp = Bp;
    else Fp = tA < tB ? A : Bp;
    const long long Op = (Fp == A) ? Bp : A;
    const int T = (Fp == A) ? tA : tB;
    const int v0 = a.tri[3 * (long long)T], v1 = a.tri[3 * (long long)T + 1], v2 = a.tri[3 * (long long)T + 2];
    if (!project_vertex(P[v0], a.W, a.H, R.s[0])) return;
    if (!project_vertex(P[v1], a.W, a.H, R.s[1])) return;
    if (!project_vertex(P[v2], a.W, a.H, R.s[2])) return;
    const float area = (R.s[1].x - R.s[0].x) * (R.s[2].y - R.s[0].y) - (R.s[1].y - R.s[0].y) * (R.s[2].x - R.s[0].x);
    if (area == 0.0f || area != area) return;
    const float sgn = area > 0.0f ? 1.0f : -1.0f;
    R.cF = make_float2((float)(Fp % a.W) + 0.5f, (float)(Fp / a.W) + 0.5f);
    R.cO = make_float2((float)(Op % a.W) + 0.5f, (float)(Op / a.W) + 0.5f);
    int best = -1;
    float bt = 0.f, beF = 0.f, beO = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float2 ea = R.s[(k + 1) % 3], eb = R.s[(k + 2) % 3];
        const float eO = sgn * edge_fn(ea, eb, R.cO);
        if (!(eO < 0.0f)) continue;
        const float eF = sgn * edge_fn(ea, eb, R.cF);
        const float t = eF / (eF - eO);
        if (best < 0 || t < bt) {
            best = k;
            bt = t;
            beF = eF;
            beO = eO;
        }
    }
    if (best < 0) return;
    const int N = a.nbr ? a.nbr[3 * (long long)T + best] : -1;
    if (N >= 0 && N < a.num_triangles) {
        const int ea = a.tri[3 * (long long)T + (best + 1) % 3], eb = a.tri[3 * (long long)T + (best + 2) % 3];
        int opp = -1;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int x = a.tri[3 * (long long)N + i];
            if (x != ea && x != eb && x >= 0 && x < a.num_vertices) opp = x;
        }
        float2 so;
        if (opp >= 0 && project_vertex(P[opp], a.W, a.H, so)) {
            const float2 qa = R.s[(best + 1) % 3], qb = R.s[(best + 2) % 3];
            const float dT = edge_fn(qa, qb, R.s[best]);
            const float dN = edge_fn(qa, qb, so);
            if ((dT > 0.0f && dN < 0.0f) || (dT < 0.0f && dN > 0.0f)) return;
        }
    }
    R.clamped = false;
    if (bt < 0.0f) { bt = 0.0f; R.clamped = true; }
    if (bt > 1.0f) { bt = 1.0f; R.clamped = true; }
    R.T = T;
    R.k = best;
    R.eF = beF;
    R.eO = beO;
    R.sgn = sgn;
    if (bt > 0.5f) {
        R.target = Op;
        R.src = Fp;
        R.w = bt - 0.5f;
        R.sign = 1.0f;
    } else {
        R.target = Fp;
        R.src = Op;
        R.w = 0.5f - bt;
        R.sign = -1.0f;
    }
    R.valid = true;
}

__device__ __forceinline__ int pixel_pairs(long long pix, int px, int py, int W, int H, long long (&pairs)[4][2]) {
    int np = 0;
    if (px > 0) { pairs[np][0] = pix - 1; pairs[np][1] = pix; ++np; }
    if (px < W - 1) { pairs[np][0] = pix; pairs[np][1] = pix + 1; ++np; }
    if (py > 0) { pairs[np][0] = pix - W; pairs[np][1] = pix; ++np; }
    if (py < H - 1) { pairs[np][0] = pix; pairs[np][1] = pix + W; ++np; }
    return np;
}

__global__ void __launch_bounds__(256) aa_fwd_kernel(AAArgs a) {
    const long long npix = (long long)a.H * a.W;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)a.B * npix) return;
    const int b = (int)(i / npix);
    const long long pix = i - (long long)b * npix;
    const int py = (int)(pix / a.W), px = (int)(pix % a.W);
    const float4* R = reinterpret_cast<const float4*>(a.rast) + (long long)b * npix;
    const float* Cc = a.color + (long long)b * npix * a.C;
    const float4* P = reinterpret_cast<const float4*>(a.pos + (long long)b * a.pos_view_stride);
    float* o = a.out + i * a.C;
    const int C = a.C;
    for (int c = 0; c < C; ++c) o[c] = Cc[pix * C + c];
    const float4 rs = R[pix];
    long long pairs[4][2];
    const int np = pixel_pairs(pix, px, py, a.W, a.H, pairs);
    for (int q = 0; q < np; ++q) {
        const long long other = pairs[q][0] == pix ? pairs[q][1] : pairs[q][0];
        const float4 ro = R[other];
        if (ro.w == rs.w) continue;
        const float4& rA = pairs[q][0] == pix ? rs : ro;
        const float4& rB = pairs[q][0] == pix ? ro : rs;
        AAPair pr;
        aa_pair(a, P, pairs[q][0], pairs[q][1], rA, rB, pr);
        if (!pr.valid || pr.target != pix) continue;
        for (int c = 0; c < C; ++c) o[c] = fmaf(pr.w, Cc[pr.src * C + c] - Cc[pix * C + c], o[c]);
    }
}

__global__ void __launch_bounds__(256) aa_bwd_kernel(AAArgs a) {
    const long long npix = (long long)a.H * a.W;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)a.B * npix) return;
    const int b = (int)(i / npix);
    const long long pix = i - (long long)b * npix;
    const int py = (int)(pix / a.W), px = (int)(pix % a.W);
    const float4* R = reinterpret_cast<const float4*>(a.rast) + (long long)b * npix;
    const float* Cc = a.color + (long long)b * npix * a.C;
    const float* Gd = a.grad_out + (long long)b * npix * a.C;
    const float4* P = reinterpret_cast<const float4*>(a.pos + (long long)b * a.pos_view_stride);
    float4* GP = reinterpret_cast<float4*>(a.grad_pos + (long long)b * a.pos_view_stride);
    const int C = a.C;
    float* gc = a.grad_color + i * C;
    for (int c = 0; c < C; ++c) gc[c] = Gd[pix * C + c];
    const float4 rs = R[pix];
    long long pairs[4][2];
    const int np = pixel_pairs(pix, px, py, a.W, a.H, pairs);
    for (int q = 0; q < np; ++q) {
        const long long other = pairs[q][0] == pix ? pairs[q][1] : pairs[q][0];
        const float4 ro = R[other];
        if (ro.w == rs.w) continue;
        const float4& rA = pairs[q][0] == pix ? rs : ro;
        const float4& rB = pairs[q][0] == pix ? ro : rs;
        AAPair pr;
        aa_pair(a, P, pairs[q][0], pairs[q][1], rA, rB, pr);
        if (!pr.valid) continue;
        if (pr.target == pix)
            for (int c = 0; c < C; ++c) gc[c] = fmaf(-pr.w, Gd[pix * C + c], gc[c]);
        if (pr.src == pix)
            for (int c = 0; c < C; ++c) gc[c] = fmaf(pr.w, Gd[pr.target * C + c], gc[c]);
        if (pairs[q][0] != pix || pr.clamped || !a.grad_pos) continue;
        float dLdw = 0.f;
        for (int c = 0; c < C; ++c) dLdw = fmaf(Gd[pr.target * C + c], Cc[pr.src * C + c] - Cc[pr.target * C + c], dLdw);
        const float dLdt = dLdw * pr.sign * a.boost;
        const float den = pr.eF - pr.eO;
        const float inv2 = 1.0f / (den * den);
        const float dts[2] = {-pr.eO * inv2, pr.eF * inv2};
        const float2 ea = pr.s[(pr.k + 1) % 3], eb = pr.s[(pr.k + 2) % 3];
        const float2 cs[2] = {pr.cF, pr.cO};
        float gA0 = 0.f, gA1 = 0.f, gB0 = 0.f, gB1 = 0.f;
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            const float f = dLdt * dts[m] * pr.sgn;
            gA0 = fmaf(f, eb.y - cs[m].y, gA0);
            gA1 = fmaf(f, cs[m].x - eb.x, gA1);
            gB0 = fmaf(f, cs[m].y - ea.y, gB0);
            gB1 = fmaf(f, ea.x - cs[m].x, gB1);
        }
        const int vA = a.tri[3 * (long long)pr.T + (pr.k + 1) % 3], vB = a.tri[3 * (long long)pr.T + (pr.k + 2) % 3];
        const float hx = 0.5f * (float)a.W, hy = 0.5f * (float)a.H;
        const float4 pA = P[vA], pB = P[vB];
        const float iwA = 1.0f / pA.w, iwB = 1.0f / pB.w;
        atomic_add4(GP + vA, make_float4(gA0 * hx * iwA, gA1 * hy * iwA, 0.f,
                                         -(gA0 * hx * pA.x + gA1 * hy * pA.y) * iwA * iwA));
        atomic_add4(GP + vB, make_float4(gB0 * hx * iwB, gB1 * hy * iwB, 0.f,
                                         -(gB0 * hx * pB.x + gB1 * hy * pB.y) * iwB * iwB));
    }
}

int launch_aa_fwd(const AAArgs& a, cudaStream_t s) {
    const long long n = (long long)a.B * a.H * a.W;
    if (n == 0) return 0;
    aa_fwd_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    return 0;
}

int launch_aa_bwd(const AAArgs& a, cudaStream_t s) {
    const long long n = (long long)a.B * a.H * a.W;
    if (n == 0) return 0;
    aa_bwd_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    return 0;
}

}  // namespace drp
