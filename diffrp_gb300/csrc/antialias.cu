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
// Per-triangle setup (one thread per (view, triangle)): screen-space vertices,
// orientation and a 3-bit silhouette mask, so that a pixel pair needs one
// 32-byte record instead of a chain of index / vertex / neighbour gathers.
//   rec[0] = (s0.x, s0.y, s1.x, s1.y)
//   rec[1] = (s2.x, s2.y, sgn, mask bits)   sgn = 0: not usable (w <= 0 or
//            zero / NaN screen area).  mask bit k: edge k is a silhouette.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool project_vertex(const float4& p, int W, int H, float2& s) {
    if (!(p.w > 0.0f)) return false;
    s.x = (p.x / p.w + 1.0f) * ((float)W * 0.5f);
    s.y = (p.y / p.w + 1.0f) * ((float)H * 0.5f);
    return true;
}

__device__ __forceinline__ float edge_fn(const float2& a, const float2& b, const float2& p) {
    return (b.x - a.x) * (p.y - a.y) - (b.y - a.y) * (p.x - a.x);
}

__global__ void __launch_bounds__(256) aa_setup_kernel(AAArgs a) {
    const int b = blockIdx.y;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.num_triangles) return;
    float4* rec = reinterpret_cast<float4*>(a.tri_rec) + ((long long)b * a.num_triangles + t) * 2;
    const float4* P = reinterpret_cast<const float4*>(a.pos + (long long)b * a.pos_view_stride);
    const int v[3] = {a.tri[3 * t], a.tri[3 * t + 1], a.tri[3 * t + 2]};
    float2 s[3];
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (v[i] < 0 || v[i] >= a.num_vertices || !project_vertex(P[v[i]], a.W, a.H, s[i])) {
            ok = false;
            s[i] = make_float2(0.f, 0.f);
        }
    }
    float sgn = 0.0f;
    unsigned mask = 0;
    if (ok) {
        const float area = (s[1].x - s[0].x) * (s[2].y - s[0].y) - (s[1].y - s[0].y) * (s[2].x - s[0].x);
        if (!(area == 0.0f || area != area)) sgn = area > 0.0f ? 1.0f : -1.0f;
    }
    if (sgn != 0.0f) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            bool sil = true;
            const int N = a.nbr ? a.nbr[3 * t + k] : -1;
            if (N >= 0 && N < a.num_triangles) {
                const int ea = v[(k + 1) % 3], eb = v[(k + 2) % 3];
                int opp = -1;
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const int x = a.tri[3 * (long long)N + i];
                    if (x != ea && x != eb && x >= 0 && x < a.num_vertices) opp = x;
                }
                float2 so;
                if (opp >= 0 && project_vertex(P[opp], a.W, a.H, so)) {
                    const float2 qa = s[(k + 1) % 3], qb = s[(k + 2) % 3];
                    const float dT = edge_fn(qa, qb, s[k]);
                    const float dN = edge_fn(qa, qb, so);
                    if ((dT > 0.0f && dN < 0.0f) || (dT < 0.0f && dN > 0.0f)) sil = false;
                }
            }
            if (sil) mask |= 1u << k;
        }
    }
    rec[0] = make_float4(s[0].x, s[0].y, s[1].x, s[1].y);
    rec[1] = make_float4(s[2].x, s[2].y, sgn, __uint_as_float(mask));
}

// ---------------------------------------------------------------------------
// Pair evaluation.
// ---------------------------------------------------------------------------
struct AAPair {
    bool valid, clamped;
    int target, src;  // pixel indices within the view
    float w, sign, sgn, eF, eO;
    int T, k;
    float2 s[3];
    float2 cF, cO;
};

// rA, rB: rast rows of the two pixels; A is the left/lower pixel of the pair.
__device__ __forceinline__ void aa_pair(const AAArgs& a, const float4* rec, int A, int Bp, const float4& rA,
                                        const float4& rB, AAPair& R) {
    R.valid = false;
    const int tA = rast_tri(rA.w), tB = rast_tri(rB.w);
    const int cA = (tA >= 0 && tA < a.num_triangles) ? tA : -1;
    const int cB = (tB >= 0 && tB < a.num_triangles) ? tB : -1;
    if (cA == cB) return;
    int Fp;
    if (cA < 0) Fp = Bp;
    else if (cB < 0) Fp = A;
    else if (rA.z < rB.z) Fp = A;
    else if (rB.z < rA.z) Fp = Bp;
    else Fp = cA < cB ? A : Bp;
    const int Op = (Fp == A) ? Bp : A;
    const int T = (Fp == A) ? cA : cB;
    const float4 q0 = rec[2 * (long long)T], q1 = rec[2 * (long long)T + 1];
    const float sgn = q1.z;
    if (sgn == 0.0f) return;
    const unsigned mask = __float_as_uint(q1.w);
    R.s[0] = make_float2(q0.x, q0.y);
    R.s[1] = make_float2(q0.z, q0.w);
    R.s[2] = make_float2(q1.x, q1.y);
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
    if (best < 0 || !((mask >> best) & 1u)) return;
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

// Pair slot q of a pixel, in the fixed order left, right, below, above:
// (first pixel, second pixel) with the first being the left / lower one.
__device__ __forceinline__ bool pair_slot(int q, int pix, int px, int py, int W, int H, int& A, int& B) {
    switch (q) {
    case 0: A = pix - 1; B = pix; return px > 0;
    case 1: A = pix; B = pix + 1; return px < W - 1;
    case 2: A = pix - W; B = pix; return py > 0;
    default: A = pix; B = pix + W; return py < H - 1;
    }
}

__global__ void __launch_bounds__(256) aa_fwd_kernel(AAArgs a) {
    const int b = blockIdx.y;
    const int npix = a.H * a.W;
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    const int py = pix / a.W, px = pix - py * a.W;
    const int C = a.C;
    const float4* R = reinterpret_cast<const float4*>(a.rast) + (long long)b * npix;
    const float* Cc = a.color + (long long)b * npix * C;
    const float4* rec = reinterpret_cast<const float4*>(a.tri_rec) + (long long)b * a.num_triangles * 2;
    float* o = a.out + ((long long)b * npix + pix) * C;
    const float* cs = Cc + (long long)pix * C;
    const float4 rs = R[pix];
    // Blends that land on this pixel, per pair slot: source pixel and weight.
    int src[4];
    float wt[4];
    bool any = false;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        src[q] = -1;
        wt[q] = 0.f;
        int A, B;
        if (!pair_slot(q, pix, px, py, a.W, a.H, A, B)) continue;
        const int other = A == pix ? B : A;
        const float4 ro = R[other];
        if (ro.w == rs.w) continue;
        AAPair pr;
        aa_pair(a, rec, A, B, A == pix ? rs : ro, A == pix ? ro : rs, pr);
        if (pr.valid && pr.target == pix) {
            src[q] = pr.src;
            wt[q] = pr.w;
            any = true;
        }
    }
    if (!any) {
        if ((C & 3) == 0 && (((uintptr_t)cs | (uintptr_t)o) & 15) == 0) {
            for (int c = 0; c < C; c += 4)
                *reinterpret_cast<float4*>(o + c) = *reinterpret_cast<const float4*>(cs + c);
        } else {
            for (int c = 0; c < C; ++c) o[c] = cs[c];
        }
        return;
    }
    for (int c = 0; c < C; ++c) {
        float v = cs[c];
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (src[q] >= 0) v = fmaf(wt[q], Cc[(long long)src[q] * C + c] - cs[c], v);
        o[c] = v;
    }
}

__global__ void __launch_bounds__(256) aa_bwd_kernel(AAArgs a) {
    const int b = blockIdx.y;
    const int npix = a.H * a.W;
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    const int py = pix / a.W, px = pix - py * a.W;
    const int C = a.C;
    const float4* R = reinterpret_cast<const float4*>(a.rast) + (long long)b * npix;
    const float* Cc = a.color + (long long)b * npix * C;
    const float* Gd = a.grad_out + (long long)b * npix * C;
    const float4* P = reinterpret_cast<const float4*>(a.pos + (long long)b * a.pos_view_stride);
    float4* GP = a.grad_pos ? reinterpret_cast<float4*>(a.grad_pos + (long long)b * a.pos_view_stride) : nullptr;
    const float4* rec = reinterpret_cast<const float4*>(a.tri_rec) + (long long)b * a.num_triangles * 2;
    float* gc = a.grad_color + ((long long)b * npix + pix) * C;
    const float* gs = Gd + (long long)pix * C;
    const float4 rs = R[pix];
    // Colour-gradient terms per pair slot: role (0 none, 1 this pixel is the
    // blend target: scale own gradient, 2 the source: gather the target's
    // gradient), the target pixel and the weight.
    int role[4], tgt[4];
    float wt[4];
    bool any = false;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        role[q] = 0;
        tgt[q] = 0;
        wt[q] = 0.f;
        int A, B;
        if (!pair_slot(q, pix, px, py, a.W, a.H, A, B)) continue;
        const int other = A == pix ? B : A;
        const float4 ro = R[other];
        if (ro.w == rs.w) continue;
        AAPair p;
        aa_pair(a, rec, A, B, A == pix ? rs : ro, A == pix ? ro : rs, p);
        if (!p.valid) continue;
        role[q] = p.target == pix ? 1 : 2;
        tgt[q] = p.target;
        wt[q] = p.w;
        any = true;
        if (!GP || A != pix || p.clamped) continue;
        // Edge-position gradient, once per pair (owned by its first pixel).
        float dLdw = 0.f;
        for (int c = 0; c < C; ++c)
            dLdw = fmaf(Gd[(long long)p.target * C + c], Cc[(long long)p.src * C + c] - Cc[(long long)p.target * C + c],
                        dLdw);
        const float dLdt = dLdw * p.sign * a.boost;
        const float den = p.eF - p.eO;
        const float inv2 = 1.0f / (den * den);
        const float dtF = -p.eO * inv2, dtO = p.eF * inv2;
        const float2 ea = p.s[(p.k + 1) % 3], eb = p.s[(p.k + 2) % 3];
        const float fF = dLdt * dtF * p.sgn, fO = dLdt * dtO * p.sgn;
        const float gA0 = fmaf(fF, eb.y - p.cF.y, fO * (eb.y - p.cO.y));
        const float gA1 = fmaf(fF, p.cF.x - eb.x, fO * (p.cO.x - eb.x));
        const float gB0 = fmaf(fF, p.cF.y - ea.y, fO * (p.cO.y - ea.y));
        const float gB1 = fmaf(fF, ea.x - p.cF.x, fO * (ea.x - p.cO.x));
        const int vA = a.tri[3 * (long long)p.T + (p.k + 1) % 3], vB = a.tri[3 * (long long)p.T + (p.k + 2) % 3];
        const float hx = 0.5f * (float)a.W, hy = 0.5f * (float)a.H;
        const float4 pA = P[vA], pB = P[vB];
        const float iwA = 1.0f / pA.w, iwB = 1.0f / pB.w;
        atomic_add4(GP + vA, make_float4(gA0 * hx * iwA, gA1 * hy * iwA, 0.f,
                                         -(gA0 * hx * pA.x + gA1 * hy * pA.y) * iwA * iwA));
        atomic_add4(GP + vB, make_float4(gB0 * hx * iwB, gB1 * hy * iwB, 0.f,
                                         -(gB0 * hx * pB.x + gB1 * hy * pB.y) * iwB * iwB));
    }
    if (!any) {
        if ((C & 3) == 0 && (((uintptr_t)gs | (uintptr_t)gc) & 15) == 0) {
            for (int c = 0; c < C; c += 4)
                *reinterpret_cast<float4*>(gc + c) = *reinterpret_cast<const float4*>(gs + c);
        } else {
            for (int c = 0; c < C; ++c) gc[c] = gs[c];
        }
        return;
    }
    for (int c = 0; c < C; ++c) {
        float v = gs[c];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (role[q] == 1) v = fmaf(-wt[q], gs[c], v);
            else if (role[q] == 2) v = fmaf(wt[q], Gd[(long long)tgt[q] * C + c], v);
        }
        gc[c] = v;
    }
}

size_t aa_ws_bytes(int B, long long F) { return (size_t)B * (size_t)F * 32 + 256; }

static void launch_aa_setup(const AAArgs& a, cudaStream_t s) {
    if (a.num_triangles <= 0) return;
    dim3 grid((unsigned)((a.num_triangles + 255) / 256), (unsigned)a.B);
    aa_setup_kernel<<<grid, 256, 0, s>>>(a);
}

int launch_aa_fwd(const AAArgs& a, cudaStream_t s) {
    const int npix = a.H * a.W;
    if (npix == 0) return 0;
    launch_aa_setup(a, s);
    dim3 grid((unsigned)((npix + 255) / 256), (unsigned)a.B);
    aa_fwd_kernel<<<grid, 256, 0, s>>>(a);
    return 0;
}

int launch_aa_bwd(const AAArgs& a, cudaStream_t s) {
    const int npix = a.H * a.W;
    if (npix == 0) return 0;
    launch_aa_setup(a, s);
    dim3 grid((unsigned)((npix + 255) / 256), (unsigned)a.B);
    aa_bwd_kernel<<<grid, 256, 0, s>>>(a);
    return 0;
}

}  // namespace drp
