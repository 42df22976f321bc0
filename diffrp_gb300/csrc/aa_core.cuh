// aa_core.cuh -- analytic silhouette antialiasing building blocks shared by
// the plain antialias kernels (antialias.cu) and the batched pipeline
// (batch.cu): the per-triangle screen-space record, the evaluation of one
// 4-neighbour pixel pair, and the per-pixel forward / backward.
#pragma once
#include "drp_common.cuh"

namespace drp {

__device__ __forceinline__ bool project_vertex(const float4& p, int W, int H, float2& s) {
    if (!(p.w > 0.0f)) return false;
    s.x = (p.x / p.w + 1.0f) * ((float)W * 0.5f);
    s.y = (p.y / p.w + 1.0f) * ((float)H * 0.5f);
    return true;
}

__device__ __forceinline__ float edge_fn(const float2& a, const float2& b, const float2& p) {
    return (b.x - a.x) * (p.y - a.y) - (b.y - a.y) * (p.x - a.x);
}

// Per-triangle record: rec[0] = (s0.x, s0.y, s1.x, s1.y), rec[1] = (s2.x,
// s2.y, sgn, mask bits); sgn = 0 marks an unusable triangle (a vertex with
// w <= 0, zero / NaN screen area); mask bit k: edge k (vertices k+1, k+2) is
// a silhouette (no neighbour across it, or the neighbour's opposite vertex
// projects to the same side of the edge as this triangle's).  opp: the
// topology table (opposite vertex across each edge, -1 for none) or null.
__device__ __forceinline__ void aa_tri_record(const float4* P, const int* tri, const int* opp_tab, long long t,
                                              long long F, long long V, int W, int H, float4* rec) {
    const int v[3] = {tri[3 * t], tri[3 * t + 1], tri[3 * t + 2]};
    float2 s[3];
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (v[i] < 0 || v[i] >= V || !project_vertex(P[v[i]], W, H, s[i])) {
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
            const int opp = opp_tab ? opp_tab[3 * t + k] : -1;
            if (opp >= 0 && opp < V) {
                float2 so;
                if (project_vertex(P[opp], W, H, so)) {
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

struct AAPair {
    bool valid, clamped;
    int target, src;  // pixel indices within the view
    float w, sign, sgn, eF, eO;
    int T, k;
    float2 s[3];
    float2 cF, cO;
};

// Pair (A, B) with A the left / lower pixel at column ax, row ay and B its
// right (vertical = false) or upper (vertical = true) neighbour; rA, rB their
// rast rows; rec the view's triangle records (F triangles).
__device__ __forceinline__ void aa_pair(const float4* rec, long long F, int A, int Bp, int ax, int ay, bool vertical,
                                        const float4& rA, const float4& rB, AAPair& R) {
    R.valid = false;
    const int tA = rast_tri(rA.w), tB = rast_tri(rB.w);
    const int cA = (tA >= 0 && tA < F) ? tA : -1;
    const int cB = (tB >= 0 && tB < F) ? tB : -1;
    if (cA == cB) return;
    int Fp;
    if (cA < 0) Fp = Bp;
    else if (cB < 0) Fp = A;
    else if (rA.z < rB.z) Fp = A;
    else if (rB.z < rA.z) Fp = Bp;
    else Fp = cA < cB ? A : Bp;
    const int Op = (Fp == A) ? Bp : A;
    const int T = (Fp == A) ? cA : cB;
    const float4 q1 = rec[2 * (long long)T + 1];
    const float sgn = q1.z;
    const unsigned mask = __float_as_uint(q1.w);
    // A triangle without a silhouette edge never blends: its exit edge, if
    // any, fails the mask test below.  Inside a closed mesh that is almost
    // every pair, so stop before the edge functions.
    if (sgn == 0.0f || mask == 0u) return;
    const float4 q0 = rec[2 * (long long)T];
    R.s[0] = make_float2(q0.x, q0.y);
    R.s[1] = make_float2(q0.z, q0.w);
    R.s[2] = make_float2(q1.x, q1.y);
    const float2 ctrA = make_float2((float)ax + 0.5f, (float)ay + 0.5f);
    const float2 ctrB = vertical ? make_float2(ctrA.x, (float)(ay + 1) + 0.5f)
                                 : make_float2((float)(ax + 1) + 0.5f, ctrA.y);
    R.cF = Fp == A ? ctrA : ctrB;
    R.cO = Fp == A ? ctrB : ctrA;
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
// (first pixel, second pixel) with the first being the left / lower one, at
// column ax, row ay; vertical for the below / above pairs.
__device__ __forceinline__ bool pair_slot(int q, int pix, int px, int py, int W, int H, int& A, int& B, int& ax,
                                          int& ay, bool& vertical) {
    switch (q) {
    case 0: A = pix - 1; B = pix; ax = px - 1; ay = py; vertical = false; return px > 0;
    case 1: A = pix; B = pix + 1; ax = px; ay = py; vertical = false; return px < W - 1;
    case 2: A = pix - W; B = pix; ax = px; ay = py - 1; vertical = true; return py > 0;
    default: A = pix; B = pix + W; ax = px; ay = py; vertical = true; return py < H - 1;
    }
}

// Copy C floats (128-bit groups when C % 4 == 0 and both ends are 16-byte
// aligned); up to four groups are loaded before the first store.
__device__ __forceinline__ void copy_channels(const float* src, float* dst, int C) {
    if ((C & 3) == 0 && (((uintptr_t)src | (uintptr_t)dst) & 15) == 0) {
        const float4* s4 = reinterpret_cast<const float4*>(src);
        float4* d4 = reinterpret_cast<float4*>(dst);
        const int G = C >> 2;
        for (int g0 = 0; g0 < G; g0 += 4) {
            float4 v[4];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (g0 + k < G) v[k] = s4[g0 + k];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (g0 + k < G) d4[g0 + k] = v[k];
        }
    } else {
        for (int c = 0; c < C; ++c) dst[c] = src[c];
    }
}

// Blend terms of one pixel: for each pair slot (left, right, below, above)
// whose pair blends into this pixel, the source pixel and its weight.  The
// pixel's and its four neighbours' rast rows are loaded together, before any
// of them is used.  Returns whether any slot blends.  pair_bits (may be null)
// gets bit q set when slot q's pair blends in either direction -- the pixels
// the antialias backward has to visit.
__device__ __forceinline__ bool aa_fwd_terms(const float4* R, const float4* rec, long long F, int W, int H, int pix,
                                             int (&src)[4], float (&wt)[4], unsigned* pair_bits = nullptr) {
    const int py = pix / W, px = pix - py * W;
    int A[4], B[4], ax[4], ay[4];
    bool vert[4], has[4];
    float4 rn[4];
    const float4 rs = R[pix];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        has[q] = pair_slot(q, pix, px, py, W, H, A[q], B[q], ax[q], ay[q], vert[q]);
        if (has[q]) rn[q] = R[A[q] == pix ? B[q] : A[q]];
    }
    bool any = false;
    unsigned bits = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        src[q] = -1;
        wt[q] = 0.f;
        if (!has[q] || rn[q].w == rs.w) continue;
        AAPair pr;
        const bool first = A[q] == pix;
        aa_pair(rec, F, A[q], B[q], ax[q], ay[q], vert[q], first ? rs : rn[q], first ? rn[q] : rs, pr);
        if (pr.valid) bits |= 1u << q;
        if (pr.valid && pr.target == pix) {
            src[q] = pr.src;
            wt[q] = pr.w;
            any = true;
        }
    }
    if (pair_bits) *pair_bits = bits;
    return any;
}

// aa_fwd_terms for a warp of consecutive pixels of one image (lane l + 1
// holds pixel pix + 1; lanes past the image pass in = false).  A pixel's
// left pair is its left lane's right pair -- the same pair, evaluated from
// the same inputs -- so it is taken from that lane by shuffle instead of
// being evaluated a second time (lane 0 and pixels of column 0 evaluate
// theirs).  The terms are identical to aa_fwd_terms'.  All 32 lanes call.
__device__ __forceinline__ bool aa_fwd_terms_row(const float4* R, const float4* rec, long long F, int W, int H,
                                                 int pix, bool in, int (&src)[4], float (&wt)[4],
                                                 unsigned* pair_bits = nullptr) {
    const int lane = threadIdx.x & 31;
    const int py = pix / W, px = pix - py * W;
    const bool share = lane > 0 && px > 0;  // the left lane holds pixel pix - 1 of this row
    int A[4], B[4], ax[4], ay[4];
    bool vert[4], has[4];
    float4 rn[4];
    float4 rs = make_float4(0.f, 0.f, 0.f, 0.f);
    if (in) rs = R[pix];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        has[q] = in && pair_slot(q, pix, px, py, W, H, A[q], B[q], ax[q], ay[q], vert[q]) && !(q == 0 && share);
        if (has[q]) rn[q] = R[A[q] == pix ? B[q] : A[q]];
    }
    bool any = false;
    unsigned bits = 0;
    int right = 0;  // the right pair's target: 1 this pixel, 2 its right neighbour (0: no pair)
    float right_w = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        src[q] = -1;
        wt[q] = 0.f;
        if (!has[q] || rn[q].w == rs.w) continue;
        AAPair pr;
        const bool first = A[q] == pix;
        aa_pair(rec, F, A[q], B[q], ax[q], ay[q], vert[q], first ? rs : rn[q], first ? rn[q] : rs, pr);
        if (pr.valid) bits |= 1u << q;
        if (pr.valid && pr.target == pix) {
            src[q] = pr.src;
            wt[q] = pr.w;
            any = true;
        }
        if (q == 1 && pr.valid) {
            right = pr.target == pix ? 1 : 2;
            right_w = pr.w;
        }
    }
    const int left = __shfl_up_sync(0xffffffffu, right, 1);
    const float left_w = __shfl_up_sync(0xffffffffu, right_w, 1);
    if (in && share && left != 0) {
        bits |= 1u;
        if (left == 2) {  // this pixel is the pair's target, its left neighbour the source
            src[0] = pix - 1;
            wt[0] = left_w;
            any = true;
        }
    }
    if (pair_bits) *pair_bits = bits;
    return any;
}

// Forward of one pixel: out = c + sum over pair slots targeting this pixel of
// w (c[src] - c), in slot order (fmaf).  R, Cc: the view's rast and colour.
// COPY = false: o already holds c (the caller wrote it), so pixels without a
// blend are left untouched.  pair_bits: as aa_fwd_terms.
template <bool COPY>
__device__ __forceinline__ void aa_fwd_pixel(const float4* R, const float* Cc, const float4* rec, long long F, int W,
                                             int H, int C, int pix, float* o, unsigned* pair_bits = nullptr) {
    const float* cs = Cc + (long long)pix * C;
    int src[4];
    float wt[4];
    const bool any = aa_fwd_terms(R, rec, F, W, H, pix, src, wt, pair_bits);
    if (!any) {
        if (COPY) copy_channels(cs, o, C);
        return;
    }
    for (int c = 0; c < C; ++c) {
        const float base = cs[c];
        float v = base;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (src[q] >= 0) v = fmaf(wt[q], Cc[(long long)src[q] * C + c] - base, v);
        o[c] = v;
    }
}

__device__ __forceinline__ float l1_sign(float d, float scale) {
    return d > 0.0f ? scale : (d < 0.0f ? -scale : 0.0f);
}

// Forward of one pixel with the mean-absolute-error loss fused
// (aa_fwd_pixel_l1 = aa_fwd_terms + aa_l1_channels): the output value of
// every channel as aa_fwd_pixel computes it (written to o when o is not
// null), g = sign(out - target) * scale (written when g is not null), and
// the return value is the pixel's sum of |out - target| in channel order.
// tg, o, g: this pixel's target, output and gradient rows; pair_bits: as
// aa_fwd_terms.  sign_nz / sign_pos (may be null; at most 32 channels): bit c
// set when out - target of channel c is nonzero / positive, which is g
// without the buffer.  aa_l1_channels takes the blend terms (src, wt, any)
// from aa_fwd_terms or aa_fwd_terms_row.
__device__ __forceinline__ float aa_l1_channels(const float* Cc, int C, int pix, const int (&src)[4],
                                                const float (&wt)[4], bool any, const float* tg, float scale, float* o,
                                                float* g, unsigned* sign_nz = nullptr, unsigned* sign_pos = nullptr) {
    const float* cs = Cc + (long long)pix * C;
    float s = 0.0f;
    unsigned nz = 0u, ps = 0u;
    const bool vec = (C & 3) == 0 && (((uintptr_t)cs | (uintptr_t)tg | (uintptr_t)(g ? g : cs) |
                                       (uintptr_t)(o ? o : cs)) & 15) == 0;
    if (vec) {
        for (int c = 0; c < C; c += 4) {
            const float4 b4 = *reinterpret_cast<const float4*>(cs + c);
            const float4 t4 = *reinterpret_cast<const float4*>(tg + c);
            const float base[4] = {b4.x, b4.y, b4.z, b4.w};
            float v[4] = {b4.x, b4.y, b4.z, b4.w};
            if (any) {
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (src[q] < 0) continue;
                    const float4 s4 = *reinterpret_cast<const float4*>(Cc + (long long)src[q] * C + c);
                    const float sv[4] = {s4.x, s4.y, s4.z, s4.w};
#pragma unroll
                    for (int k = 0; k < 4; ++k) v[k] = fmaf(wt[q], sv[k] - base[k], v[k]);
                }
            }
            if (o) *reinterpret_cast<float4*>(o + c) = make_float4(v[0], v[1], v[2], v[3]);
            const float tv[4] = {t4.x, t4.y, t4.z, t4.w};
            float gv[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float d = v[k] - tv[k];
                s += fabsf(d);
                gv[k] = l1_sign(d, scale);
                if (d > 0.0f || d < 0.0f) nz |= 1u << ((c + k) & 31);
                if (d > 0.0f) ps |= 1u << ((c + k) & 31);
            }
            if (g) *reinterpret_cast<float4*>(g + c) = make_float4(gv[0], gv[1], gv[2], gv[3]);
        }
    } else {
        for (int c = 0; c < C; ++c) {
            const float base = cs[c];
            float v = base;
            if (any) {
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (src[q] >= 0) v = fmaf(wt[q], Cc[(long long)src[q] * C + c] - base, v);
            }
            if (o) o[c] = v;
            const float d = v - tg[c];
            s += fabsf(d);
            if (g) g[c] = l1_sign(d, scale);
            if (d > 0.0f || d < 0.0f) nz |= 1u << (c & 31);
            if (d > 0.0f) ps |= 1u << (c & 31);
        }
    }
    if (sign_nz) *sign_nz = nz;
    if (sign_pos) *sign_pos = ps;
    return s;
}

__device__ __forceinline__ float aa_fwd_pixel_l1(const float4* R, const float* Cc, const float4* rec, long long F,
                                                 int W, int H, int C, int pix, const float* tg, float scale, float* o,
                                                 float* g, unsigned* pair_bits = nullptr, unsigned* sign_nz = nullptr,
                                                 unsigned* sign_pos = nullptr) {
    int src[4];
    float wt[4];
    const bool any = aa_fwd_terms(R, rec, F, W, H, pix, src, wt, pair_bits);
    return aa_l1_channels(Cc, C, pix, src, wt, any, tg, scale, o, g, sign_nz, sign_pos);
}

// The incoming image gradient at flat index i (pixel * C + channel), as the
// backward reads it.  GradBuffer: a gradient buffer times a scale (a loss's
// upstream gradient applied on the fly; 1 leaves the values unchanged).
// GradL1: the gradient of the mean-absolute-error loss, sign(out - target) *
// scale, formed from the output and the target instead of a stored buffer.
// aligned() / load4(i): the same values four at a time (i a multiple of 4,
// the buffers 16-byte aligned).
struct GradBuffer {
    const float* g;
    float s;
    __device__ __forceinline__ float operator()(long long i) const { return g[i] * s; }
    __device__ __forceinline__ bool aligned() const { return (reinterpret_cast<uintptr_t>(g) & 15) == 0; }
    __device__ __forceinline__ float4 load4(long long i) const {
        const float4 v = *reinterpret_cast<const float4*>(g + i);
        return make_float4(v.x * s, v.y * s, v.z * s, v.w * s);
    }
};

struct GradL1 {
    const float* out;
    const float* tgt;
    float scale;
    __device__ __forceinline__ float operator()(long long i) const { return l1_sign(out[i] - tgt[i], scale); }
    __device__ __forceinline__ bool aligned() const {
        return ((reinterpret_cast<uintptr_t>(out) | reinterpret_cast<uintptr_t>(tgt)) & 15) == 0;
    }
    __device__ __forceinline__ float4 load4(long long i) const {
        const float4 o = *reinterpret_cast<const float4*>(out + i), t = *reinterpret_cast<const float4*>(tgt + i);
        return make_float4(l1_sign(o.x - t.x, scale), l1_sign(o.y - t.y, scale), l1_sign(o.z - t.z, scale),
                           l1_sign(o.w - t.w, scale));
    }
};

// Backward pair terms of one pixel.  For every pair slot: role (0 none, 1 this
// pixel is the blend target, 2 the source), the target pixel and the weight;
// the edge-vertex gradients of each pair are scattered here, once per pair
// (by its first pixel), into GP (may be null).
// Edge-vertex gradient of one valid, unclamped pair (scattered by the pair's
// first pixel): dL/dt through the blend weight, then t through the exit
// edge's two screen vertices to their clip coordinates.
template <class G>
__device__ __forceinline__ void aa_edge_grad_g(const AAPair& p, const float* Cc, const G& grad, int C,
                                               const float4* P, const int* tri, float4* GP, float boost, int W,
                                               int H) {
    float dLdw = 0.f;
    if ((C & 3) == 0 && grad.aligned() && (reinterpret_cast<uintptr_t>(Cc) & 15) == 0) {
        // 128-bit loads, the same channel-order accumulation
        for (int c = 0; c < C; c += 4) {
            const float4 g = grad.load4((long long)p.target * C + c);
            const float4 cs = *reinterpret_cast<const float4*>(Cc + (long long)p.src * C + c);
            const float4 ct = *reinterpret_cast<const float4*>(Cc + (long long)p.target * C + c);
            dLdw = fmaf(g.x, cs.x - ct.x, dLdw);
            dLdw = fmaf(g.y, cs.y - ct.y, dLdw);
            dLdw = fmaf(g.z, cs.z - ct.z, dLdw);
            dLdw = fmaf(g.w, cs.w - ct.w, dLdw);
        }
    } else {
        for (int c = 0; c < C; ++c)
            dLdw = fmaf(grad((long long)p.target * C + c),
                        Cc[(long long)p.src * C + c] - Cc[(long long)p.target * C + c], dLdw);
    }
    const float dLdt = dLdw * p.sign * boost;
    const float den = p.eF - p.eO;
    const float inv2 = 1.0f / (den * den);
    const float dtF = -p.eO * inv2, dtO = p.eF * inv2;
    const float2 ea = p.s[(p.k + 1) % 3], eb = p.s[(p.k + 2) % 3];
    const float fF = dLdt * dtF * p.sgn, fO = dLdt * dtO * p.sgn;
    const float gA0 = fmaf(fF, eb.y - p.cF.y, fO * (eb.y - p.cO.y));
    const float gA1 = fmaf(fF, p.cF.x - eb.x, fO * (p.cO.x - eb.x));
    const float gB0 = fmaf(fF, p.cF.y - ea.y, fO * (p.cO.y - ea.y));
    const float gB1 = fmaf(fF, ea.x - p.cF.x, fO * (ea.x - p.cO.x));
    const int vA = tri[3 * (long long)p.T + (p.k + 1) % 3], vB = tri[3 * (long long)p.T + (p.k + 2) % 3];
    const float hx = 0.5f * (float)W, hy = 0.5f * (float)H;
    const float4 pA = P[vA], pB = P[vB];
    const float iwA = 1.0f / pA.w, iwB = 1.0f / pB.w;
    atomic_add4(GP + vA, make_float4(gA0 * hx * iwA, gA1 * hy * iwA, 0.f,
                                     -(gA0 * hx * pA.x + gA1 * hy * pA.y) * iwA * iwA));
    atomic_add4(GP + vB, make_float4(gB0 * hx * iwB, gB1 * hy * iwB, 0.f,
                                     -(gB0 * hx * pB.x + gB1 * hy * pB.y) * iwB * iwB));
}

__device__ __forceinline__ void aa_edge_grad(const AAPair& p, const float* Cc, const float* Gd, int C,
                                             const float4* P, const int* tri, float4* GP, float boost, float gscale,
                                             int W, int H) {
    aa_edge_grad_g(p, Cc, GradBuffer{Gd, gscale}, C, P, tri, GP, boost, W, H);
}

struct AATerms {
    int role[4], tgt[4];
    float wt[4];
    bool any;
};

__device__ __forceinline__ void aa_bwd_terms(const float4* R, const float* Cc, const float* Gd, const float4* rec,
                                             long long F, int W, int H, int C, const float4* P, const int* tri,
                                             float4* GP, float boost, int pix, AATerms& at, float gscale = 1.0f) {
    const int py = pix / W, px = pix - py * W;
    int As[4], Bs[4], axs[4], ays[4];
    bool verts[4], has[4];
    float4 rn[4];
    const float4 rs = R[pix];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        has[q] = pair_slot(q, pix, px, py, W, H, As[q], Bs[q], axs[q], ays[q], verts[q]);
        if (has[q]) rn[q] = R[As[q] == pix ? Bs[q] : As[q]];
    }
    at.any = false;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        at.role[q] = 0;
        at.tgt[q] = 0;
        at.wt[q] = 0.f;
        if (!has[q]) continue;
        const int A = As[q], B = Bs[q];
        const float4 ro = rn[q];
        if (ro.w == rs.w) continue;
        AAPair p;
        aa_pair(rec, F, A, B, axs[q], ays[q], verts[q], A == pix ? rs : ro, A == pix ? ro : rs, p);
        if (!p.valid) continue;
        at.role[q] = p.target == pix ? 1 : 2;
        at.tgt[q] = p.target;
        at.wt[q] = p.w;
        at.any = true;
        if (!GP || A != pix || p.clamped) continue;
        aa_edge_grad(p, Cc, Gd, C, P, tri, GP, boost, gscale, W, H);
    }
}

// Colour gradient of channel c of a pixel from its terms (slot order).
// gscale multiplies every incoming gradient as it is read (a loss gradient
// applied on the fly; 1 leaves them unchanged).
template <class G>
__device__ __forceinline__ float aa_bwd_channel_g(const AATerms& at, const G& grad, int C, int pix, int c) {
    const float gs = grad((long long)pix * C + c);
    float v = gs;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if (at.role[q] == 1) v = fmaf(-at.wt[q], gs, v);
        else if (at.role[q] == 2) v = fmaf(at.wt[q], grad((long long)at.tgt[q] * C + c), v);
    }
    return v;
}

__device__ __forceinline__ float aa_bwd_channel(const AATerms& at, const float* Gd, int C, int pix, int c,
                                                float gscale = 1.0f) {
    return aa_bwd_channel_g(at, GradBuffer{Gd, gscale}, C, pix, c);
}

}  // namespace drp
