// raster_core.cuh -- rasterisation building blocks shared by the plain
// (per-call) pipeline in raster.cu and the batched pipeline in batch.cu:
// triangle setup into 48-byte primitive records, tile binning, per-tile
// primitive preparation (int32 edge steps with trivial accept / reject) and
// the fine raster of one tile by one CTA.
#pragma once
#include "drp_common.cuh"
#include "drp_internal.h"

namespace drp {

// Primitive record (3 x int4 = 48 bytes).
//   r0 = {X0, Y0, X1, Y1}                 fixed-point vertices
//   r1 = {X2, Y2, tri, px0 | px1 << 16}
//   r2 = {Z0, A, B (float bits), py0 | py1 << 16 | COMPLEX << 31}
// A culled record has px0 = 1, px1 = 0 (empty range).  COMPLEX records were
// clipped; the fine raster re-derives their polygon from the clip vertices.
#define PRIM_COMPLEX 0x80000000u

struct PrimBox {
    int px0, px1, py0, py1;
    bool complex_;
};

__device__ __forceinline__ PrimBox unpack_box(const int4& r1, const int4& r2) {
    PrimBox b;
    uint32_t xs = (uint32_t)r1.w, ys = (uint32_t)r2.w;
    b.px0 = xs & 0xffff;
    b.px1 = xs >> 16;
    b.py0 = ys & 0x7fff;
    b.py1 = (ys >> 16) & 0x7fff;
    b.complex_ = (ys & PRIM_COMPLEX) != 0;
    return b;
}

// Warp-aggregated increment of counter[idx] by 1; returns the old value for
// this lane (its slot).  All lanes in `active` must call it.
__device__ __forceinline__ uint32_t warp_agg_inc(uint32_t* counter, uint32_t idx, unsigned active) {
    unsigned peers = __match_any_sync(active, idx);
    int leader = __ffs(peers) - 1;
    int lane = lane_id();
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter + idx, (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

// Triangle setup into a primitive record.  P: the view's clip vertices,
// t: the triangle's index in `tri` (written into the record and used as the
// visibility id), vertex indices already validated.  Returns false when the
// triangle covers no pixel centre (culled record).
__device__ __forceinline__ bool build_prim(const float4& p0, const float4& p1, const float4& p2, long long t, int W,
                                           int H, int4* rec, PrimBox& box) {
    int4 r0 = make_int4(0, 0, 0, 0), r1 = make_int4(0, 0, (int)t, 0), r2 = make_int4(0, 0, 0, 0);
    const int kind = needs_clip_or_cull(p0, p1, p2);
    int64_t mnx = 0, mxx = -1, mny = 0, mxy = -1;
    bool ok = false;
    if (kind == 1) {
        const int32_t X0 = snap_coord(p0.x, p0.w, W), Y0 = snap_coord(p0.y, p0.w, H);
        const int32_t X1 = snap_coord(p1.x, p1.w, W), Y1 = snap_coord(p1.y, p1.w, H);
        const int32_t X2 = snap_coord(p2.x, p2.w, W), Y2 = snap_coord(p2.y, p2.w, H);
        const float Z0 = p0.z / p0.w, Z1 = p1.z / p1.w, Z2 = p2.z / p2.w;
        const int64_t area2 = (int64_t)(X1 - X0) * (int64_t)(Y2 - Y0) - (int64_t)(Y1 - Y0) * (int64_t)(X2 - X0);
        if (area2 != 0) {
            Plane pl = depth_plane(X0, Y0, Z0, X1, Y1, Z1, X2, Y2, Z2, area2);
            r0 = make_int4(X0, Y0, X1, Y1);
            r1 = make_int4(X2, Y2, (int)t, 0);
            r2 = make_int4(__float_as_int(pl.Z0), __float_as_int(pl.A), __float_as_int(pl.B), 0);
            mnx = min(min(X0, X1), X2);
            mxx = max(max(X0, X1), X2);
            mny = min(min(Y0, Y1), Y2);
            mxy = max(max(Y0, Y1), Y2);
            ok = true;
        }
    } else if (kind == 2) {
        Poly poly;
        setup_clipped(p0, p1, p2, W, H, poly);
        if (poly.n >= 3) {
            mnx = mxx = poly.X[0];
            mny = mxy = poly.Y[0];
            for (int i = 1; i < poly.n; ++i) {
                mnx = min(mnx, (int64_t)poly.X[i]);
                mxx = max(mxx, (int64_t)poly.X[i]);
                mny = min(mny, (int64_t)poly.Y[i]);
                mxy = max(mxy, (int64_t)poly.Y[i]);
            }
            ok = true;
        }
    }
    bool live = false;
    box.px0 = 1;
    box.px1 = 0;
    box.py0 = box.py1 = 0;
    box.complex_ = kind == 2;
    if (ok) {
        int64_t x0 = ceil_shift(mnx - DRP_HALF_SUBPIX), x1 = floor_shift(mxx - DRP_HALF_SUBPIX);
        int64_t y0 = ceil_shift(mny - DRP_HALF_SUBPIX), y1 = floor_shift(mxy - DRP_HALF_SUBPIX);
        x0 = max(x0, (int64_t)0);
        x1 = min(x1, (int64_t)(W - 1));
        y0 = max(y0, (int64_t)0);
        y1 = min(y1, (int64_t)(H - 1));
        if (x0 <= x1 && y0 <= y1) {
            box.px0 = (int)x0;
            box.px1 = (int)x1;
            box.py0 = (int)y0;
            box.py1 = (int)y1;
            live = true;
            r2.w = (int)((uint32_t)box.py0 | ((uint32_t)box.py1 << 16) | (kind == 2 ? PRIM_COMPLEX : 0u));
        }
    }
    if (!live) {
        r2.w = 0;
        box.px0 = 1;
        box.px1 = 0;
    }
    r1.w = (int)((uint32_t)box.px0 | ((uint32_t)box.px1 << 16));
    rec[0] = r0;
    rec[1] = r1;
    rec[2] = r2;
    return live;
}

// For every tile the box overlaps: count (list == null) or append `pidx` to
// the tile's list through the cursors (warp-aggregated slots; entries past
// `capacity` are dropped and the tile falls back to a full scan).
// depth == 0: counters are cursors into one list of `capacity` entries
// (slot = list index); depth > 0: counters count per tile and tile t's
// entries go to list[t * depth + slot] while slot < depth (fixed-depth bins).
// All 32 lanes of the warp call this (live = false for lanes with nothing to
// bin), with one counters / tiles_x for the whole warp.  The warp's (box,
// tile) pairs are dealt out over its lanes -- pair k to lane k % 32 -- so a
// box covering many tiles costs its warp ceil(pairs / 32) rounds of
// dependent atomics instead of one round per tile of the largest box.
template <int TILE_LOG2>
__device__ __forceinline__ void bin_box(const PrimBox& bx, bool live, int tiles_x, uint32_t* counters,
                                        uint32_t* list, unsigned long long capacity, uint32_t pidx,
                                        uint32_t depth = 0) {
    const unsigned FULL = 0xffffffffu;
    const int lane = lane_id();
    const int tx0 = bx.px0 >> TILE_LOG2, tx1 = bx.px1 >> TILE_LOG2, ty0 = bx.py0 >> TILE_LOG2,
              ty1 = bx.py1 >> TILE_LOG2;
    const int n = live ? (tx1 - tx0 + 1) * (ty1 - ty0 + 1) : 0;
    const int w = live ? tx1 - tx0 + 1 : 1;
    int incl = n;  // inclusive prefix of the lanes' pair counts
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(FULL, incl, d);
        if (lane >= d) incl += y;
    }
    const int total = __shfl_sync(FULL, incl, 31);
    const int start = incl - n;
    for (int k0 = 0; k0 < total; k0 += 32) {  // warp-uniform trip count
        const int k = k0 + lane;
        // owner of pair k: the number of lanes whose prefix ends at or before k
        int o = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const int v = __shfl_sync(FULL, incl, o + step - 1);
            if (v <= k) o += step;
        }
        const int o_start = __shfl_sync(FULL, start, o), o_w = __shfl_sync(FULL, w, o);
        const int o_tx0 = __shfl_sync(FULL, tx0, o), o_ty0 = __shfl_sync(FULL, ty0, o);
        const uint32_t o_pidx = __shfl_sync(FULL, pidx, o);
        const bool has = k < total;
        const unsigned active = __ballot_sync(FULL, has);
        if (!has) continue;
        const int r = k - o_start;
        const uint32_t tile = (uint32_t)((o_ty0 + r / o_w) * tiles_x + o_tx0 + r % o_w);
        const uint32_t slot = warp_agg_inc(counters, tile, active);
        if (depth) {
            if (slot < depth) list[(unsigned long long)tile * depth + slot] = o_pidx;
        } else if (list && slot < capacity) {
            list[slot] = o_pidx;
        }
    }
}

// Rasterise one fan sub-triangle into the tile's key buffer (group-strided,
// shared-memory atomicMin).  Used for clipped polygons, whose fan
// sub-triangles each carry their own depth plane.
template <int TILE_LOG2>
__device__ __forceinline__ void raster_subtri_tile(int64_t X0, int64_t Y0, int64_t X1, int64_t Y1, int64_t X2,
                                                   int64_t Y2, const Plane& pl, uint32_t tri, int tx0, int ty0,
                                                   int W, int H, int rank, int group, unsigned long long* keys,
                                                   const unsigned long long* prev) {
    constexpr int T = 1 << TILE_LOG2;
    const int64_t area2 = (X1 - X0) * (Y2 - Y0) - (Y1 - Y0) * (X2 - X0);
    if (area2 == 0) return;
    int64_t ax = X0, ay = Y0, bx = X1, by = Y1, cx = X2, cy = Y2;
    if (area2 < 0) {
        bx = X2; by = Y2; cx = X1; cy = Y1;
    }
    int64_t mnx = min(min(X0, X1), X2), mxx = max(max(X0, X1), X2);
    int64_t mny = min(min(Y0, Y1), Y2), mxy = max(max(Y0, Y1), Y2);
    const int x0 = (int)max(ceil_shift(mnx - DRP_HALF_SUBPIX), (int64_t)tx0);
    const int x1 = (int)min(floor_shift(mxx - DRP_HALF_SUBPIX), (int64_t)min(tx0 + T - 1, W - 1));
    const int y0 = (int)max(ceil_shift(mny - DRP_HALF_SUBPIX), (int64_t)ty0);
    const int y1 = (int)min(floor_shift(mxy - DRP_HALF_SUBPIX), (int64_t)min(ty0 + T - 1, H - 1));
    if (x0 > x1 || y0 > y1) return;
    const int w = x1 - x0 + 1;
    const int n = w * (y1 - y0 + 1);
    for (int i = rank; i < n; i += group) {
        const int px = x0 + i % w, py = y0 + i / w;
        const int64_t sx = (int64_t)px * DRP_SUBPIX + DRP_HALF_SUBPIX;
        const int64_t sy = (int64_t)py * DRP_SUBPIX + DRP_HALF_SUBPIX;
        if (!edge_inside(bx, by, cx, cy, sx, sy)) continue;
        if (!edge_inside(cx, cy, ax, ay, sx, sy)) continue;
        if (!edge_inside(ax, ay, bx, by, sx, sy)) continue;
        const float z = (pl.Z0 + pl.A * (float)(sx - X0)) + pl.B * (float)(sy - Y0);
        if (!(z >= -1.0f && z <= 1.0f)) continue;
        const unsigned long long k = ((unsigned long long)depth_order(z) << 32) | (unsigned long long)tri;
        const int li = ((py - ty0) << TILE_LOG2) + (px - tx0);
        if (prev && !(k > prev[li])) continue;
        if (k < keys[li]) atomicMin(keys + li, k);
    }
}

template <int TILE_LOG2>
__device__ __noinline__ void raster_complex_tile(const float4* P, const int* tri_idx, int W, int H, uint32_t tri,
                                                 int tx0, int ty0, int rank, int group, unsigned long long* keys,
                                                 const unsigned long long* prev) {
    const int i0 = tri_idx[3 * (long long)tri], i1 = tri_idx[3 * (long long)tri + 1],
              i2 = tri_idx[3 * (long long)tri + 2];
    Poly poly;
    setup_clipped(P[i0], P[i1], P[i2], W, H, poly);
    for (int i = 1; i + 1 < poly.n; ++i) {
        const int64_t X0 = poly.X[0], Y0 = poly.Y[0], X1 = poly.X[i], Y1 = poly.Y[i];
        const int64_t X2 = poly.X[i + 1], Y2 = poly.Y[i + 1];
        const int64_t area2 = (X1 - X0) * (Y2 - Y0) - (Y1 - Y0) * (X2 - X0);
        if (area2 == 0) continue;
        const Plane pl = depth_plane(X0, Y0, poly.Z[0], X1, Y1, poly.Z[i], X2, Y2, poly.Z[i + 1], area2);
        raster_subtri_tile<TILE_LOG2>(X0, Y0, X1, Y1, X2, Y2, pl, tri, tx0, ty0, W, H, rank, group, keys, prev);
    }
}

// A primitive prepared for one tile.  Edge k passes at tile pixel (dx, dy)
// when C[k] + A[k] dx + B[k] dy >= 0 (top-left bias folded into C).  Edges
// that accept every pixel of the tile are reduced to A = B = C = 0.  BIG
// primitives have an edge too long for 32-bit steps and are tested in 64-bit
// from the (oriented) vertices.
#define TP_ACTIVE 1
#define TP_BIG 2
#define TP_COMPLEX 4
#define TP_NEG 8  // clockwise in the snapped screen frame (the other facing class)

struct __align__(16) TilePrim {
    int4 e0;    // A0, B0, C0, A1
    int4 e1;    // B1, C1, A2, B2
    int4 e2;    // C2, flags, X0, Y0
    float4 z;   // Z0, Az, Bz, tri (bits)
    int4 v01;   // oriented vertices for the BIG path: x0, y0, x1, y1
    int4 v2b;   // x2, y2, local bbox x0 | x1 << 16, y0 | y1 << 16
};

template <int T>
__device__ __forceinline__ void prepare_tile_prim(const int4* rec, int tx0, int ty0, int W, int H, TilePrim& tp) {
    tp.e2.y = 0;
    const int4 r1 = rec[1], r2 = rec[2];
    const PrimBox bx = unpack_box(r1, r2);
    if (bx.px0 > bx.px1 || bx.px1 < tx0 || bx.px0 >= tx0 + T || bx.py1 < ty0 || bx.py0 >= ty0 + T) return;
    tp.z.w = __int_as_float(r1.z);
    const int lx0 = max(bx.px0, tx0) - tx0, lx1 = min(min(bx.px1, tx0 + T - 1), W - 1) - tx0;
    const int ly0 = max(bx.py0, ty0) - ty0, ly1 = min(min(bx.py1, ty0 + T - 1), H - 1) - ty0;
    tp.v2b.z = lx0 | (lx1 << 16);
    tp.v2b.w = ly0 | (ly1 << 16);
    if (bx.complex_) {
        tp.e2.y = TP_COMPLEX;
        return;
    }
    const int4 r0 = rec[0];
    const int64_t X0 = r0.x, Y0 = r0.y, X1 = r0.z, Y1 = r0.w, X2 = r1.x, Y2 = r1.y;
    const int64_t area2 = (X1 - X0) * (Y2 - Y0) - (Y1 - Y0) * (X2 - X0);
    int64_t vx[3] = {X0, X1, X2}, vy[3] = {Y0, Y1, Y2};
    if (area2 < 0) {
        vx[1] = X2; vy[1] = Y2; vx[2] = X1; vy[2] = Y1;
    }
    const int64_t ox = (int64_t)tx0 * DRP_SUBPIX + DRP_HALF_SUBPIX;
    const int64_t oy = (int64_t)ty0 * DRP_SUBPIX + DRP_HALF_SUBPIX;
    bool big = false;
    int A[3], B[3], C[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int p = (k + 1) % 3, q = (k + 2) % 3;  // edges b->c, c->a, a->b
        const int64_t dx = vx[q] - vx[p], dy = vy[q] - vy[p];
        const bool tl = (dy < 0) || (dy == 0 && dx < 0);
        const int64_t Cb = dx * (oy - vy[p]) - dy * (ox - vx[p]) - (tl ? 0 : 1);
        const int64_t SX = -dy * DRP_SUBPIX, SY = dx * DRP_SUBPIX;
        const int64_t lo = (min(SX, (int64_t)0) + min(SY, (int64_t)0)) * (T - 1);
        const int64_t hi = (max(SX, (int64_t)0) + max(SY, (int64_t)0)) * (T - 1);
        A[k] = B[k] = C[k] = 0;
        if (Cb + hi < 0) return;  // no pixel centre of the tile is inside this edge
        if (Cb + lo >= 0) continue;  // every pixel centre of the tile is inside
        if (hi - lo < ((int64_t)1 << 30)) {
            A[k] = (int)SX;
            B[k] = (int)SY;
            C[k] = (int)Cb;
        } else {
            big = true;
        }
    }
    tp.e0 = make_int4(A[0], B[0], C[0], A[1]);
    tp.e1 = make_int4(B[1], C[1], A[2], B[2]);
    tp.e2 = make_int4(C[2], TP_ACTIVE | (big ? TP_BIG : 0) | (area2 < 0 ? TP_NEG : 0), (int)X0, (int)Y0);
    tp.z.x = __int_as_float(r2.x);
    tp.z.y = __int_as_float(r2.y);
    tp.z.z = __int_as_float(r2.z);
    tp.v01 = make_int4((int)vx[0], (int)vy[0], (int)vx[1], (int)vy[1]);
    tp.v2b.x = (int)vx[2];
    tp.v2b.y = (int)vy[2];
}

// A lower bound of the depth (z/w) of every fragment the primitive can
// produce: the plane's minimum over the triangle is at a vertex; fragments are
// evaluated as (Z0 + A dx) + B dy in float, so the bound is lowered by a few
// ulps of the largest term (2^-20 relative; each of the three roundings is at
// most 2^-24 of its result).
__device__ __forceinline__ float prim_depth_lower_bound(const TilePrim& tp) {
    const float Z0 = tp.z.x, A = tp.z.y, B = tp.z.z;
    const int X0 = tp.e2.z, Y0 = tp.e2.w;
    const float dx[3] = {(float)(tp.v01.x - X0), (float)(tp.v01.z - X0), (float)(tp.v2b.x - X0)};
    const float dy[3] = {(float)(tp.v01.y - Y0), (float)(tp.v01.w - Y0), (float)(tp.v2b.y - Y0)};
    float zmin = 3.0e38f, ax = 0.0f, by = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float za = A * dx[i], zb = B * dy[i];
        zmin = fminf(zmin, (Z0 + za) + zb);
        ax = fmaxf(ax, fabsf(za));
        by = fmaxf(by, fabsf(zb));
    }
    const float m = fabsf(Z0) + ax + by;
    return zmin - m * 9.5367431640625e-7f - 1.0e-30f;  // 2^-20 of the magnitude
}

__device__ __forceinline__ bool tile_prim_covers(const TilePrim& tp, const int4& e0, const int4& e1, const int4& e2,
                                                 int dx, int dy, int sx, int sy) {
    if (!(e2.y & TP_BIG)) {
        return (e0.z + e0.x * dx + e0.y * dy >= 0) && (e1.y + e0.w * dx + e1.x * dy >= 0) &&
               (e2.x + e1.z * dx + e1.w * dy >= 0);
    }
    const int4 v01 = tp.v01, v2b = tp.v2b;
    return edge_inside(v01.z, v01.w, v2b.x, v2b.y, sx, sy) && edge_inside(v2b.x, v2b.y, v01.x, v01.y, sx, sy) &&
           edge_inside(v01.x, v01.y, v01.z, v01.w, sx, sy);
}

__device__ __forceinline__ unsigned long long tile_prim_key(const float4& z4, int X0, int Y0, int sx, int sy,
                                                            bool& ok) {
    const float z = (z4.x + z4.y * (float)(sx - X0)) + z4.z * (float)(sy - Y0);
    ok = (z >= -1.0f && z <= 1.0f);
    return ((unsigned long long)depth_order(z) << 32) | (unsigned long long)__float_as_uint(z4.w);
}

// Pixel q of thread tid inside a tile.  The tile is cut into 8x4 pixel
// blocks, numbered row-major (T/8 per row); lanes are row-major inside a
// block.  With one pixel per thread warp w owns block w; with four (32-pixel
// tiles, 256 threads) warp w owns the 2x2 blocks of the 16x8 region at
// ((w & 1) * 16, (w >> 1) * 8), q walking them row-major.  A warp can then
// skip a primitive whose block mask misses its blocks with one uniform test.
// (Spreading a warp's four blocks over the tile instead -- one per pair of
// block rows -- balanced the warps better but made every primitive hit more
// warps: the fine raster took 13 us longer on the single-mesh step.)
template <int TILE_LOG2, int NTHREADS>
__device__ __forceinline__ int tile_block(int tid, int q) {
    constexpr int T = 1 << TILE_LOG2;
    constexpr int PPT = T * T / NTHREADS;
    static_assert(PPT == 1 || (PPT == 4 && T == 32), "tile_pixel: unsupported tile shape");
    const int w = tid >> 5;
    if (PPT == 4) return ((((w >> 1) << 1) | (q >> 1)) * (T / 8)) + (((w & 1) << 1) | (q & 1));
    return w + q * (NTHREADS >> 5);
}

template <int TILE_LOG2, int NTHREADS>
__device__ __forceinline__ void tile_pixel(int tid, int q, int& dx, int& dy, int& bx, int& by) {
    constexpr int T = 1 << TILE_LOG2;
    const int blk = tile_block<TILE_LOG2, NTHREADS>(tid, q);
    bx = (blk % (T / 8)) * 8;
    by = (blk / (T / 8)) * 4;
    dx = bx + (tid & 7);
    dy = by + ((tid >> 3) & 3);
}

// Bit b set when the local bbox [x0, x1] x [y0, y1] overlaps 8x4 block b
// (row-major, T/8 blocks per row; at most 32 blocks per tile).
template <int T>
__device__ __forceinline__ uint32_t block_mask(int x0, int x1, int y0, int y1) {
    constexpr int CW = T / 8;
    constexpr unsigned long long REP = CW == 4 ? 0x11111111ull : (CW == 2 ? 0x55ull : 0x3ull);
    const unsigned long long cols = (2ull << (x1 >> 3)) - (1ull << (x0 >> 3));
    const unsigned long long rows = (1ull << (((y1 >> 2) + 1) * CW)) - (1ull << ((y0 >> 2) * CW));
    return (uint32_t)(cols * REP & rows);
}

// Column bits of one block row where a tile-local edge C + A dx + B dy holds
// a pixel centre: bit i for the 8x4 block at columns [8i, 8i + 8) of the
// rows [by, by + 4).  The edge's largest value over a block is at the corner
// its steps point to; along the row it changes by 8 A per block.  In range of
// int32 for every pixel of the tile (prepare_tile_prim keeps 32-bit steps only
// where the edge's span over the tile is below 2^30).
template <int COLS>
__device__ __forceinline__ uint32_t edge_row_blocks(int A, int B, int C, int by) {
    const int v = C + (A > 0 ? 7 * A : 0) + B * (B > 0 ? by + 3 : by);
    uint32_t bits = 0u;
#pragma unroll
    for (int i = 0; i < COLS; ++i) bits |= (v + 8 * i * A >= 0 ? 1u : 0u) << i;
    return bits;
}

// Narrow each prepared primitive's bounding-box block mask to the 8x4 blocks
// that hold a pixel centre inside all three of its edges (exact: a block
// dropped here has no pixel the primitive covers).  The bounding box of a
// thin or diagonal triangle meets many blocks it never touches; each such
// block would otherwise test the primitive at all 32 pixels.  One lane per
// (primitive, block row): a warp handles 32 / (T / 4) primitives at a time
// (4 on 32-pixel tiles), each lane testing the T / 8 blocks of its row, and
// the rows' bits are OR-ed across the primitive's lanes.  BIG primitives
// (64-bit edges) keep their bounding-box mask.  The result goes to
// pcls[class][j] (class: facing, TP_NEG), 0 in the other class's row, so the
// fine loop selects a class and a block with one load.
template <int T, int NTHREADS>
__device__ __forceinline__ void refine_block_masks(const TilePrim* prims, const uint32_t* pmask,
                                                   uint32_t (*pcls)[NTHREADS], int n) {
    constexpr int ROWS = T / 4, COLS = T / 8;  // 8x4 blocks per tile column / row
    constexpr int PPW = 32 / ROWS;              // primitives per warp pass
    constexpr int NW = NTHREADS / 32;
    static_assert(ROWS * COLS <= 32 && 32 % ROWS == 0, "refine_block_masks: at most 32 blocks per tile");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sub = lane / ROWS, row = lane % ROWS;
    const int shift = row * COLS;
    for (int j0 = warp * PPW; j0 < n; j0 += NW * PPW) {
        const int j = j0 + sub;
        uint32_t bits = 0u;
        int neg = 0;
        if (j < n) {
            const int fl = prims[j].e2.y;
            neg = (fl & TP_NEG) ? 1 : 0;
            bits = (pmask[j] >> shift) & ((1u << COLS) - 1u);
            if (bits && !(fl & TP_BIG)) {
                const int4 e0 = prims[j].e0, e1 = prims[j].e1, e2 = prims[j].e2;
                const int by = row * 4;
                bits &= edge_row_blocks<COLS>(e0.x, e0.y, e0.z, by) & edge_row_blocks<COLS>(e0.w, e1.x, e1.y, by) &
                        edge_row_blocks<COLS>(e1.z, e1.w, e2.x, by);
            }
        }
        uint32_t m = bits << shift;
#pragma unroll
        for (int off = 1; off < ROWS; off <<= 1) m |= __shfl_xor_sync(0xffffffffu, m, off);
        if (row == 0 && j < n) {
            pcls[neg][j] = m;
            pcls[1 - neg][j] = 0u;
        }
    }
}

// One tile's work for the fine raster.
struct FineTile {
    const int4* recs;           // primitive records
    const uint32_t* list;       // this tile's list entries (first entry)
    uint32_t cnt;               // list length
    bool overflow;              // list incomplete: scan [scan_base, scan_base + scan_count)
    long long scan_base, scan_count;
    int tx0, ty0, W, H;
    const float4* P;            // the view's clip vertices (complex primitives)
    const int* tri;
    const unsigned long long* prev;  // the view's previous-layer keys or null
    uint32_t* stats;            // device error bits or null
};

// Fine raster of one tile by one CTA, then emit(px, py, key, ndc x, ndc y)
// for every pixel of the tile inside the viewport.
//   TPT == 0: pixel-parallel.  The tile's 8x4 pixel blocks are handed to the
//             warps one at a time from a shared counter; a warp tests its
//             block's 32 pixels (one per lane, keys in registers) against
//             every primitive whose bounding box meets the block, nearer
//             facing class first, then the other class with the blocks'
//             depth bound, and emits the block at once when the keys are
//             final.  A warp that drew light blocks takes more of them, so
//             the warps of a CTA reach the tile's barriers together (fixed
//             16x8 regions per warp left half of them waiting at the
//             barriers for the busiest one).  Keys go through shared memory
//             only when a tile needs more than one chunk of primitives or
//             has clipped (complex) primitives.
//   TPT  > 0: groups of TPT threads walk one primitive's bbox within the tile
//             and resolve keys with shared-memory atomicMin.
//   PEEL = false: ft.prev is ignored (no previous layer).
template <int TILE_LOG2, int TPT, bool PEEL, class Emit>
__device__ __forceinline__ void fine_tile(const FineTile& ft, Emit& emit) {
    constexpr int T = 1 << TILE_LOG2;
    constexpr int NPIX = T * T;
    constexpr int NTHREADS = NPIX < 256 ? NPIX : 256;
    constexpr int PPT = NPIX / NTHREADS;
    constexpr int NBLK = NPIX / 32;  // 8x4 blocks
    constexpr int CHUNK = NTHREADS;  // primitives prepared per pass: one per thread
    constexpr int GROUPS = TPT > 0 ? NTHREADS / TPT : 1;
    __shared__ unsigned long long keys[NPIX];
    __shared__ TilePrim prims[CHUNK];
    __shared__ uint32_t pmask[CHUNK];  // 8x4 blocks each prepared primitive's bbox overlaps
    __shared__ uint32_t pcls[2][CHUNK];  // TPT == 0: [facing class][prim] narrowed block masks
    __shared__ uint32_t pzlo[CHUNK];   // depth_order of a lower bound of the primitive's fragment depths
    __shared__ int n_complex;
    __shared__ int blk_next;           // next 8x4 block a warp takes (TPT == 0)
    __shared__ float col_ndc[T], row_ndc[T];

    const int tx0 = ft.tx0, ty0 = ft.ty0, W = ft.W, H = ft.H;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const unsigned long long* prev_g = PEEL ? ft.prev : nullptr;

    if (TPT > 0) {
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            int dx, dy, bx, by;
            tile_pixel<TILE_LOG2, NTHREADS>(tid, q, dx, dy, bx, by);
            keys[(dy << TILE_LOG2) + dx] = ~0ull;
        }
    }
    if (tid == 0) n_complex = 0;
    if (tid < T) col_ndc[tid] = pixel_ndc(tx0 + tid, W);
    else if (tid < 2 * T) row_ndc[tid - T] = pixel_ndc(ty0 + tid - T, H);

    const bool overflow = ft.overflow;
    const long long pbase = ft.scan_base;
    const long long total = overflow ? ft.scan_count : (long long)ft.cnt;
    const int4* recs = ft.recs;
    if (overflow && tid == 0 && ft.stats) atomicOr(ft.stats + 2, DRP_DEVERR_LIST_OVERFLOW);
    __syncthreads();

    if (TPT == 0 && total == 0) {
        // no primitive meets the tile: every pixel is background
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            int dx, dy, bx, by;
            tile_pixel<TILE_LOG2, NTHREADS>(tid, q, dx, dy, bx, by);
            const int px = tx0 + dx, py = ty0 + dy;
            if (px < W && py < H) emit(px, py, ~0ull, col_ndc[dx], row_ndc[dy]);
        }
        return;
    }

    for (long long base = 0; base < total; base += CHUNK) {
        const int n = (int)min((long long)CHUNK, total - base);
        const bool last_chunk = base + CHUNK >= total;
        if (tid < n && tid < CHUNK) {
            const long long pidx = overflow ? pbase + base + tid : (long long)ft.list[base + tid];
            TilePrim& tp = prims[tid];
            prepare_tile_prim<T>(recs + pidx * 3, tx0, ty0, W, H, tp);
            const int fl = tp.e2.y;
            if (fl & TP_COMPLEX) atomicAdd(&n_complex, 1);
            pmask[tid] = (fl & TP_ACTIVE) ? block_mask<T>(tp.v2b.z & 0xffff, tp.v2b.z >> 16, tp.v2b.w & 0xffff,
                                                          tp.v2b.w >> 16)
                                          : 0u;
            if (TPT == 0 && (fl & TP_ACTIVE)) pzlo[tid] = depth_order(prim_depth_lower_bound(tp));
        }
        if (tid == 0) blk_next = 0;
        __syncthreads();
        if (TPT == 0) {
            refine_block_masks<T, NTHREADS>(prims, pmask, pcls, n);
            __syncthreads();
            // Facing class holding the nearest primitive (every warp computes
            // the same answer).
            uint32_t zmin0 = 0xffffffffu, zmin1 = 0xffffffffu;
            for (int j = lane; j < n; j += 32) {
                if (pcls[0][j]) zmin0 = min(zmin0, pzlo[j]);
                if (pcls[1][j]) zmin1 = min(zmin1, pzlo[j]);
            }
            const int first = __reduce_min_sync(0xffffffffu, zmin0) <= __reduce_min_sync(0xffffffffu, zmin1) ? 0 : 1;
            // keys are final at the end of this chunk unless a clipped
            // primitive still has to be rasterised (second pass below)
            const bool final_keys = last_chunk && n_complex == 0;
            for (;;) {
                int b = 0;
                if (lane == 0) b = atomicAdd(&blk_next, 1);
                b = __shfl_sync(0xffffffffu, b, 0);
                if (b >= NBLK) break;
                const int dx = (b % (T / 8)) * 8 + (lane & 7);
                const int dy = (b / (T / 8)) * 4 + (lane >> 3);
                const int px = tx0 + dx, py = ty0 + dy;
                const int sx = px * DRP_SUBPIX + DRP_HALF_SUBPIX, sy = py * DRP_SUBPIX + DRP_HALF_SUBPIX;
                const int li = (dy << TILE_LOG2) + dx;
                unsigned long long best = base == 0 ? ~0ull : keys[li];
                unsigned long long pk = 0;
                if (prev_g) pk = (px < W && py < H) ? prev_g[py * W + px] : ~0ull;
                const uint32_t bit = 1u << b;
                for (int pass = 0; pass < 2; ++pass) {
                    const int want = pass == 0 ? first : 1 - first;
                    // The other class is skipped wherever its depth lower
                    // bound lies behind every key the block already holds
                    // (such a primitive cannot win a pixel: exact).
                    const uint32_t bmax =
                        pass == 0 ? 0xffffffffu : __reduce_max_sync(0xffffffffu, (uint32_t)(best >> 32));
                    for (int j0 = 0; j0 < n; j0 += 32) {
                        const int j = j0 + lane;
                        const bool meets = j < n && (pcls[want][j] & bit) && pzlo[j] <= bmax;
                        uint32_t hits = __ballot_sync(0xffffffffu, meets);
                        while (hits) {
                            const int h = __ffs(hits) - 1;
                            hits &= hits - 1;
                            const TilePrim& tp = prims[j0 + h];
                            const int4 e0 = tp.e0, e1 = tp.e1, e2 = tp.e2;
                            if (!tile_prim_covers(tp, e0, e1, e2, dx, dy, sx, sy)) continue;
                            bool ok;
                            const unsigned long long k = tile_prim_key(tp.z, e2.z, e2.w, sx, sy, ok);
                            if (ok && k < best && (!prev_g || k > pk)) best = k;
                        }
                    }
                }
                if (final_keys) {
                    if (px < W && py < H) emit(px, py, best, col_ndc[dx], row_ndc[dy]);
                } else {
                    keys[li] = best;
                }
            }
        } else {
            constexpr int G = TPT > 0 ? TPT : 1;
            const int rank = tid % G;
            for (int j = tid / G; j < n; j += GROUPS) {
                const TilePrim& tp = prims[j];
                const int4 e2 = tp.e2;
                if (!(e2.y & TP_ACTIVE)) continue;
                const int4 e0 = tp.e0, e1 = tp.e1, v2b = tp.v2b;
                const int x0 = v2b.z & 0xffff, x1 = v2b.z >> 16, y0 = v2b.w & 0xffff, y1 = v2b.w >> 16;
                for (int dy = y0; dy <= y1; ++dy) {
                    for (int dx = x0 + rank; dx <= x1; dx += G) {
                        const int sx = (tx0 + dx) * DRP_SUBPIX + DRP_HALF_SUBPIX;
                        const int sy = (ty0 + dy) * DRP_SUBPIX + DRP_HALF_SUBPIX;
                        if (!tile_prim_covers(tp, e0, e1, e2, dx, dy, sx, sy)) continue;
                        bool ok;
                        const unsigned long long k = tile_prim_key(tp.z, e2.z, e2.w, sx, sy, ok);
                        if (!ok) continue;
                        const int li = (dy << TILE_LOG2) + dx;
                        if (prev_g && !(k > prev_g[(ty0 + dy) * W + tx0 + dx])) continue;
                        if (k < keys[li]) atomicMin(keys + li, k);
                    }
                }
            }
        }
        __syncthreads();
    }
    if (TPT == 0 && n_complex == 0) return;  // every block was emitted in the last chunk
    if (n_complex > 0) {
        // Clipped polygons (rare): second pass over the list, group-parallel.
        __shared__ unsigned long long prev_s[NPIX];
        if (prev_g) {
#pragma unroll
            for (int q = 0; q < PPT; ++q) {
                int dx, dy, bx, by;
                tile_pixel<TILE_LOG2, NTHREADS>(tid, q, dx, dy, bx, by);
                const int px = tx0 + dx, py = ty0 + dy;
                prev_s[(dy << TILE_LOG2) + dx] = (px < W && py < H) ? prev_g[py * W + px] : ~0ull;
            }
        }
        __syncthreads();
        constexpr int CG = 8;
        for (long long j = tid / CG; j < total; j += NTHREADS / CG) {
            const long long pidx = overflow ? pbase + j : (long long)ft.list[j];
            const int4 r1 = recs[pidx * 3 + 1], r2 = recs[pidx * 3 + 2];
            const PrimBox bx = unpack_box(r1, r2);
            if (!bx.complex_ || bx.px0 > bx.px1 || bx.px1 < tx0 || bx.px0 >= tx0 + T || bx.py1 < ty0 ||
                bx.py0 >= ty0 + T)
                continue;
            raster_complex_tile<TILE_LOG2>(ft.P, ft.tri, W, H, (uint32_t)r1.z, tx0, ty0, tid % CG, CG, keys,
                                           prev_g ? prev_s : nullptr);
        }
        __syncthreads();
    }

    // Emit.
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        int dx, dy, bx, by;
        tile_pixel<TILE_LOG2, NTHREADS>(tid, q, dx, dy, bx, by);
        const int px = tx0 + dx, py = ty0 + dy;
        if (px >= W || py >= H) continue;
        emit(px, py, keys[(dy << TILE_LOG2) + dx], col_ndc[dx], row_ndc[dy]);
    }
}

// ---------------------------------------------------------------------------
// Exclusive scan of per-tile list counts -> offsets (and cursors), total
// entries -> stats (u64).  Chunks of kScanChunk tiles: one block per chunk,
// 16 contiguous tiles per thread.  More than one chunk takes two launches:
// chunk sums, then each block adds the sums of the chunks before it (at most
// a few hundred values) and scans its own chunk.  No inter-block waiting.
// ---------------------------------------------------------------------------

// Block-wide inclusive scan of one u64 per thread (kScanThreads threads).
__device__ inline unsigned long long scan_block_u64(unsigned long long x, unsigned long long* warp_sums,
                                                    unsigned long long& block_total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long v = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int off = 1; off < kScanThreads / 32; off <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, v, off);
            if (lane >= off) v += y;
        }
        if (lane < kScanThreads / 32) warp_sums[lane] = v;
    }
    __syncthreads();
    block_total = warp_sums[kScanThreads / 32 - 1];
    return (warp ? warp_sums[warp - 1] : 0) + x;
}

static __global__ void __launch_bounds__(kScanThreads) scan_chunk_sums_kernel(const uint32_t* counts, long long n,
                                                                              unsigned long long* sums) {
    __shared__ unsigned long long red[kScanThreads / 32];
    const long long base = (long long)blockIdx.x * kScanChunk;
    unsigned long long s = 0;
#pragma unroll
    for (int k = 0; k < kScanPerThread; ++k) {
        const long long i = base + (long long)k * kScanThreads + threadIdx.x;
        if (i < n) s += counts[i];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
#pragma unroll
        for (int w = 0; w < kScanThreads / 32; ++w) t += red[w];
        sums[blockIdx.x] = t;
    }
}

// counts / offsets / cursors must be 16-byte aligned (workspace carve).
static __global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(const uint32_t* counts, uint32_t* offsets,
                                                                         uint32_t* cursors, long long n,
                                                                         const unsigned long long* chunk_sums,
                                                                         unsigned long long* total) {
    __shared__ unsigned long long warp_sums[kScanThreads / 32];
    __shared__ unsigned long long prefix_sh;
    const long long b = blockIdx.x;
    // Sum of the chunks before this one (fixed order per thread, then a tree).
    unsigned long long p = 0;
    for (long long j = threadIdx.x; j < b; j += kScanThreads) p += chunk_sums[j];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) p += __shfl_xor_sync(0xffffffffu, p, off);
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = p;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
#pragma unroll
        for (int w = 0; w < kScanThreads / 32; ++w) t += warp_sums[w];
        prefix_sh = t;
    }
    __syncthreads();
    const unsigned long long prefix = prefix_sh;

    const long long lo = b * kScanChunk + (long long)threadIdx.x * kScanPerThread;
    const bool full = lo + kScanPerThread <= n;
    uint32_t c[kScanPerThread];
    if (full) {
        const uint4* src = reinterpret_cast<const uint4*>(counts + lo);
#pragma unroll
        for (int k = 0; k < kScanPerThread / 4; ++k) {
            const uint4 v = src[k];
            c[4 * k] = v.x;
            c[4 * k + 1] = v.y;
            c[4 * k + 2] = v.z;
            c[4 * k + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanPerThread; ++k) c[k] = lo + k < n ? counts[lo + k] : 0u;
    }
    unsigned long long s = 0;
#pragma unroll
    for (int k = 0; k < kScanPerThread; ++k) s += c[k];
    unsigned long long chunk_total;
    __syncthreads();  // warp_sums reuse
    unsigned long long run = prefix + scan_block_u64(s, warp_sums, chunk_total) - s;
    uint32_t o[kScanPerThread];
#pragma unroll
    for (int k = 0; k < kScanPerThread; ++k) {
        o[k] = (uint32_t)min(run, (unsigned long long)0xffffffffu);
        run += c[k];
    }
    if (full) {
        uint4* d0 = reinterpret_cast<uint4*>(offsets + lo);
        uint4* d1 = reinterpret_cast<uint4*>(cursors + lo);
#pragma unroll
        for (int k = 0; k < kScanPerThread / 4; ++k) {
            const uint4 v = make_uint4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
            d0[k] = v;
            d1[k] = v;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanPerThread; ++k)
            if (lo + k < n) {
                offsets[lo + k] = o[k];
                cursors[lo + k] = o[k];
            }
    }
    if (b == gridDim.x - 1 && threadIdx.x == 0) *total = prefix + chunk_total;
    // largest tile count -> stats word 3 (words 0..1 hold the total, 2 the
    // device error bits); it sizes fixed-depth bins
    uint32_t mx = 0;
#pragma unroll
    for (int k = 0; k < kScanPerThread; ++k) mx = max(mx, c[k]);
    mx = __reduce_max_sync(0xffffffffu, mx);
    if ((threadIdx.x & 31) == 0 && mx) atomicMax(reinterpret_cast<uint32_t*>(total) + 3, mx);
}

// chunk_sums: scan_chunks(n) u64 of scratch (unused when n <= kScanChunk).
static inline void launch_tile_scan(const uint32_t* counts, uint32_t* offsets, uint32_t* cursors, long long n,
                                    unsigned long long* chunk_sums, unsigned long long* total, cudaStream_t s) {
    const long long chunks = scan_chunks(n);
    if (chunks <= 0) return;
    if (chunks > 1) {
        scan_chunk_sums_kernel<<<(unsigned)chunks, kScanThreads, 0, s>>>(counts, n, chunk_sums);
        drp_note_launch();
    }
    scan_tiles_kernel<<<(unsigned)chunks, kScanThreads, 0, s>>>(counts, offsets, cursors, n, chunk_sums, total);
    drp_note_launch();
}

// Fine-raster work order: the n tiles by decreasing list length (counting
// sort on min(count, 1023), ties in any order), so the longest tiles start
// first and the short ones fill in behind them (longest-processing-time-first
// list scheduling; with about one tile per resident CTA the tail otherwise
// waits on whichever long tiles were handed out last).  Any permutation gives
// the same raster: tiles are independent.  One CTA; meant for launches of a
// few tiles per resident fine CTA.
constexpr int kOrderThreads = 1024;
static __global__ void __launch_bounds__(kOrderThreads) tile_order_kernel(const uint32_t* __restrict__ counts, long long n,
                                                                          uint32_t* __restrict__ order) {
    __shared__ uint32_t start[kOrderThreads];  // bucket k holds tiles of count 1023 - k (1023: or more)
    __shared__ uint32_t warp_tot[kOrderThreads / 32];
    pdl_wait();
    pdl_launch_dependents();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    start[tid] = 0;
    __syncthreads();
    for (long long t = tid; t < n; t += kOrderThreads) atomicAdd(&start[1023 - min(counts[t], 1023u)], 1u);
    __syncthreads();
    const uint32_t v = start[tid];
    uint32_t x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_tot[lane];
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += y;
        }
        warp_tot[lane] = w;
    }
    __syncthreads();
    start[tid] = x - v + (warp > 0 ? warp_tot[warp - 1] : 0u);
    __syncthreads();
    for (long long t = tid; t < n; t += kOrderThreads)
        order[atomicAdd(&start[1023 - min(counts[t], 1023u)], 1u)] = (uint32_t)t;
}

static inline void launch_tile_order(const uint32_t* counts, long long n, uint32_t* order, cudaStream_t s) {
    launch_pdl(tile_order_kernel, dim3(1), dim3(kOrderThreads), s, counts, n, order);
    drp_note_launch();
}

}  // namespace drp
