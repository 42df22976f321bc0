// raster.cu -- forward rasterisation (setup, tile binning, fine raster + shade)
// and the rasterisation backward pass (d(u, v, z/w, rast_db) / d clip pos).
//
// Replaces dr.DepthPeeler(...).rasterize_next_layer() / dr.rasterize as called
// at diffrp/rendering/surface_deferred.py:260-262.
//
// Pipeline for one call (all views at once):
//   1. setup_count  -- one thread per (view, triangle): trivial reject,
//      near/guard clipping, fixed-point snap (8 sub-pixel bits), depth plane,
//      pixel bbox; writes a 48-byte primitive record and counts the screen
//      tiles it overlaps (warp-aggregated atomics via __match_any_sync).
//   2. scan_tiles   -- exclusive scan of the per-tile counts (one CTA).
//   3. fill_tiles   -- appends primitive ids to tile lists (warp-aggregated
//      cursors: one atomic per group of lanes hitting the same tile, ranks from
//      __popc of the peer ballot).
//   4. fine_raster  -- one CTA per tile: 64-bit (ordered z/w << 32 | tri)
//      keys resolved with shared-memory atomicMin, then each thread shades its
//      pixel(s) from the winning triangle's clip vertices and writes rast,
//      rast_db and (optionally) the keys for depth peeling.  Tiles whose list
//      overflowed the caller's capacity scan the whole view's primitives
//      instead, so the result never depends on the capacity.
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

struct ViewRange {
    int first, count;
};

__device__ __forceinline__ ViewRange view_range(const int* ranges, int b, int F) {
    ViewRange r;
    if (ranges) {
        r.first = ranges[2 * b];
        r.count = ranges[2 * b + 1];
    } else {
        r.first = 0;
        r.count = F;
    }
    return r;
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

template <int TILE_LOG2>
__global__ void __launch_bounds__(256) setup_count_kernel(RasterArgs a) {
    const int b = blockIdx.y;
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.max_view_tris) return;
    const ViewRange vr = view_range(a.ranges, b, (int)a.num_triangles);
    int4* rec = reinterpret_cast<int4*>(a.ws.prims) + ((long long)b * a.max_view_tris + j) * 3;
    int4 r0 = make_int4(0, 0, 0, 0), r1 = make_int4(0, 0, 0, 1), r2 = make_int4(0, 0, 0, 0);
    int px0 = 1, px1 = 0, py0 = 0, py1 = 0;
    bool live = false;
    if (j < vr.count) {
        const long long t = (long long)vr.first + j;
        const int i0 = a.tri[3 * t], i1 = a.tri[3 * t + 1], i2 = a.tri[3 * t + 2];
        if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= a.num_vertices || i1 >= a.num_vertices || i2 >= a.num_vertices) {
            atomicOr(a.ws.stats + 2, DRP_DEVERR_BAD_INDEX);
        } else {
            const float4* P = reinterpret_cast<const float4*>(a.pos + (long long)b * a.pos_view_stride);
            const float4 p0 = P[i0], p1 = P[i1], p2 = P[i2];
            const int kind = needs_clip_or_cull(p0, p1, p2);
            int64_t mnx = 0, mxx = -1, mny = 0, mxy = -1;
            bool ok = false;
            if (kind == 1) {
                const int32_t X0 = snap_coord(p0.x, p0.w, a.W), Y0 = snap_coord(p0.y, p0.w, a.H);
                const int32_t X1 = snap_coord(p1.x, p1.w, a.W), Y1 = snap_coord(p1.y, p1.w, a.H);
                const int32_t X2 = snap_coord(p2.x, p2.w, a.W), Y2 = snap_coord(p2.y, p2.w, a.H);
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
                setup_clipped(p0, p1, p2, a.W, a.H, poly);
                if (poly.n >= 3) {
                    mnx = mxx = poly.X[0];
                    mny = mxy = poly.Y[0];
                    for (int i = 1; i < poly.n; ++i) {
                        mnx = min(mnx, (int64_t)poly.X[i]);
                        mxx = max(mxx, (int64_t)poly.X[i]);
                        mny = min(mny, (int64_t)poly.Y[i]);
                        mxy = max(mxy, (int64_t)poly.Y[i]);
                    }
                    r1 = make_int4(0, 0, (int)t, 0);
                    ok = true;
                }
            }
            if (ok) {
                int64_t x0 = ceil_shift(mnx - DRP_HALF_SUBPIX), x1 = floor_shift(mxx - DRP_HALF_SUBPIX);
                int64_t y0 = ceil_shift(mny - DRP_HALF_SUBPIX), y1 = floor_shift(mxy - DRP_HALF_SUBPIX);
                x0 = max(x0, (int64_t)0);
                x1 = min(x1, (int64_t)(a.W - 1));
                y0 = max(y0, (int64_t)0);
                y1 = min(y1, (int64_t)(a.H - 1));
                if (x0 <= x1 && y0 <= y1) {
                    px0 = (int)x0;
                    px1 = (int)x1;
                    py0 = (int)y0;
                    py1 = (int)y1;
                    live = true;
                    r2.w = (int)((uint32_t)py0 | ((uint32_t)py1 << 16) | (kind == 2 ? PRIM_COMPLEX : 0u));
                }
            }
        }
    }
    if (!live) {
        px0 = 1;
        px1 = 0;
        r2.w = 0;
    }
    r1.w = (int)((uint32_t)px0 | ((uint32_t)px1 << 16));
    rec[0] = r0;
    rec[1] = r1;
    rec[2] = r2;

    // Count overlapped tiles.
    const int tiles_x = (a.W + (1 << TILE_LOG2) - 1) >> TILE_LOG2;
    const int tiles_y = (a.H + (1 << TILE_LOG2) - 1) >> TILE_LOG2;
    uint32_t* counts = a.ws.tile_count + (long long)b * tiles_x * tiles_y;
    int tx0 = px0 >> TILE_LOG2, tx1 = px1 >> TILE_LOG2, ty0 = py0 >> TILE_LOG2, ty1 = py1 >> TILE_LOG2;
    int n = live ? (tx1 - tx0 + 1) * (ty1 - ty0 + 1) : 0;
    int w = tx1 - tx0 + 1;
    for (int i = 0;; ++i) {
        unsigned active = __ballot_sync(__activemask(), i < n);
        if (i >= n) break;
        uint32_t tile = (uint32_t)((ty0 + i / w) * tiles_x + tx0 + i % w);
        warp_agg_inc(counts, tile, active);
    }
}

// Exclusive scan of tile counts -> offsets (and cursors); total entries -> stats.
__global__ void __launch_bounds__(1024) scan_tiles_kernel(const uint32_t* counts, uint32_t* offsets,
                                                          uint32_t* cursors, long long n,
                                                          unsigned long long* total) {
    __shared__ unsigned long long warp_sums[32];
    const int tid = threadIdx.x;
    const long long per = (n + blockDim.x - 1) / blockDim.x;
    const long long lo = min(n, per * tid), hi = min(n, lo + per);
    unsigned long long s = 0;
    for (long long i = lo; i < hi; ++i) s += counts[i];
    // block exclusive scan of s
    unsigned long long x = s;
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        unsigned long long y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long v = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, v, off);
            if (lane >= off) v += y;
        }
        warp_sums[lane] = v;
    }
    __syncthreads();
    unsigned long long base = (warp ? warp_sums[warp - 1] : 0) + x - s;
    for (long long i = lo; i < hi; ++i) {
        uint32_t o = (uint32_t)min(base, (unsigned long long)0xffffffffu);
        offsets[i] = o;
        cursors[i] = o;
        base += counts[i];
    }
    if (tid == blockDim.x - 1) *total = base;
}

template <int TILE_LOG2>
__global__ void __launch_bounds__(256) fill_tiles_kernel(RasterArgs a) {
    const int b = blockIdx.y;
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.max_view_tris) return;
    const long long pidx = (long long)b * a.max_view_tris + j;
    const int4* rec = reinterpret_cast<const int4*>(a.ws.prims) + pidx * 3;
    const PrimBox bx = unpack_box(rec[1], rec[2]);
    const int tiles_x = (a.W + (1 << TILE_LOG2) - 1) >> TILE_LOG2;
    const int tiles_y = (a.H + (1 << TILE_LOG2) - 1) >> TILE_LOG2;
    uint32_t* cursors = a.ws.tile_cursor + (long long)b * tiles_x * tiles_y;
    const bool live = bx.px0 <= bx.px1;
    int tx0 = bx.px0 >> TILE_LOG2, tx1 = bx.px1 >> TILE_LOG2, ty0 = bx.py0 >> TILE_LOG2, ty1 = bx.py1 >> TILE_LOG2;
    int n = live ? (tx1 - tx0 + 1) * (ty1 - ty0 + 1) : 0;
    int w = tx1 - tx0 + 1;
    for (int i = 0;; ++i) {
        unsigned active = __ballot_sync(__activemask(), i < n);
        if (i >= n) break;
        uint32_t tile = (uint32_t)((ty0 + i / w) * tiles_x + tx0 + i % w);
        uint32_t slot = warp_agg_inc(cursors, tile, active);
        if (slot < a.list_capacity) a.ws.tile_list[slot] = (uint32_t)pidx;
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
__device__ __noinline__ void raster_complex_tile(const RasterArgs& a, int b, uint32_t tri, int tx0, int ty0,
                                                 int rank, int group, unsigned long long* keys,
                                                 const unsigned long long* prev) {
    const float4* P = reinterpret_cast<const float4*>(a.pos + (long long)b * a.pos_view_stride);
    const int i0 = a.tri[3 * (long long)tri], i1 = a.tri[3 * (long long)tri + 1], i2 = a.tri[3 * (long long)tri + 2];
    Poly poly;
    setup_clipped(P[i0], P[i1], P[i2], a.W, a.H, poly);
    for (int i = 1; i + 1 < poly.n; ++i) {
        const int64_t X0 = poly.X[0], Y0 = poly.Y[0], X1 = poly.X[i], Y1 = poly.Y[i];
        const int64_t X2 = poly.X[i + 1], Y2 = poly.Y[i + 1];
        const int64_t area2 = (X1 - X0) * (Y2 - Y0) - (Y1 - Y0) * (X2 - X0);
        if (area2 == 0) continue;
        const Plane pl = depth_plane(X0, Y0, poly.Z[0], X1, Y1, poly.Z[i], X2, Y2, poly.Z[i + 1], area2);
        raster_subtri_tile<TILE_LOG2>(X0, Y0, X1, Y1, X2, Y2, pl, tri, tx0, ty0, a.W, a.H, rank, group, keys, prev);
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
    tp.e2 = make_int4(C[2], TP_ACTIVE | (big ? TP_BIG : 0), (int)X0, (int)Y0);
    tp.z.x = __int_as_float(r2.x);
    tp.z.y = __int_as_float(r2.y);
    tp.z.z = __int_as_float(r2.z);
    tp.v01 = make_int4((int)vx[0], (int)vy[0], (int)vx[1], (int)vy[1]);
    tp.v2b.x = (int)vx[2];
    tp.v2b.y = (int)vy[2];
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

// Pixel q of thread tid inside a tile: warps own 8x4 pixel blocks (blocks
// are numbered across the tile, then down), lanes are row-major inside the
// block.  A warp can then skip a primitive whose bbox misses its block with
// one uniform test.
template <int TILE_LOG2, int NTHREADS>
__device__ __forceinline__ void tile_pixel(int tid, int q, int& dx, int& dy, int& bx, int& by) {
    constexpr int T = 1 << TILE_LOG2;
    const int blk = (tid >> 5) + q * (NTHREADS >> 5);
    bx = (blk % (T / 8)) * 8;
    by = (blk / (T / 8)) * 4;
    dx = bx + (tid & 7);
    dy = by + ((tid >> 3) & 3);
}

// Fine raster + shade, one CTA per (tile, view).
//   TPT == 0: every thread owns T*T/NTHREADS pixels and tests them against
//             each primitive of the tile (keys in registers, no atomics);
//   TPT  > 0: groups of TPT threads walk one primitive's bbox within the tile
//             and resolve keys with shared-memory atomicMin.
template <int TILE_LOG2, int TPT>
__global__ void __launch_bounds__((1 << (2 * TILE_LOG2)) < 256 ? (1 << (2 * TILE_LOG2)) : 256,
                                  TILE_LOG2 == 3 ? 12 : 3)
fine_raster_kernel(RasterArgs a) {
    constexpr int T = 1 << TILE_LOG2;
    constexpr int NPIX = T * T;
    constexpr int NTHREADS = NPIX < 256 ? NPIX : 256;
    constexpr int PPT = NPIX / NTHREADS;
    constexpr int CHUNK = NTHREADS < 128 ? NTHREADS : 128;
    constexpr int GROUPS = TPT > 0 ? NTHREADS / TPT : 1;
    __shared__ unsigned long long keys[NPIX];
    __shared__ TilePrim prims[CHUNK];
    __shared__ int n_complex;
    __shared__ float col_ndc[T], row_ndc[T];

    const int b = blockIdx.y;
    const int tile = blockIdx.x;
    const int tx0 = (tile % a.tiles_x) << TILE_LOG2, ty0 = (tile / a.tiles_x) << TILE_LOG2;
    const int npix_view = a.H * a.W;
    const int tid = threadIdx.x;
    const unsigned long long* prev_g = a.prev_key ? a.prev_key + (long long)b * npix_view : nullptr;

    unsigned long long best[PPT], prevk[PPT];
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        int dx, dy, bx, by;
        tile_pixel<TILE_LOG2, NTHREADS>(tid, q, dx, dy, bx, by);
        const int px = tx0 + dx, py = ty0 + dy;
        best[q] = ~0ull;
        prevk[q] = 0;
        if (prev_g) prevk[q] = (px < a.W && py < a.H) ? prev_g[py * a.W + px] : ~0ull;
        if (TPT > 0) keys[(dy << TILE_LOG2) + dx] = ~0ull;
    }
    if (tid == 0) n_complex = 0;
    if (tid < T) col_ndc[tid] = pixel_ndc(tx0 + tid, a.W);
    else if (tid < 2 * T) row_ndc[tid - T] = pixel_ndc(ty0 + tid - T, a.H);

    const long long tidx = (long long)b * a.tiles_x * a.tiles_y + tile;
    const uint32_t cnt = a.ws.tile_count[tidx];
    const uint32_t off = a.ws.tile_offset[tidx];
    const bool overflow = (unsigned long long)off + cnt > (unsigned long long)a.list_capacity;
    const long long pbase = (long long)b * a.max_view_tris;
    const long long total = overflow ? a.max_view_tris : (long long)cnt;
    const int4* recs = reinterpret_cast<const int4*>(a.ws.prims);
    if (overflow && tid == 0) atomicOr(a.ws.stats + 2, DRP_DEVERR_LIST_OVERFLOW);
    __syncthreads();

    for (long long base = 0; base < total; base += CHUNK) {
        const int n = (int)min((long long)CHUNK, total - base);
        if (tid < n && tid < CHUNK) {
            const long long pidx = overflow ? pbase + base + tid : (long long)a.ws.tile_list[off + base + tid];
            prepare_tile_prim<T>(recs + pidx * 3, tx0, ty0, a.W, a.H, prims[tid]);
            if (prims[tid].e2.y & TP_COMPLEX) atomicAdd(&n_complex, 1);
        }
        __syncthreads();
        if (TPT == 0) {
            for (int j = 0; j < n; ++j) {
                const TilePrim& tp = prims[j];
                const int4 e2 = tp.e2;
                if (!(e2.y & TP_ACTIVE)) continue;
                const int4 e0 = tp.e0, e1 = tp.e1, v2b = tp.v2b;
                const int x0 = v2b.z & 0xffff, x1 = v2b.z >> 16, y0 = v2b.w & 0xffff, y1 = v2b.w >> 16;
#pragma unroll
                for (int q = 0; q < PPT; ++q) {
                    int dx, dy, bx, by;
                    tile_pixel<TILE_LOG2, NTHREADS>(tid, q, dx, dy, bx, by);
                    if (x1 < bx || x0 > bx + 7 || y1 < by || y0 > by + 3) continue;  // warp-uniform
                    const int sx = (tx0 + dx) * DRP_SUBPIX + DRP_HALF_SUBPIX;
                    const int sy = (ty0 + dy) * DRP_SUBPIX + DRP_HALF_SUBPIX;
                    if (!tile_prim_covers(tp, e0, e1, e2, dx, dy, sx, sy)) continue;
                    bool ok;
                    const unsigned long long k = tile_prim_key(tp.z, e2.z, e2.w, sx, sy, ok);
                    if (ok && k < best[q] && (!prev_g || k > prevk[q])) best[q] = k;
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
                        if (prev_g && !(k > prev_g[(ty0 + dy) * a.W + tx0 + dx])) continue;
                        if (k < keys[li]) atomicMin(keys + li, k);
                    }
                }
            }
        }
        __syncthreads();
    }
    if (TPT == 0) {
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            int dx, dy, bx, by;
            tile_pixel<TILE_LOG2, NTHREADS>(tid, q, dx, dy, bx, by);
            keys[(dy << TILE_LOG2) + dx] = best[q];
        }
    }
    __syncthreads();
    if (n_complex > 0) {
        // Clipped polygons (rare): second pass over the list, group-parallel.
        __shared__ unsigned long long prev_s[NPIX];
        if (prev_g) {
#pragma unroll
            for (int q = 0; q < PPT; ++q) {
                int dx, dy, bx, by;
                tile_pixel<TILE_LOG2, NTHREADS>(tid, q, dx, dy, bx, by);
                prev_s[(dy << TILE_LOG2) + dx] = prevk[q];
            }
        }
        __syncthreads();
        constexpr int CG = 8;
        for (long long j = tid / CG; j < total; j += NTHREADS / CG) {
            const long long pidx = overflow ? pbase + j : (long long)a.ws.tile_list[off + j];
            const int4 r1 = recs[pidx * 3 + 1], r2 = recs[pidx * 3 + 2];
            const PrimBox bx = unpack_box(r1, r2);
            if (!bx.complex_ || bx.px0 > bx.px1 || bx.px1 < tx0 || bx.px0 >= tx0 + T || bx.py1 < ty0 ||
                bx.py0 >= ty0 + T)
                continue;
            raster_complex_tile<TILE_LOG2>(a, b, (uint32_t)r1.z, tx0, ty0, tid % CG, CG, keys,
                                           prev_g ? prev_s : nullptr);
        }
        __syncthreads();
    }

    // Shade.
    const float4* P = reinterpret_cast<const float4*>(a.pos + (long long)b * a.pos_view_stride);
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        int dx, dy, bx, by;
        tile_pixel<TILE_LOG2, NTHREADS>(tid, q, dx, dy, bx, by);
        const int i = (dy << TILE_LOG2) + dx;
        const int px = tx0 + dx, py = ty0 + dy;
        if (px >= a.W || py >= a.H) continue;
        const long long o = (long long)b * npix_view + py * a.W + px;
        const unsigned long long k = keys[i];
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f), d = make_float4(0.f, 0.f, 0.f, 0.f);
        if (k != ~0ull) {
            const int t = (int)(uint32_t)(k & 0xffffffffu);
            const int i0 = a.tri[3 * (long long)t], i1 = a.tri[3 * (long long)t + 1], i2 = a.tri[3 * (long long)t + 2];
            const float4 p0 = P[i0], p1 = P[i1], p2 = P[i2];
            Shade S;
            shade_eval_xy(p0, p1, p2, col_ndc[i & (T - 1)], row_ndc[i >> TILE_LOG2], a.W, a.H, S);
            r = make_float4(S.u, S.v, S.zw, enc_triid(t + 1));
            if (a.rast_db) d = shade_db(S);
        }
        reinterpret_cast<float4*>(a.rast)[o] = r;
        if (a.rast_db) reinterpret_cast<float4*>(a.rast_db)[o] = d;
        if (a.out_key) a.out_key[o] = k;
    }
}

// ---------------------------------------------------------------------------
// Backward: grad_rast (u, v, z/w) [+ grad_db] -> grad_pos (float4 atomics,
// warp-segmented pre-reduction over runs of equal triangle).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) raster_bwd_kernel(RasterBwdArgs a) {
    const long long npix_view = (long long)a.H * a.W;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = i < (long long)a.B * npix_view;
    int t = -1;
    int i0 = 0, i1 = 0, i2 = 0;
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    if (in) {
        r = reinterpret_cast<const float4*>(a.rast)[i];
        t = checked_tri(r.w, a.tri, a.num_triangles, a.num_vertices, i0, i1, i2);
    }
    const int b = in ? (int)(i / npix_view) : 0;
    float v[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) v[k] = 0.f;
    if (t >= 0) {
        const long long pix = i - (long long)b * npix_view;
        const int py = (int)(pix / a.W), px = (int)(pix % a.W);
        const float4* P = reinterpret_cast<const float4*>(a.pos + (long long)b * a.pos_view_stride);
        const float4 p0 = P[i0], p1 = P[i1], p2 = P[i2];
        Shade S;
        shade_eval(p0, p1, p2, px, py, a.W, a.H, S);
        const float4 g = reinterpret_cast<const float4*>(a.grad_rast)[i];
        float4 gdb;
        if (a.grad_db) gdb = reinterpret_cast<const float4*>(a.grad_db)[i];
        float4 out[3];
        shade_grad(p0, p1, p2, S, g.x, g.y, g.z, a.grad_db ? &gdb : nullptr, out);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            v[4 * k + 0] = out[k].x;
            v[4 * k + 1] = out[k].y;
            v[4 * k + 2] = out[k].z;
            v[4 * k + 3] = out[k].w;
        }
    }
    // Segment key: the triangle, plus the view when every view has its own
    // vertices (shared pos sends all views' gradients to the same rows).
    const long long key = (t >= 0) ? (a.pos_view_stride ? (((long long)b << 32) | (long long)t) : (long long)t)
                                   : (long long)(-1 - lane_id());
    const bool head = segmented_sum<12>(key, v);
    if (t >= 0 && head) {
        float4* G = reinterpret_cast<float4*>(a.grad_pos + (long long)b * a.pos_view_stride);
        atomic_add4(G + i0, make_float4(v[0], v[1], v[2], v[3]));
        atomic_add4(G + i1, make_float4(v[4], v[5], v[6], v[7]));
        atomic_add4(G + i2, make_float4(v[8], v[9], v[10], v[11]));
    }
}

// ---------------------------------------------------------------------------
// Host-side launchers.
// ---------------------------------------------------------------------------
template <int TL>
static void launch_fine(const RasterArgs& a, int tpt, cudaStream_t s) {
    constexpr int NT = (1 << (2 * TL)) < 256 ? (1 << (2 * TL)) : 256;
    dim3 grid((unsigned)(a.tiles_x * a.tiles_y), (unsigned)a.B);
    switch (tpt) {
    case 0: fine_raster_kernel<TL, 0><<<grid, NT, 0, s>>>(a); break;
    case 1: fine_raster_kernel<TL, 1><<<grid, NT, 0, s>>>(a); break;
    case 2: fine_raster_kernel<TL, 2><<<grid, NT, 0, s>>>(a); break;
    case 4: fine_raster_kernel<TL, 4><<<grid, NT, 0, s>>>(a); break;
    case 8: fine_raster_kernel<TL, 8><<<grid, NT, 0, s>>>(a); break;
    case 16: fine_raster_kernel<TL, 16><<<grid, NT, 0, s>>>(a); break;
    default: fine_raster_kernel<TL, 32><<<grid, NT, 0, s>>>(a); break;
    }
}

template <int TL>
static void launch_bin(const RasterArgs& a, cudaStream_t s) {
    dim3 grid((unsigned)((a.max_view_tris + 255) / 256), (unsigned)a.B);
    setup_count_kernel<TL><<<grid, 256, 0, s>>>(a);
    const long long n = (long long)a.B * a.tiles_x * a.tiles_y;
    scan_tiles_kernel<<<1, 1024, 0, s>>>(a.ws.tile_count, a.ws.tile_offset, a.ws.tile_cursor, n,
                                         reinterpret_cast<unsigned long long*>(a.ws.stats));
    fill_tiles_kernel<TL><<<grid, 256, 0, s>>>(a);
}

int launch_rasterize(const RasterArgs& a, cudaStream_t s) {
    const long long ntiles = (long long)a.B * a.tiles_x * a.tiles_y;
    cudaMemsetAsync(a.ws.tile_count, 0, sizeof(uint32_t) * ntiles, s);
    cudaMemsetAsync(a.ws.stats, 0, sizeof(uint32_t) * 4, s);
    if (a.max_view_tris > 0) {
        switch (a.tile_log2) {
        case 3: launch_bin<3>(a, s); break;
        case 5: launch_bin<5>(a, s); break;
        default: launch_bin<4>(a, s); break;
        }
    } else {
        cudaMemsetAsync(a.ws.tile_offset, 0, sizeof(uint32_t) * ntiles, s);
    }
    switch (a.tile_log2) {
    case 3: launch_fine<3>(a, a.threads_per_tri, s); break;
    case 5: launch_fine<5>(a, a.threads_per_tri, s); break;
    default: launch_fine<4>(a, a.threads_per_tri, s); break;
    }
    return 0;
}

int launch_raster_bwd(const RasterBwdArgs& a, cudaStream_t s) {
    const long long n = (long long)a.B * a.H * a.W;
    if (n == 0) return 0;
    raster_bwd_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    return 0;
}

}  // namespace drp
