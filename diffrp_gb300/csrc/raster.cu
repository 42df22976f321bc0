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
#include "drp_internal.h"
#include "raster_core.cuh"

namespace drp {

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

// One thread per (view, triangle slot): build the primitive record, then
// count (kSetupCount) or list (kSetupFill, after the scan; it re-reads the
// record written by the count pass) the tiles it overlaps, or both at once
// into fixed-depth bins (kSetupBins).
constexpr int kSetupCount = 0, kSetupFill = 1, kSetupBins = 2;

template <int TILE_LOG2, int MODE>
__global__ void __launch_bounds__(256) setup_bin_kernel(RasterArgs a) {
    constexpr bool FILL = MODE == kSetupFill;
    const int b = blockIdx.y;
    // every lane stays to the binning (a warp-collective call)
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = j < a.max_view_tris;
    const long long pidx = (long long)b * a.max_view_tris + (in ? j : 0);
    int4* rec = reinterpret_cast<int4*>(a.ws.prims) + pidx * 3;
    PrimBox bx;
    bx.px0 = 1;
    bx.px1 = bx.py0 = bx.py1 = 0;
    bool live = false;
    if (FILL) {
        if (in) {
            bx = unpack_box(rec[1], rec[2]);
            live = bx.px0 <= bx.px1;
        }
    } else if (in) {
        const ViewRange vr = view_range(a.ranges, b, (int)a.num_triangles);
        if (j < vr.count) {
            const long long t = (long long)vr.first + j;
            const int i0 = a.tri[3 * t], i1 = a.tri[3 * t + 1], i2 = a.tri[3 * t + 2];
            if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= a.num_vertices || i1 >= a.num_vertices ||
                i2 >= a.num_vertices) {
                atomicOr(a.ws.stats + 2, DRP_DEVERR_BAD_INDEX);
            } else {
                const float4* P = reinterpret_cast<const float4*>(a.pos + (long long)b * a.pos_view_stride);
                live = build_prim(P[i0], P[i1], P[i2], t, a.W, a.H, rec, bx);
            }
        }
        if (!live) {
            rec[0] = make_int4(0, 0, 0, 0);
            rec[1] = make_int4(0, 0, 0, 1);
            rec[2] = make_int4(0, 0, 0, 0);
        }
    }
    const long long tiles = (long long)a.tiles_x * a.tiles_y;
    if (FILL)
        bin_box<TILE_LOG2>(bx, live, a.tiles_x, a.ws.tile_cursor + b * tiles, a.ws.tile_list, a.list_capacity,
                           (uint32_t)pidx);
    else if (MODE == kSetupBins)
        bin_box<TILE_LOG2>(bx, live, a.tiles_x, a.ws.tile_count + b * tiles,
                           a.ws.tile_list + (unsigned long long)(b * tiles) * a.bin_depth, 0, (uint32_t)pidx,
                           a.bin_depth);
    else
        bin_box<TILE_LOG2>(bx, live, a.tiles_x, a.ws.tile_count + b * tiles, nullptr, 0, 0);
}

// Writes rast (u, v, z/w, id + 1), rast_db and the visibility key of a pixel.
struct RastEmit {
    const float4* P;
    const int* tri;
    int W, H;
    float4* rast;
    float4* db;
    unsigned long long* key;
    __device__ __forceinline__ void operator()(int px, int py, unsigned long long k, float X, float Y) const {
        const long long o = (long long)py * W + px;
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f), d = make_float4(0.f, 0.f, 0.f, 0.f);
        if (k != ~0ull) {
            const int t = (int)(uint32_t)(k & 0xffffffffu);
            const float4 p0 = P[tri[3 * (long long)t]], p1 = P[tri[3 * (long long)t + 1]],
                         p2 = P[tri[3 * (long long)t + 2]];
            Shade S;
            shade_eval_xy(p0, p1, p2, X, Y, W, H, S);
            r = make_float4(S.u, S.v, S.zw, enc_triid(t + 1));
            if (db) d = shade_db(S);
        }
        rast[o] = r;
        if (db) db[o] = d;
        if (key) key[o] = k;
    }
};

// PEEL: a previous layer's keys are given (depth peeling).  Only the
// pixel-parallel shape (TPT = 0) has a separate instantiation without them.
template <int TILE_LOG2, int TPT, bool PEEL>
__global__ void __launch_bounds__((1 << (2 * TILE_LOG2)) < 256 ? (1 << (2 * TILE_LOG2)) : 256,
                                  TILE_LOG2 == 3 ? 12 : 4)
fine_raster_kernel(RasterArgs a) {
    const long long tiles = (long long)a.tiles_x * a.tiles_y;
    long long tidx = (long long)blockIdx.y * tiles + blockIdx.x;  // blocks start in this order
    if (a.tile_order) tidx = a.tile_order[tidx];
    const int b = (int)(tidx / tiles);
    const int tile = (int)(tidx - (long long)b * tiles);
    const long long npix = (long long)a.H * a.W;
    FineTile ft;
    ft.recs = reinterpret_cast<const int4*>(a.ws.prims);
    ft.cnt = a.ws.tile_count[tidx];
    if (a.bin_depth) {
        ft.list = a.ws.tile_list + (unsigned long long)tidx * a.bin_depth;
        ft.overflow = ft.cnt > a.bin_depth;
        if (ft.overflow && threadIdx.x == 0) atomicMax(a.ws.stats + 3, ft.cnt);  // sizes the next depth
    } else {
        const uint32_t off = a.ws.tile_offset[tidx];
        ft.list = a.ws.tile_list + off;
        ft.overflow = (unsigned long long)off + ft.cnt > a.list_capacity;
    }
    ft.scan_base = (long long)b * a.max_view_tris;
    ft.scan_count = a.max_view_tris;
    ft.tx0 = (tile % a.tiles_x) << TILE_LOG2;
    ft.ty0 = (tile / a.tiles_x) << TILE_LOG2;
    ft.W = a.W;
    ft.H = a.H;
    ft.P = reinterpret_cast<const float4*>(a.pos + (long long)b * a.pos_view_stride);
    ft.tri = a.tri;
    ft.prev = a.prev_key ? a.prev_key + b * npix : nullptr;
    ft.stats = a.ws.stats;
    RastEmit e;
    e.P = ft.P;
    e.tri = a.tri;
    e.W = a.W;
    e.H = a.H;
    e.rast = reinterpret_cast<float4*>(a.rast) + b * npix;
    e.db = a.rast_db ? reinterpret_cast<float4*>(a.rast_db) + b * npix : nullptr;
    e.key = a.out_key ? a.out_key + b * npix : nullptr;
    fine_tile<TILE_LOG2, TPT, PEEL>(ft, e);
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
// Up to this many tiles per resident fine CTA the blocks take the tiles in
// order of decreasing list length (tile_order_kernel).
constexpr long long kOrderTilesPerCTA = 8;

template <int TL>
static void launch_fine(const RasterArgs& args, int tpt, cudaStream_t s) {
    constexpr int NT = (1 << (2 * TL)) < 256 ? (1 << (2 * TL)) : 256;
    dim3 grid((unsigned)(args.tiles_x * args.tiles_y), (unsigned)args.B);
    // resident CTAs per SM of the instantiations (launch bounds: 4 above
    // 8-pixel tiles); the fill cursors are spent by now and hold the order
    const long long slots = (long long)drp_current_sm_count() * (TL == 3 ? 12 : 4);
    const long long ntiles = (long long)grid.x * grid.y;
    RasterArgs a = args;
    a.tile_order = nullptr;
    if (a.max_view_tris > 0 && ntiles > slots && ntiles <= kOrderTilesPerCTA * slots) {
        launch_tile_order(a.ws.tile_count, ntiles, a.ws.tile_cursor, s);
        a.tile_order = a.ws.tile_cursor;
    }
    switch (tpt) {
    case 0:
        if (a.prev_key) fine_raster_kernel<TL, 0, true><<<grid, NT, 0, s>>>(a);
        else fine_raster_kernel<TL, 0, false><<<grid, NT, 0, s>>>(a);
        drp_note_launch();
        break;
    case 1: fine_raster_kernel<TL, 1, true><<<grid, NT, 0, s>>>(a); drp_note_launch(); break;
    case 2: fine_raster_kernel<TL, 2, true><<<grid, NT, 0, s>>>(a); drp_note_launch(); break;
    case 4: fine_raster_kernel<TL, 4, true><<<grid, NT, 0, s>>>(a); drp_note_launch(); break;
    case 8: fine_raster_kernel<TL, 8, true><<<grid, NT, 0, s>>>(a); drp_note_launch(); break;
    case 16: fine_raster_kernel<TL, 16, true><<<grid, NT, 0, s>>>(a); drp_note_launch(); break;
    default: fine_raster_kernel<TL, 32, true><<<grid, NT, 0, s>>>(a); drp_note_launch(); break;
    }
}

template <int TL>
static void launch_bin(const RasterArgs& a, cudaStream_t s) {
    dim3 grid((unsigned)((a.max_view_tris + 255) / 256), (unsigned)a.B);
    if (a.bin_depth) {
        setup_bin_kernel<TL, kSetupBins><<<grid, 256, 0, s>>>(a);
        drp_note_launch();
        return;
    }
    setup_bin_kernel<TL, kSetupCount><<<grid, 256, 0, s>>>(a);
    drp_note_launch();
    const long long n = (long long)a.B * a.tiles_x * a.tiles_y;
    launch_tile_scan(a.ws.tile_count, a.ws.tile_offset, a.ws.tile_cursor, n, a.ws.chunk_sums,
                     reinterpret_cast<unsigned long long*>(a.ws.stats), s);
    setup_bin_kernel<TL, kSetupFill><<<grid, 256, 0, s>>>(a);
    drp_note_launch();
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
    drp_note_launch();
    return 0;
}

}  // namespace drp
