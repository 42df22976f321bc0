// batch.cu -- the batching form: many meshes x views x resolutions in one
// set of launches, with raster + interpolation fused and the whole backward
// (antialias, interpolation, rasterisation) fused into one pixel pass.
//
// An item is one (mesh, view, resolution) render: its clip vertices, its
// mesh's triangles and attributes, and its own output image.  All items'
// data live in packed buffers addressed through a device item table
// (drp_batch_item); host-built block maps send every 256-wide block of
// primitives or pixels to one item, so no thread searches for its item.
//
// Forward launches (independent of the number of items):
//   setup/count -> scan -> setup/fill  (tile lists for every item's tiles)
//   fine raster: persistent CTAs pull (item, tile) work from an atomic queue,
//                resolve visibility, write rast and the interpolated colour
//   antialias:   per-triangle records, then the per-pixel silhouette blend
// Backward: per-triangle records, then one fused pixel pass computing the
// antialias colour gradient, the attribute gradient (interpolation backward)
// and the vertex gradient (rasterisation backward), scattered with
// warp-segmented float4 atomics.
#include <atomic>

#include "../../include/diffrp_gb300.h"
#include "aa_core.cuh"
#include "drp_internal.h"
#include "raster_core.cuh"

namespace drp {

struct BatchArgs {
    const drp_batch_item* items;
    int num_items;
    const int2* prim_blocks;  // (item, local block) per 256 triangle slots
    long long n_prim_blocks;
    const int2* pix_blocks;   // (item, local block) per 256 pixels
    long long n_pix_blocks;
    long long total_prims, total_tiles;
    const float* pos;
    const int* tri;
    const float* attr;
    const int* nbr;
    int tile_log2, tpt;
    unsigned long long list_capacity;
    uint32_t bin_depth;  // 0: exact lists (count, scan, fill); > 0: fixed-depth bins (one pass)
    float* rast;
    float* color;
    float* out;
    // antialias state (forward writes, backward reads): per pixel whether a
    // blending pair touches it, and the list of those pixels
    unsigned char* aa_flags;
    int* aa_list;
    unsigned* aa_count;
    bool emit_out;          // the fine raster also writes the colour into out
    bool aa_records;        // the setup pass writes the antialias triangle records
    // fused mean-absolute-error loss (null target: none)
    const float* target;
    float l1_scale;
    float* l1_grad;
    float* block_loss;      // one partial per pixel block
    float* loss;
    bool l1_grads;          // the loss pass also forms the loss's gradient (drp_batch_forward_l1_grad)
    float* zero_first;      // floats zeroed by the forward's first kernel (null: none)
    long long zero_floats;
    const float* grad_scale;  // backward: device scalar multiplying grad_out, or null
    const float* grad_out;
    float* grad_pos;
    float* grad_attr;
    // workspace
    uint32_t* stats;
    uint32_t* queue;
    int4* prims;
    uint32_t *tile_count, *tile_offset, *tile_cursor, *tile_list;
    unsigned long long* chunk_sums;  // tile-scan chunk sums
    float4* aa_rec;
    const uint32_t* tile_order = nullptr;  // fine-raster work order (null: tile index order)
};

// MODE kSetupCount: triangle setup, antialias record, per-tile counts;
// kSetupFill: append to the exact lists (after the scan); kSetupBins: setup,
// record and append to fixed-depth bins in one pass.
constexpr int kSetupCount = 0, kSetupFill = 1, kSetupBins = 2;
// CTAs per 256-triangle block of the map, and triangles per CTA: the work is
// a chain of dependent loads per triangle, so smaller CTAs spread one mesh's
// few hundred map blocks over every SM.
constexpr int kSetupSplit = 4, kSetupTris = 256 / kSetupSplit;

template <int TILE_LOG2, int MODE>
__global__ void __launch_bounds__(2 * kSetupTris) batch_setup_bin_kernel(BatchArgs a) {
    pdl_wait();
    pdl_launch_dependents();
    constexpr bool FILL = MODE == kSetupFill;
    const int2 blk = a.prim_blocks[blockIdx.x / kSetupSplit];
    const drp_batch_item& it = a.items[blk.x];
    const long long j0 = (long long)blk.y * 256 + (blockIdx.x % kSetupSplit) * kSetupTris;
    // Count / bin launches with antialias records use 2 * kSetupTris threads:
    // the upper half writes the records of the CTA's triangles while the
    // lower half sets them up and bins them (two shorter chains of dependent
    // loads instead of one).  Whole warps take one side.
    if (threadIdx.x >= kSetupTris) {
        const long long jr = j0 + (threadIdx.x - kSetupTris);
        if (!FILL && a.aa_records && jr < it.tri_count)
            aa_tri_record(reinterpret_cast<const float4*>(a.pos) + it.pos_offset,
                          a.tri + 3 * (long long)it.tri_first, a.nbr ? a.nbr + 3 * (long long)it.tri_first : nullptr,
                          jr, it.tri_count, it.num_vertices, it.width, it.height,
                          a.aa_rec + (it.prim_offset + jr) * 2);
        return;
    }
    // every lane stays to the binning (a warp-collective call)
    const long long j = j0 + threadIdx.x;
    const bool in = j < it.tri_count;
    const long long pidx = it.prim_offset + (in ? j : 0);
    int4* rec = a.prims + pidx * 3;
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
        const long long t = (long long)it.tri_first + j;
        const int i0 = a.tri[3 * t], i1 = a.tri[3 * t + 1], i2 = a.tri[3 * t + 2];
        if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= it.num_vertices || i1 >= it.num_vertices || i2 >= it.num_vertices) {
            atomicOr(a.stats + 2, DRP_DEVERR_BAD_INDEX);
        } else {
            const float4* P = reinterpret_cast<const float4*>(a.pos) + it.pos_offset;
            live = build_prim(P[i0], P[i1], P[i2], j, it.width, it.height, rec, bx);
        }
        if (!live) {
            rec[0] = make_int4(0, 0, 0, 0);
            rec[1] = make_int4(0, 0, 0, 1);
            rec[2] = make_int4(0, 0, 0, 0);
        }
    }
    if (FILL) {
        bin_box<TILE_LOG2>(bx, live, it.tiles_x, a.tile_cursor + it.tile_offset, a.tile_list, a.list_capacity,
                           (uint32_t)pidx);
    } else {
        if (MODE == kSetupBins)
            bin_box<TILE_LOG2>(bx, live, it.tiles_x, a.tile_count + it.tile_offset,
                               a.tile_list + (unsigned long long)it.tile_offset * a.bin_depth, 0, (uint32_t)pidx,
                               a.bin_depth);
        else
            bin_box<TILE_LOG2>(bx, live, it.tiles_x, a.tile_count + it.tile_offset, nullptr, 0, 0);
    }
}

// rast + interpolated attributes of one pixel (interpolator.py:45 order).
// The colour also goes to out (when not null): the antialias pass then only
// rewrites the pixels it blends.
struct BatchEmit {
    const float4* P;
    const int* tri;  // the item's mesh triangles (local vertex indices)
    const float* A;  // the item's mesh attributes
    int W, H, C;
    bool vec;  // 128-bit attribute / colour / output access: C % 4 == 0 and all bases 16-byte aligned
    float4* rast;
    float* color;
    float* out;
    __device__ __forceinline__ void operator()(int px, int py, unsigned long long k, float X, float Y) const {
        const long long o = (long long)py * W + px;
        float* col = color + o * C;
        float* oc = out ? out + o * C : nullptr;
        if (k == ~0ull) {
            rast[o] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (vec) {
                for (int c = 0; c < C; c += 4) {
                    *reinterpret_cast<float4*>(col + c) = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (oc) *reinterpret_cast<float4*>(oc + c) = make_float4(0.f, 0.f, 0.f, 0.f);
                }
            } else {
                for (int c = 0; c < C; ++c) {
                    col[c] = 0.f;
                    if (oc) oc[c] = 0.f;
                }
            }
            return;
        }
        const int t = (int)(uint32_t)(k & 0xffffffffu);
        const int i0 = tri[3 * (long long)t], i1 = tri[3 * (long long)t + 1], i2 = tri[3 * (long long)t + 2];
        Shade S;
        shade_eval_xy(P[i0], P[i1], P[i2], X, Y, W, H, S);
        rast[o] = make_float4(S.u, S.v, S.zw, enc_triid(t + 1));
        const float* a0 = A + (long long)i0 * C;
        const float* a1 = A + (long long)i1 * C;
        const float* a2 = A + (long long)i2 * C;
        if (vec) {
            for (int c = 0; c < C; c += 4) {
                const float4 x0 = __ldg(reinterpret_cast<const float4*>(a0 + c));
                const float4 x1 = __ldg(reinterpret_cast<const float4*>(a1 + c));
                const float4 x2 = __ldg(reinterpret_cast<const float4*>(a2 + c));
                float4 o;
                o.x = fmaf(x0.x - x2.x, S.u, fmaf(x1.x - x2.x, S.v, x2.x));
                o.y = fmaf(x0.y - x2.y, S.u, fmaf(x1.y - x2.y, S.v, x2.y));
                o.z = fmaf(x0.z - x2.z, S.u, fmaf(x1.z - x2.z, S.v, x2.z));
                o.w = fmaf(x0.w - x2.w, S.u, fmaf(x1.w - x2.w, S.v, x2.w));
                *reinterpret_cast<float4*>(col + c) = o;
                if (oc) *reinterpret_cast<float4*>(oc + c) = o;
            }
        } else {
            for (int c = 0; c < C; ++c) {
                const float v = fmaf(a0[c] - a2[c], S.u, fmaf(a1[c] - a2[c], S.v, a2[c]));
                col[c] = v;
                if (oc) oc[c] = v;
            }
        }
    }
};

__device__ __forceinline__ int find_item_by_tile(const drp_batch_item* items, int n, long long tile) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (items[mid].tile_offset <= tile) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int TILE_LOG2, int TPT>
__global__ void __launch_bounds__((1 << (2 * TILE_LOG2)) < 256 ? (1 << (2 * TILE_LOG2)) : 256,
                                  TILE_LOG2 == 3 ? 12 : 4)
batch_fine_kernel(BatchArgs a) {
    // The tile's parameters live in shared memory, filled by thread 0 with
    // the job: held in registers through the fine raster they pushed its
    // working set past the 64 registers of 4 CTAs per SM (spills).
    __shared__ long long job;
    __shared__ FineTile ft;
    __shared__ BatchEmit e;
    pdl_wait();
    pdl_launch_dependents();
    for (;;) {
        __syncthreads();  // every thread is done with the previous tile's job, ft and e
        if (threadIdx.x == 0) {
            const long long j = (long long)atomicAdd(a.queue, 1u);
            const long long t = j < a.total_tiles && a.tile_order ? (long long)a.tile_order[j] : j;
            job = t;
            if (t < a.total_tiles) {
                const int ii = find_item_by_tile(a.items, a.num_items, t);
                const drp_batch_item& it = a.items[ii];
                const int tile = (int)(t - it.tile_offset);
                ft.recs = a.prims;
                ft.cnt = a.tile_count[t];
                if (a.bin_depth) {
                    ft.list = a.tile_list + (unsigned long long)t * a.bin_depth;
                    ft.overflow = ft.cnt > a.bin_depth;
                    if (ft.overflow) atomicMax(a.stats + 3, ft.cnt);  // sizes the next depth
                } else {
                    const uint32_t off = a.tile_offset[t];
                    ft.list = a.tile_list + off;
                    ft.overflow = (unsigned long long)off + ft.cnt > a.list_capacity;
                }
                ft.scan_base = it.prim_offset;
                ft.scan_count = it.tri_count;
                ft.tx0 = (tile % it.tiles_x) << TILE_LOG2;
                ft.ty0 = (tile / it.tiles_x) << TILE_LOG2;
                ft.W = it.width;
                ft.H = it.height;
                ft.P = reinterpret_cast<const float4*>(a.pos) + it.pos_offset;
                ft.tri = a.tri + 3 * (long long)it.tri_first;
                ft.prev = nullptr;
                ft.stats = a.stats;
                e.P = ft.P;
                e.tri = ft.tri;
                e.A = a.attr + it.attr_offset;
                e.W = it.width;
                e.H = it.height;
                e.C = it.channels;
                e.rast = reinterpret_cast<float4*>(a.rast) + it.pixel_offset;
                e.color = a.color + it.image_offset;
                e.out = a.emit_out ? a.out + it.image_offset : nullptr;
                e.vec = (it.channels & 3) == 0 &&
                        ((reinterpret_cast<uintptr_t>(e.A) | reinterpret_cast<uintptr_t>(e.color) |
                          reinterpret_cast<uintptr_t>(e.out)) & 15) == 0;
            }
        }
        __syncthreads();
        if (job >= a.total_tiles) break;
        fine_tile<TILE_LOG2, TPT, false>(ft, e);
    }
}

__global__ void __launch_bounds__(256) batch_aa_setup_kernel(BatchArgs a) {
    pdl_wait();
    pdl_launch_dependents();
    const int2 blk = a.prim_blocks[blockIdx.x];
    const drp_batch_item& it = a.items[blk.x];
    const long long j = (long long)blk.y * 256 + threadIdx.x;
    if (j >= it.tri_count) return;
    const float4* P = reinterpret_cast<const float4*>(a.pos) + it.pos_offset;
    aa_tri_record(P, a.tri + 3 * (long long)it.tri_first, a.nbr ? a.nbr + 3 * (long long)it.tri_first : nullptr, j,
                  it.tri_count, it.num_vertices, it.width, it.height, a.aa_rec + (it.prim_offset + j) * 2);
}

// Record a pixel some blending pair touches: its flag, and (warp-aggregated)
// its global index in the list the antialias backward walks.  All 32 lanes
// of the warp call it.
// FLAGS = false: the list only (the forward that forms the loss's gradient
// has no backward pass to read the per-pixel flags).
template <bool FLAGS = true>
__device__ __forceinline__ void aa_note_pixel(const BatchArgs& a, long long gpix, bool in, unsigned bits) {
    if (!a.aa_flags) return;
    if (FLAGS && in) a.aa_flags[gpix] = bits ? 1 : 0;
    const bool need = in && bits != 0u;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(a.aa_count, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (need) a.aa_list[base + __popc(m & ((1u << lane) - 1u))] = (int)gpix;
}

__global__ void __launch_bounds__(256) batch_aa_fwd_kernel(BatchArgs a) {
    pdl_wait();
    pdl_launch_dependents();
    const int2 blk = a.pix_blocks[blockIdx.x];
    const drp_batch_item& it = a.items[blk.x];
    const int pix = blk.y * 256 + threadIdx.x;
    const bool in = pix < it.width * it.height;
    unsigned bits = 0;
    if (in) {
        const float4* R = reinterpret_cast<const float4*>(a.rast) + it.pixel_offset;
        // out already holds the colour (written by the fine raster): only blended pixels change
        aa_fwd_pixel<false>(R, a.color + it.image_offset, a.aa_rec + it.prim_offset * 2, it.tri_count, it.width,
                            it.height, it.channels, pix, a.out + it.image_offset + (long long)pix * it.channels,
                            &bits);
    }
    aa_note_pixel(a, it.pixel_offset + pix, in, bits);
}

// Antialias forward with the mean-absolute-error loss fused: every pixel's
// output (written when out is set), sign gradient and |error| sum; one
// partial per 256-pixel block, added in index order by the final reduction
// (reproducible loss).
__global__ void __launch_bounds__(256, 5) batch_aa_l1_kernel(BatchArgs a) {
    __shared__ float warp_sum[8];
    pdl_wait();
    pdl_launch_dependents();
    const int2 blk = a.pix_blocks[blockIdx.x];
    const drp_batch_item& it = a.items[blk.x];
    const int pix = blk.y * 256 + threadIdx.x;
    float s = 0.0f;
    const bool in = pix < it.width * it.height;
    unsigned bits = 0;
    {
        const float4* R = reinterpret_cast<const float4*>(a.rast) + it.pixel_offset;
        int src[4];
        float wt[4];
        const bool any = aa_fwd_terms_row(R, a.aa_rec + it.prim_offset * 2, it.tri_count, it.width, it.height, pix,
                                          in, src, wt, &bits);  // all lanes: pairs shared along the row
        if (in) {
            const long long row = it.image_offset + (long long)pix * it.channels;
            s = aa_l1_channels(a.color + it.image_offset, it.channels, pix, src, wt, any, a.target + row,
                               a.l1_scale, a.out ? a.out + row : nullptr, a.l1_grad + row);
        }
    }
    aa_note_pixel(a, it.pixel_offset + pix, in, bits);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
#pragma unroll
        for (int w = 0; w < 8; ++w) t += warp_sum[w];
        a.block_loss[blockIdx.x] = t;
    }
}

__device__ __forceinline__ int find_item_by_pixel(const drp_batch_item* items, int n, long long gpix) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (items[mid].pixel_offset <= gpix) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Whole backward of the listed pixels (those a blending pair touches, about
// the silhouettes): edge-vertex gradients (scattered once per pair by its
// first pixel), the pixel's antialiased colour gradient, and with it the
// pixel's interpolation backward (attribute atomics) and rasterisation
// backward (vertex atomics).  batch_bwd_kernel skips these pixels, so the two
// kernels are independent and run side by side.  The list is short and each
// pixel's chain of dependent loads is long, so a group of LANES lanes takes
// one pixel: lane q evaluates pair slots q, q + LANES, ... (and scatters a
// slot's edge gradient when it owns the pair), the group exchanges the slot
// terms by shuffles, the lanes share the channels (c = q, q + LANES, ...) and
// sum d/du, d/dv by shuffles.  Grid-stride over the device-side count, so
// the launch needs no host sync; the grid is one resident wave
// (list_kernel_grid).  L1G (the forward that forms the loss's gradient): the
// kernel follows the antialias / loss pass on the launch chain, and its last
// block first adds the loss from that pass's partials (no separate
// final-sum launch).
// The incoming image gradient of one item: the gradient buffer times the
// upstream scale, or (L1G, the forward that forms the loss's gradient) the
// L1 sign gradient from the output and the target.
template <bool L1G>
struct ItemGrad;
template <>
struct ItemGrad<false> {
    static __device__ __forceinline__ GradBuffer of(const BatchArgs& a, const drp_batch_item& it, float gsc) {
        return GradBuffer{a.grad_out + it.image_offset, gsc};
    }
};
template <>
struct ItemGrad<true> {
    static __device__ __forceinline__ GradL1 of(const BatchArgs& a, const drp_batch_item& it, float) {
        return GradL1{a.out + it.image_offset, a.target + it.image_offset, a.l1_scale};
    }
};

// Lanes per listed pixel in batch_aa_bwd_kernel.  Two lanes cover twice the
// pixels of four per resident wave (the single-mesh step lists ~45K pixels:
// one wave with two, two with four), but each lane's chain of slot
// evaluations doubles and the kernel needs 74 registers; four measured
// slightly faster on the single-mesh step (157.1 vs 159.2 us per step).
#ifndef DRP_LIST_LANES
#define DRP_LIST_LANES 4
#endif
constexpr int kListLanes = DRP_LIST_LANES;

template <bool L1G, int LANES>
__global__ void __launch_bounds__(256) batch_aa_bwd_kernel(BatchArgs a) {
    static_assert(LANES == 2 || LANES == 4, "two or four lanes per listed pixel");
    constexpr int SLOTS = 4 / LANES;  // pair slots each lane evaluates
    pdl_wait();
    pdl_launch_dependents();
    // the forward that forms the loss's gradient ends here: its last block
    // also adds the loss (the partials of the antialias / loss pass)
    static_assert(kFinalThreads == 256, "the list kernel's blocks form the loss");
    if (L1G && blockIdx.x == gridDim.x - 1)
        l1_final_block<kFinalThreads>(a.block_loss, a.n_pix_blocks, a.l1_scale, a.loss);
    const unsigned n = *a.aa_count;
    const float gsc = (!L1G && a.grad_scale) ? *a.grad_scale : 1.0f;
    const int lane = threadIdx.x & 31, q = lane & (LANES - 1), qbase = lane & ~(LANES - 1);
    const long long groups = ((long long)gridDim.x * blockDim.x) / LANES;
    for (long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / LANES;; i += groups) {
        const bool active = i < n;
        if (!__any_sync(0xffffffffu, active)) break;  // warp-uniform exit (lane groups step together)
        int role[SLOTS], tgt[SLOTS], pix = 0, C = 0;
        float wt[SLOTS];
#pragma unroll
        for (int j = 0; j < SLOTS; ++j) {
            role[j] = 0;
            tgt[j] = 0;
            wt[j] = 0.f;
        }
        const drp_batch_item* itp = nullptr;
        if (active) {
            const long long gpix = a.aa_list[i];
            itp = &a.items[find_item_by_pixel(a.items, a.num_items, gpix)];
            const drp_batch_item& it = *itp;
            pix = (int)(gpix - it.pixel_offset);
            C = it.channels;
            const int W = it.width, H = it.height;
            const int py = pix / W, px = pix - py * W;
            const float4* R = reinterpret_cast<const float4*>(a.rast) + it.pixel_offset;
            const float4 rs = R[pix];
#pragma unroll
            for (int j = 0; j < SLOTS; ++j) {
                int A, B, ax, ay;
                bool vert;
                if (!pair_slot(q + j * LANES, pix, px, py, W, H, A, B, ax, ay, vert)) continue;
                const float4 ro = R[A == pix ? B : A];
                if (ro.w == rs.w) continue;
                AAPair p;
                aa_pair(a.aa_rec + it.prim_offset * 2, it.tri_count, A, B, ax, ay, vert, A == pix ? rs : ro,
                        A == pix ? ro : rs, p);
                if (!p.valid) continue;
                role[j] = p.target == pix ? 1 : 2;
                tgt[j] = p.target;
                wt[j] = p.w;
                if (A == pix && !p.clamped)
                    aa_edge_grad_g(p, a.color + it.image_offset, ItemGrad<L1G>::of(a, it, gsc), C,
                                   reinterpret_cast<const float4*>(a.pos) + it.pos_offset,
                                   a.tri + 3 * (long long)it.tri_first,
                                   reinterpret_cast<float4*>(a.grad_pos) + it.pos_offset, 1.0f, W, H);
            }
        }
        // slot k was evaluated by lane (k % LANES) of the group, as its
        // (k / LANES)-th slot
        AATerms at;
        at.any = false;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int src = qbase | (k % LANES);
            at.role[k] = __shfl_sync(0xffffffffu, role[k / LANES], src);
            at.tgt[k] = __shfl_sync(0xffffffffu, tgt[k / LANES], src);
            at.wt[k] = __shfl_sync(0xffffffffu, wt[k / LANES], src);
            at.any = at.any || at.role[k] != 0;
        }
        int t = -1, i0 = 0, i1 = 0, i2 = 0;
        float gu = 0.f, gv = 0.f;
        if (active) {
            const drp_batch_item& it = *itp;
            const int* tri = a.tri + 3 * (long long)it.tri_first;
            const float4 r = reinterpret_cast<const float4*>(a.rast)[it.pixel_offset + pix];
            t = checked_tri(r.w, tri, it.tri_count, it.num_vertices, i0, i1, i2);
            if (t >= 0) {
                const auto grad = ItemGrad<L1G>::of(a, it, gsc);
                const float* A = a.attr + it.attr_offset;
                float* GA = a.grad_attr + it.attr_offset;
                const float u = r.x, v = r.y, w = 1.0f - u - v;
                for (int c = q; c < C; c += LANES) {
                    const float g = aa_bwd_channel_g(at, grad, C, pix, c);
                    const float x0 = A[(long long)i0 * C + c], x1 = A[(long long)i1 * C + c],
                                x2 = A[(long long)i2 * C + c];
                    atomicAdd(GA + (long long)i0 * C + c, g * u);
                    atomicAdd(GA + (long long)i1 * C + c, g * v);
                    atomicAdd(GA + (long long)i2 * C + c, g * w);
                    gu = fmaf(g, x0 - x2, gu);
                    gv = fmaf(g, x1 - x2, gv);
                }
            }
        }
#pragma unroll
        for (int off = 1; off < LANES; off <<= 1) {
            gu += __shfl_xor_sync(0xffffffffu, gu, off);
            gv += __shfl_xor_sync(0xffffffffu, gv, off);
        }
        if (active && t >= 0 && q == 0) {
            const drp_batch_item& it = *itp;
            const int W = it.width, H = it.height;
            const int py = pix / W, px = pix - py * W;
            const float X = fmaf((float)(2 * px + 1), __frcp_rn((float)W), -1.0f);
            const float Y = fmaf((float)(2 * py + 1), __frcp_rn((float)H), -1.0f);
            const float4* P = reinterpret_cast<const float4*>(a.pos) + it.pos_offset;
            float4* GP = reinterpret_cast<float4*>(a.grad_pos) + it.pos_offset;
            float4 g3[3];
            uv_grad_fast(P[i0], P[i1], P[i2], X, Y, gu, gv, g3);
            atomic_add4(GP + i0, make_float4(g3[0].x, g3[0].y, 0.f, g3[0].w));
            atomic_add4(GP + i1, make_float4(g3[1].x, g3[1].y, 0.f, g3[1].w));
            atomic_add4(GP + i2, make_float4(g3[2].x, g3[2].y, 0.f, g3[2].w));
        }
    }
}

// One resident wave of the listed-pixel kernel (its CTAs per SM from the
// occupancy query, cached per instantiation), capped by the pixel blocks.
template <bool L1G>
static long long list_kernel_grid(long long pix_blocks) {
    static std::atomic<int> per_sm{0};
    int per = per_sm.load(std::memory_order_relaxed);
    if (per == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_aa_bwd_kernel<L1G, kListLanes>, 256, 0);
        per = per > 0 ? per : 1;
        per_sm.store(per, std::memory_order_relaxed);
    }
    const int sms = drp_current_sm_count();
    const long long grid = (long long)(sms > 0 ? sms : 1) * per;
    return pix_blocks < grid ? pix_blocks : grid;
}

// Fused backward of one pixel: antialias colour gradient -> interpolation
// backward (attribute gradients, d/du, d/dv) -> rasterisation backward
// (vertex gradients).  Warps never straddle items (256-pixel blocks).
__global__ void __launch_bounds__(256, 4) batch_bwd_kernel(BatchArgs a) {
    pdl_wait();
    pdl_launch_dependents();
    const int2 blk = a.pix_blocks[blockIdx.x];
    const drp_batch_item& it = a.items[blk.x];
    const int pix = blk.y * 256 + threadIdx.x;
    const int W = it.width, H = it.height, C = it.channels;
    const bool in = pix < W * H;
    const float4* R = reinterpret_cast<const float4*>(a.rast) + it.pixel_offset;
    const float* Cc = a.color + it.image_offset;
    const float* Gd = a.grad_out + it.image_offset;
    const float4* P = reinterpret_cast<const float4*>(a.pos) + it.pos_offset;
    float4* GP = reinterpret_cast<float4*>(a.grad_pos) + it.pos_offset;
    const int* tri = a.tri + 3 * (long long)it.tri_first;
    const float* A = a.attr + it.attr_offset;
    float* GA = a.grad_attr + it.attr_offset;
    const float4* rec = a.aa_rec + it.prim_offset * 2;

    // incoming gradients are multiplied by gsc as they are read (a fused
    // loss's upstream gradient; exactly 1 otherwise)
    const float gsc = a.grad_scale ? *a.grad_scale : 1.0f;
    AATerms at;
    at.any = false;
    int t = -1, i0 = 0, i1 = 0, i2 = 0;
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    // With the forward's antialias state, the pixels a blend touches belong
    // to batch_aa_bwd_kernel (their whole backward) and are skipped here; the
    // other pixels have no antialias terms.  Without it the terms are
    // evaluated here for every pixel.
    const bool flagged = in && a.aa_flags && a.aa_flags[it.pixel_offset + pix];
    if (in && !flagged) {
        if (!a.aa_flags) aa_bwd_terms(R, Cc, Gd, rec, it.tri_count, W, H, C, P, tri, GP, 1.0f, pix, at, gsc);
        r = R[pix];
        t = checked_tri(r.w, tri, it.tri_count, it.num_vertices, i0, i1, i2);
    }
    const Seg seg = seg_setup(t >= 0 ? (long long)t : (long long)(-1 - lane_id()));
    const float u = r.x, v = r.y, w = 1.0f - u - v;
    float gu = 0.f, gv = 0.f;
    const bool vec = (C & 3) == 0 && ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(GA) |
                                       reinterpret_cast<uintptr_t>(Gd)) & 15) == 0;
    // Channel groups of 4: the next group's loads are issued before this
    // group's reduction and atomics, which would otherwise hold them back.
    float g[4], x0[4], x1[4], x2[4];
    auto load_group = [&](int c0) {
        if (vec) {
            const float4 gq = __ldg(reinterpret_cast<const float4*>(Gd + (long long)pix * C + c0));
            const float4 q0 = __ldg(reinterpret_cast<const float4*>(A + (long long)i0 * C + c0));
            const float4 q1 = __ldg(reinterpret_cast<const float4*>(A + (long long)i1 * C + c0));
            const float4 q2 = __ldg(reinterpret_cast<const float4*>(A + (long long)i2 * C + c0));
            g[0] = gq.x * gsc; g[1] = gq.y * gsc; g[2] = gq.z * gsc; g[3] = gq.w * gsc;
            x0[0] = q0.x; x0[1] = q0.y; x0[2] = q0.z; x0[3] = q0.w;
            x1[0] = q1.x; x1[1] = q1.y; x1[2] = q1.z; x1[3] = q1.w;
            x2[0] = q2.x; x2[1] = q2.y; x2[2] = q2.z; x2[3] = q2.w;
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int c = c0 + k < C ? c0 + k : C - 1;
                g[k] = c0 + k < C ? Gd[(long long)pix * C + c] * gsc : 0.f;
                x0[k] = A[(long long)i0 * C + c];
                x1[k] = A[(long long)i1 * C + c];
                x2[k] = A[(long long)i2 * C + c];
            }
        }
    };
    if (t >= 0) load_group(0);
    for (int c0 = 0; c0 < C; c0 += 4) {
        float val[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) val[k] = 0.f;
        if (t >= 0) {
            if (at.any) {
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (c0 + k < C) g[k] = aa_bwd_channel(at, Gd, C, pix, c0 + k, gsc);
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                val[k] = g[k] * u;
                val[4 + k] = g[k] * v;
                val[8 + k] = g[k] * w;
                gu = fmaf(g[k], x0[k] - x2[k], gu);
                gv = fmaf(g[k], x1[k] - x2[k], gv);
            }
            if (c0 + 4 < C) load_group(c0 + 4);
        }
        seg_reduce<12>(seg, val);
        if (t >= 0 && seg.head) {
            if (vec) {
                atomic_add4(reinterpret_cast<float4*>(GA + (long long)i0 * C + c0),
                            make_float4(val[0], val[1], val[2], val[3]));
                atomic_add4(reinterpret_cast<float4*>(GA + (long long)i1 * C + c0),
                            make_float4(val[4], val[5], val[6], val[7]));
                atomic_add4(reinterpret_cast<float4*>(GA + (long long)i2 * C + c0),
                            make_float4(val[8], val[9], val[10], val[11]));
            } else {
                for (int k = 0; k < 4 && c0 + k < C; ++k) {
                    atomicAdd(GA + (long long)i0 * C + c0 + k, val[k]);
                    atomicAdd(GA + (long long)i1 * C + c0 + k, val[4 + k]);
                    atomicAdd(GA + (long long)i2 * C + c0 + k, val[8 + k]);
                }
            }
        }
    }
    // u and v do not depend on clip z, so each vertex gradient is (x, y, 0, w):
    // nine values to reduce
    float pv[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) pv[k] = 0.f;
    if (t >= 0) {
        const int py = pix / W, px = pix - py * W;
        const float X = fmaf((float)(2 * px + 1), __frcp_rn((float)W), -1.0f);
        const float Y = fmaf((float)(2 * py + 1), __frcp_rn((float)H), -1.0f);
        float4 g3[3];
        uv_grad_fast(P[i0], P[i1], P[i2], X, Y, gu, gv, g3);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            pv[3 * k] = g3[k].x;
            pv[3 * k + 1] = g3[k].y;
            pv[3 * k + 2] = g3[k].w;
        }
    }
    seg_reduce<9>(seg, pv);
    if (t >= 0 && seg.head) {
        atomic_add4(GP + i0, make_float4(pv[0], pv[1], 0.f, pv[2]));
        atomic_add4(GP + i1, make_float4(pv[3], pv[4], 0.f, pv[5]));
        atomic_add4(GP + i2, make_float4(pv[6], pv[7], 0.f, pv[8]));
    }
}

// The backward of one pixel no blending pair touches, with the upstream
// gradient sign(out - target) * scale given by the sign masks (bit c:
// nonzero / positive): interpolation backward (attribute gradients) and
// rasterisation backward (vertex gradients), reduced over runs of one
// triangle in the warp and scattered with float4 atomics.  All 32 lanes call
// it (active = false for the others); a warp without an active lane on a
// triangle returns at once.
// r, t, i0..i2: the pixel's rast row, triangle (-1: none, or not active)
// and vertex indices, loaded by the caller before its antialias work.
__device__ __forceinline__ void pixel_backward_l1(const BatchArgs& a, const drp_batch_item& it, int pix, float4 r,
                                                  int t, int i0, int i1, int i2, unsigned nz, unsigned ps) {
    const int W = it.width, H = it.height, C = it.channels;
    const float* A = a.attr + it.attr_offset;
    float* GA = a.grad_attr + it.attr_offset;
    const float4* P = reinterpret_cast<const float4*>(a.pos) + it.pos_offset;
    float4* GP = reinterpret_cast<float4*>(a.grad_pos) + it.pos_offset;
    if (!__any_sync(0xffffffffu, t >= 0)) return;  // background or listed pixels only: nothing to add
    const Seg seg = seg_setup(t >= 0 ? (long long)t : (long long)(-1 - lane_id()));
    const float u = r.x, v = r.y, w = 1.0f - u - v;
    const float sc = a.l1_scale;
    float gu = 0.f, gv = 0.f;
    const bool vec = (C & 3) == 0 && ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(GA)) & 15) == 0;
    for (int c0 = 0; c0 < C; c0 += 4) {
        float val[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) val[k] = 0.f;
        if (t >= 0) {
            float g[4], x0[4], x1[4], x2[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int c = c0 + k;
                g[k] = (c < C && ((nz >> c) & 1u)) ? (((ps >> c) & 1u) ? sc : -sc) : 0.f;
            }
            if (vec) {
                const float4 q0 = __ldg(reinterpret_cast<const float4*>(A + (long long)i0 * C + c0));
                const float4 q1 = __ldg(reinterpret_cast<const float4*>(A + (long long)i1 * C + c0));
                const float4 q2 = __ldg(reinterpret_cast<const float4*>(A + (long long)i2 * C + c0));
                x0[0] = q0.x; x0[1] = q0.y; x0[2] = q0.z; x0[3] = q0.w;
                x1[0] = q1.x; x1[1] = q1.y; x1[2] = q1.z; x1[3] = q1.w;
                x2[0] = q2.x; x2[1] = q2.y; x2[2] = q2.z; x2[3] = q2.w;
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int c = c0 + k < C ? c0 + k : C - 1;
                    x0[k] = A[(long long)i0 * C + c];
                    x1[k] = A[(long long)i1 * C + c];
                    x2[k] = A[(long long)i2 * C + c];
                }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                val[k] = g[k] * u;
                val[4 + k] = g[k] * v;
                val[8 + k] = g[k] * w;
                gu = fmaf(g[k], x0[k] - x2[k], gu);
                gv = fmaf(g[k], x1[k] - x2[k], gv);
            }
        }
        seg_reduce<12>(seg, val);
        if (t >= 0 && seg.head) {
            if (vec) {
                atomic_add4(reinterpret_cast<float4*>(GA + (long long)i0 * C + c0),
                            make_float4(val[0], val[1], val[2], val[3]));
                atomic_add4(reinterpret_cast<float4*>(GA + (long long)i1 * C + c0),
                            make_float4(val[4], val[5], val[6], val[7]));
                atomic_add4(reinterpret_cast<float4*>(GA + (long long)i2 * C + c0),
                            make_float4(val[8], val[9], val[10], val[11]));
            } else {
                for (int k = 0; k < 4 && c0 + k < C; ++k) {
                    atomicAdd(GA + (long long)i0 * C + c0 + k, val[k]);
                    atomicAdd(GA + (long long)i1 * C + c0 + k, val[4 + k]);
                    atomicAdd(GA + (long long)i2 * C + c0 + k, val[8 + k]);
                }
            }
        }
    }
    float pv[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) pv[k] = 0.f;
    if (t >= 0) {
        const int py = pix / W, px = pix - py * W;
        const float X = fmaf((float)(2 * px + 1), __frcp_rn((float)W), -1.0f);
        const float Y = fmaf((float)(2 * py + 1), __frcp_rn((float)H), -1.0f);
        float4 g3[3];
        uv_grad_fast(P[i0], P[i1], P[i2], X, Y, gu, gv, g3);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            pv[3 * k] = g3[k].x;
            pv[3 * k + 1] = g3[k].y;
            pv[3 * k + 2] = g3[k].w;
        }
    }
    seg_reduce<9>(seg, pv);
    if (t >= 0 && seg.head) {
        atomic_add4(GP + i0, make_float4(pv[0], pv[1], 0.f, pv[2]));
        atomic_add4(GP + i1, make_float4(pv[3], pv[4], 0.f, pv[5]));
        atomic_add4(GP + i2, make_float4(pv[6], pv[7], 0.f, pv[8]));
    }
}

// Antialias + L1 loss with the loss's gradient formed in the same pass
// (drp_batch_forward_l1_grad).  Every pixel: its output and |error| partial
// as batch_aa_l1_kernel computes them.  Then, for the pixels no blending pair
// touches (the listed ones belong to batch_aa_bwd_kernel<true>, which forms
// the sign from the output and the target), the pixel's whole backward with
// the upstream gradient sign(out - target) * scale: interpolation backward
// (attribute gradients) and rasterisation backward (vertex gradients),
// reduced over runs of one triangle in the warp and scattered with float4
// atomics -- the work batch_bwd_kernel does for those pixels, done while
// the pixel's rast row and signs are at hand, with no gradient image written
// or read back.  The signs pass between the two phases as two bit masks, so
// an item may have at most 32 channels (more: DRP_DEVERR_CHANNELS, and the
// item gets no gradient here).  Warps never straddle items (256-pixel blocks).
__global__ void __launch_bounds__(256, 4) batch_aa_l1_grad_kernel(BatchArgs a) {
    __shared__ float warp_sum[8];
    pdl_wait();
    pdl_launch_dependents();
    const int2 blk = a.pix_blocks[blockIdx.x];
    const drp_batch_item& it = a.items[blk.x];
    const int pix = blk.y * 256 + threadIdx.x;
    const int W = it.width, H = it.height, C = it.channels;
    const bool in = pix < W * H;
    const float4* R = reinterpret_cast<const float4*>(a.rast) + it.pixel_offset;
    // the backward's rast row and vertex indices, loaded first so that their
    // latency overlaps the antialias work
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    int t = -1, i0 = 0, i1 = 0, i2 = 0;
    if (in) {
        r = R[pix];
        t = checked_tri(r.w, a.tri + 3 * (long long)it.tri_first, it.tri_count, it.num_vertices, i0, i1, i2);
    }
    float s = 0.0f;
    unsigned bits = 0u, nz = 0u, ps = 0u;
    {
        int src[4];
        float wt[4];
        const bool any = aa_fwd_terms_row(R, a.aa_rec + it.prim_offset * 2, it.tri_count, W, H, pix, in, src, wt,
                                          &bits);  // all lanes: pairs shared along the row
        if (in) {
            const long long row = it.image_offset + (long long)pix * C;
            s = aa_l1_channels(a.color + it.image_offset, C, pix, src, wt, any, a.target + row, a.l1_scale,
                               a.out + row, nullptr, &nz, &ps);
        }
    }
    aa_note_pixel<false>(a, it.pixel_offset + pix, in, bits);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = s;
    // the block's loss partial is added at the end: a barrier here would hold
    // every warp's backward until the slowest antialias pixel of the block
    pixel_backward_l1(a, it, pix, r, (bits == 0u && C <= 32) ? t : -1, i0, i1, i2, nz, ps);
    if (C > 32 && threadIdx.x == 0) atomicOr(a.stats + 2, DRP_DEVERR_CHANNELS);
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
#pragma unroll
        for (int w = 0; w < 8; ++w) t += warp_sum[w];
        a.block_loss[blockIdx.x] = t;
    }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
struct BatchLayout {
    size_t stats, queue, prims, count, offset, cursor, chunks, list, aa, total;
};

BatchLayout batch_layout(long long total_prims, long long total_tiles, unsigned long long cap) {
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    BatchLayout L;
    L.stats = 0;
    L.queue = 64;
    L.prims = 256;
    L.count = up(L.prims + (size_t)total_prims * 48);
    L.offset = up(L.count + (size_t)total_tiles * 4);
    L.cursor = up(L.offset + (size_t)total_tiles * 4);
    L.chunks = up(L.cursor + (size_t)total_tiles * 4);
    // the antialias records sit before the list: their offset must not depend
    // on the list capacity (the backward may reuse the forward's records)
    L.aa = up(L.chunks + (size_t)scan_chunks(total_tiles) * 8);
    L.list = up(L.aa + (size_t)total_prims * 32);
    L.total = up(L.list + (size_t)cap * 4);
    return L;
}

// Antialias state block: list count at 0, per-pixel flags at 256, the pixel
// list (int32) after them.
static size_t aa_state_bytes(long long total_pixels, size_t* list_off) {
    const size_t flags_end = 256 + (size_t)total_pixels;
    const size_t lo = (flags_end + 255) / 256 * 256;
    if (list_off) *list_off = lo;
    return lo + (size_t)total_pixels * 4;
}

static void carve_aa_state(BatchArgs& a, void* state, long long total_pixels) {
    if (!state) return;
    size_t lo = 0;
    aa_state_bytes(total_pixels, &lo);
    char* p = static_cast<char*>(state);
    a.aa_count = reinterpret_cast<unsigned*>(p);
    a.aa_flags = reinterpret_cast<unsigned char*>(p + 256);
    a.aa_list = reinterpret_cast<int*>(p + lo);
}

static void carve(BatchArgs& a, void* ws, const BatchLayout& L) {
    char* w = static_cast<char*>(ws);
    a.stats = reinterpret_cast<uint32_t*>(w + L.stats);
    a.queue = reinterpret_cast<uint32_t*>(w + L.queue);
    a.prims = reinterpret_cast<int4*>(w + L.prims);
    a.tile_count = reinterpret_cast<uint32_t*>(w + L.count);
    a.tile_offset = reinterpret_cast<uint32_t*>(w + L.offset);
    a.tile_cursor = reinterpret_cast<uint32_t*>(w + L.cursor);
    a.tile_list = reinterpret_cast<uint32_t*>(w + L.list);
    a.chunk_sums = reinterpret_cast<unsigned long long*>(w + L.chunks);
    a.aa_rec = reinterpret_cast<float4*>(w + L.aa);
}

// Up to this many tiles per resident fine CTA the work order is sorted.
constexpr long long kOrderTilesPerCTA = 8;

// Zeroes the stats / work-queue block (256 bytes), the antialias pixel-list
// count and the per-tile counts that a forward accumulates into: one kernel
// in the forward's launch chain instead of three memsets.
// Also zeroes `zero_n` floats at `zero` (the gradient buffers of
// drp_batch_forward_l1_grad, when the call is asked to start them at zero).
__global__ void __launch_bounds__(256) batch_clear_kernel(uint32_t* stats, unsigned* aa_count,
                                                          uint32_t* tile_count, long long tiles, float* zero,
                                                          long long zero_n) {
    pdl_wait();
    pdl_launch_dependents();
    const long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    if (i0 < 64) stats[i0] = 0u;
    if (i0 == 0 && aa_count) *aa_count = 0u;
    for (long long i = i0; i < tiles; i += stride) tile_count[i] = 0u;
    if (zero) {
        // 16-byte groups from the first aligned float (the buffer start is
        // at least 4-byte aligned), scalar head and tail
        const long long head = (long long)(((16 - (reinterpret_cast<uintptr_t>(zero) & 15)) & 15) >> 2);
        const long long h = head < zero_n ? head : zero_n;
        if (i0 < h) zero[i0] = 0.f;
        float4* z4 = reinterpret_cast<float4*>(zero + h);
        const long long n4 = (zero_n - h) >> 2;
        for (long long i = i0; i < n4; i += stride) z4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        const long long t0 = h + 4 * n4;
        if (i0 < zero_n - t0) zero[t0 + i0] = 0.f;
    }
}

template <int TL, int TPT>
static void launch_batch_fine(const BatchArgs& a, cudaStream_t s) {
    constexpr int NT = (1 << (2 * TL)) < 256 ? (1 << (2 * TL)) : 256;
    // persistent grid: every resident CTA slot of the device (occupancy per
    // kernel instantiation is device-independent for one architecture)
    static std::atomic<int> per_sm{0};
    int per = per_sm.load(std::memory_order_relaxed);
    if (per == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_fine_kernel<TL, TPT>, NT, 0);
        per = per > 0 ? per : 1;
        per_sm.store(per, std::memory_order_relaxed);
    }
    const int sms = drp_current_sm_count();
    const long long grid = (long long)(sms > 0 ? sms : 1) * per;
    const long long g = a.total_tiles < grid ? a.total_tiles : grid;
    if (g <= 0) return;
    // With a few tiles per resident CTA, hand the longest tile lists out
    // first (the order goes into the fill cursors, which are spent by now).
    BatchArgs b = a;
    b.tile_order = nullptr;
    if (a.total_tiles > g && a.total_tiles <= kOrderTilesPerCTA * grid) {
        launch_tile_order(a.tile_count, a.total_tiles, a.tile_cursor, s);
        b.tile_order = a.tile_cursor;
    }
    launch_pdl(batch_fine_kernel<TL, TPT>, dim3((unsigned)g), dim3(NT), s, b);
    drp_note_launch();
}

template <int TL>
static void launch_batch_raster(const BatchArgs& a, cudaStream_t s) {
    if (a.n_prim_blocks > 0 && a.bin_depth) {
        launch_pdl(batch_setup_bin_kernel<TL, kSetupBins>, dim3((unsigned)(a.n_prim_blocks * kSetupSplit)),
                   dim3(a.aa_records ? 2 * kSetupTris : kSetupTris), s, a);
        drp_note_launch();
    } else if (a.n_prim_blocks > 0) {
        launch_pdl(batch_setup_bin_kernel<TL, kSetupCount>, dim3((unsigned)(a.n_prim_blocks * kSetupSplit)),
                   dim3(a.aa_records ? 2 * kSetupTris : kSetupTris), s, a);
        drp_note_launch();
        launch_tile_scan(a.tile_count, a.tile_offset, a.tile_cursor, a.total_tiles, a.chunk_sums,
                         reinterpret_cast<unsigned long long*>(a.stats), s);
        batch_setup_bin_kernel<TL, kSetupFill><<<(unsigned)(a.n_prim_blocks * kSetupSplit), kSetupTris, 0, s>>>(a);
        drp_note_launch();
    } else {
        cudaMemsetAsync(a.tile_offset, 0, sizeof(uint32_t) * a.total_tiles, s);
    }
    switch (a.tpt) {
    case 0: launch_batch_fine<TL, 0>(a, s); break;
    case 1: launch_batch_fine<TL, 1>(a, s); break;
    case 2: launch_batch_fine<TL, 2>(a, s); break;
    case 4: launch_batch_fine<TL, 4>(a, s); break;
    case 8: launch_batch_fine<TL, 8>(a, s); break;
    case 16: launch_batch_fine<TL, 16>(a, s); break;
    default: launch_batch_fine<TL, 32>(a, s); break;
    }
}

// A side stream with its fork / join events, one per host thread and device,
// created on first use outside stream capture (inside a capture, before the
// first ordinary call, the caller's stream serves alone).  Captured forks
// and joins become graph edges.  The caller's stream belongs to the current
// device, as for every launch of this library (a stream query here would
// invalidate a capture in progress).
struct SideStream {
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};

static bool side_stream(cudaStream_t s, SideStream& out) {
    constexpr int kMaxDev = 64;
    thread_local SideStream cache[kMaxDev];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) {
        cudaGetLastError();
        return false;
    }
    SideStream& c = cache[dev];
    if (!c.stream) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
            cudaGetLastError();
            return false;
        }
        SideStream n;
        if (cudaStreamCreateWithFlags(&n.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&n.fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&n.join, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            if (n.stream) cudaStreamDestroy(n.stream);
            if (n.fork) cudaEventDestroy(n.fork);
            return false;
        }
        c = n;
    }
    out = c;
    return true;
}

int launch_batch_forward(BatchArgs a, void* ws, const BatchLayout& L, cudaStream_t s) {
    carve(a, ws, L);
    {
        // stats and work queue, list count, tile counts (and the buffers a
        // gradient-forming forward is asked to zero)
        long long need = a.total_tiles > 64 ? a.total_tiles : 64;
        if (a.zero_first && a.zero_floats / 4 > need) need = a.zero_floats / 4;
        const int sms = drp_current_sm_count();
        long long blocks = (need + 255) / 256;
        const long long cap = (long long)(sms > 0 ? sms : 1) * 4;
        if (blocks > cap) blocks = cap;
        launch_pdl(batch_clear_kernel, dim3((unsigned)blocks), dim3(256), s, a.stats, a.aa_count, a.tile_count,
                   (long long)a.total_tiles, a.zero_first, a.zero_floats);
        drp_note_launch();
    }
    switch (a.tile_log2) {
    case 3: launch_batch_raster<3>(a, s); break;
    case 5: launch_batch_raster<5>(a, s); break;
    default: launch_batch_raster<4>(a, s); break;
    }
    // (the antialias triangle records were written by the setup / count pass)
    if (a.target && a.l1_grads) {
        if (a.n_pix_blocks > 0) {
            launch_pdl(batch_aa_l1_grad_kernel, dim3((unsigned)a.n_pix_blocks), dim3(256), s, a);
            drp_note_launch();
            // the listed pixels' whole backward, and (its last block) the
            // final loss sum: one launch on the chain
            const long long g = list_kernel_grid<true>(a.n_pix_blocks);
            launch_pdl(batch_aa_bwd_kernel<true, kListLanes>, dim3((unsigned)g), dim3(256), s, a);
            drp_note_launch();
        } else {
            launch_l1_final(a.block_loss, a.n_pix_blocks, a.l1_scale, a.loss, s);
        }
        return 0;
    }
    if (a.target) {
        if (a.n_pix_blocks > 0) {
            launch_pdl(batch_aa_l1_kernel, dim3((unsigned)a.n_pix_blocks), dim3(256), s, a);
            drp_note_launch();
        }
        launch_l1_final(a.block_loss, a.n_pix_blocks, a.l1_scale, a.loss, s);
        return 0;
    }
    if (!a.out) return 0;  // raster + interpolation only (recomputing them for the backward)
    if (a.n_pix_blocks > 0) {
        launch_pdl(batch_aa_fwd_kernel, dim3((unsigned)a.n_pix_blocks), dim3(256), s, a);
        drp_note_launch();
    }
    return 0;
}

int launch_batch_backward(BatchArgs a, void* ws, const BatchLayout& L, bool reuse_records, cudaStream_t s) {
    carve(a, ws, L);
    if (a.n_prim_blocks > 0 && !reuse_records) {
        launch_pdl(batch_aa_setup_kernel, dim3((unsigned)a.n_prim_blocks), dim3(256), s, a);
        drp_note_launch();
    }
    if (a.n_pix_blocks <= 0) return 0;
    if (!a.aa_flags) {
        batch_bwd_kernel<<<(unsigned)a.n_pix_blocks, 256, 0, s>>>(a);
        drp_note_launch();
        return 0;
    }
    // The listed pixels' kernel (latency-bound, a few percent of the pixels)
    // and the fused backward of all other pixels are independent: fork the
    // list kernel onto a side stream so it fills the SMs beside the main
    // kernel and its tail, then join.  Both only add into the gradients.
    const long long g = list_kernel_grid<false>(a.n_pix_blocks);
    SideStream side;
    const bool fork = side_stream(s, side);
    if (fork) {
        cudaEventRecord(side.fork, s);
        cudaStreamWaitEvent(side.stream, side.fork, 0);
    }
    batch_bwd_kernel<<<(unsigned)a.n_pix_blocks, 256, 0, s>>>(a);
    drp_note_launch();
    batch_aa_bwd_kernel<false, kListLanes><<<(unsigned)g, 256, 0, fork ? side.stream : s>>>(a);
    drp_note_launch();
    if (fork) {
        cudaEventRecord(side.join, side.stream);
        cudaStreamWaitEvent(s, side.join, 0);
    }
    return 0;
}

}  // namespace drp

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
#define DRP_API extern "C" __attribute__((visibility("default")))

namespace {
int bfail(const char* msg) {
    drp_set_last_error(msg);
    return DRP_STATUS_INVALID_ARGUMENT;
}
}  // namespace

DRP_API int drp_batch_plan(drp_batch_item* items, int num_items, int tile_log2, long long* totals) {
    if (!items || num_items <= 0 || !totals) return bfail("drp_batch_plan: bad arguments");
    if (tile_log2 < 3 || tile_log2 > 5) return bfail("drp_batch_plan: tile_log2 must be 3, 4 or 5");
    long long prims = 0, tiles = 0, pixels = 0, floats = 0, pblocks = 0, xblocks = 0;
    for (int i = 0; i < num_items; ++i) {
        drp_batch_item& it = items[i];
        if (it.height <= 0 || it.width <= 0 || it.height > DRP_MAX_RESOLUTION || it.width > DRP_MAX_RESOLUTION ||
            it.channels <= 0 || it.tri_count < 0 || it.tri_first < 0 || it.num_vertices < 0 || it.pos_offset < 0 ||
            it.attr_offset < 0)
            return bfail("drp_batch_plan: item with invalid size, resolution or offset");
        it.tiles_x = (it.width + (1 << tile_log2) - 1) >> tile_log2;
        it.tiles_y = (it.height + (1 << tile_log2) - 1) >> tile_log2;
        it.prim_offset = prims;
        it.tile_offset = tiles;
        it.pixel_offset = pixels;
        it.image_offset = floats;
        prims += it.tri_count;
        tiles += (long long)it.tiles_x * it.tiles_y;
        pixels += (long long)it.width * it.height;
        floats += (long long)it.width * it.height * it.channels;
        pblocks += (it.tri_count + 255) / 256;
        xblocks += ((long long)it.width * it.height + 255) / 256;
    }
    totals[0] = prims;
    totals[1] = tiles;
    totals[2] = pixels;
    totals[3] = floats;
    totals[4] = pblocks;
    totals[5] = xblocks;
    return DRP_STATUS_OK;
}

DRP_API int drp_batch_block_maps(const drp_batch_item* items, int num_items, int* prim_block_map,
                                 int* pixel_block_map) {
    if (!items || num_items <= 0 || !prim_block_map || !pixel_block_map) return bfail("drp_batch_block_maps: null");
    long long p = 0, x = 0;
    for (int i = 0; i < num_items; ++i) {
        const long long nb = (items[i].tri_count + 255) / 256;
        for (long long k = 0; k < nb; ++k, ++p) {
            prim_block_map[2 * p] = i;
            prim_block_map[2 * p + 1] = (int)k;
        }
        const long long xb = ((long long)items[i].width * items[i].height + 255) / 256;
        for (long long k = 0; k < xb; ++k, ++x) {
            pixel_block_map[2 * x] = i;
            pixel_block_map[2 * x + 1] = (int)k;
        }
    }
    return DRP_STATUS_OK;
}

DRP_API int drp_batch_aa_state_size(long long total_pixels, size_t* bytes) {
    if (!bytes || total_pixels <= 0) return bfail("drp_batch_aa_state_size: bad arguments");
    *bytes = drp::aa_state_bytes(total_pixels, nullptr);
    return DRP_STATUS_OK;
}

DRP_API int drp_batch_workspace_size(long long total_prims, long long total_tiles, unsigned long long list_capacity,
                                     size_t* bytes) {
    if (!bytes || total_prims < 0 || total_tiles < 0 || list_capacity > 0x7fffffffull)
        return bfail("drp_batch_workspace_size: bad arguments");
    *bytes = drp::batch_layout(total_prims, total_tiles, list_capacity).total;
    return DRP_STATUS_OK;
}

static int batch_common(void* ws, size_t ws_bytes, const drp_batch_item* items, int num_items,
                        const int* prim_block_map, long long prim_blocks, const int* pixel_block_map,
                        long long pixel_blocks, long long total_prims, long long total_tiles,
                        unsigned long long list_capacity, const float* pos, const int* tri, const float* attr,
                        drp::BatchArgs& a, drp::BatchLayout& L) {
    if (!ws || (reinterpret_cast<uintptr_t>(ws) & 255)) return bfail("batch: workspace must be 256-byte aligned");
    if (!items || num_items <= 0 || !pos || !tri || !attr) return bfail("batch: null table or buffer");
    if ((prim_blocks > 0 && !prim_block_map) || (pixel_blocks > 0 && !pixel_block_map) || prim_blocks < 0 ||
        pixel_blocks < 0 || prim_blocks > 0x7fffffffll / drp::kSetupSplit || pixel_blocks > 0x7fffffffll)
        return bfail("batch: bad block maps");
    if ((reinterpret_cast<uintptr_t>(pos) & 15)) return bfail("batch: pos must be 16-byte aligned");
    if (list_capacity > 0x7fffffffull) return bfail("batch: list_capacity above 2^31 - 1");
    L = drp::batch_layout(total_prims, total_tiles, list_capacity);
    if (ws_bytes < L.total) {
        drp_set_last_error("batch: workspace too small");
        return DRP_STATUS_WORKSPACE_TOO_SMALL;
    }
    a = drp::BatchArgs{};
    a.items = items;
    a.num_items = num_items;
    a.prim_blocks = reinterpret_cast<const int2*>(prim_block_map);
    a.n_prim_blocks = prim_blocks;
    a.pix_blocks = reinterpret_cast<const int2*>(pixel_block_map);
    a.n_pix_blocks = pixel_blocks;
    a.total_prims = total_prims;
    a.total_tiles = total_tiles;
    a.pos = pos;
    a.tri = tri;
    a.attr = attr;
    a.list_capacity = list_capacity;
    return DRP_STATUS_OK;
}

DRP_API int drp_batch_forward(void* workspace, size_t workspace_bytes, const drp_batch_item* items, int num_items,
                              const int* prim_block_map, long long prim_blocks, const int* pixel_block_map,
                              long long pixel_blocks, long long total_prims, long long total_tiles, const float* pos,
                              const int* tri, const float* attr, const int* nbr, int tile_log2, int threads_per_tri,
                              unsigned long long list_capacity, unsigned bin_depth, float* rast, float* color,
                              float* out, void* aa_state, long long total_pixels, void* stream) {
    drp::BatchArgs a;
    drp::BatchLayout L;
    int st = batch_common(workspace, workspace_bytes, items, num_items, prim_block_map, prim_blocks, pixel_block_map,
                          pixel_blocks, total_prims, total_tiles, list_capacity, pos, tri, attr, a, L);
    if (st) return st;
    if (tile_log2 < 3 || tile_log2 > 5) return bfail("batch: tile_log2 must be 3, 4 or 5");
    if (threads_per_tri < 0 || threads_per_tri > 32 || (threads_per_tri & (threads_per_tri - 1)))
        return bfail("batch: threads_per_tri must be 0 or a power of two <= 32");
    if (!rast || !color || (reinterpret_cast<uintptr_t>(rast) & 15)) return bfail("batch: bad outputs");
    if (bin_depth && (unsigned long long)total_tiles * bin_depth > list_capacity)
        return bfail("batch: list_capacity below total_tiles * bin_depth");
    a.nbr = nbr;
    a.tile_log2 = tile_log2;
    a.tpt = threads_per_tri;
    a.bin_depth = bin_depth;
    a.rast = rast;
    a.color = color;
    a.out = out;
    if (aa_state && ((reinterpret_cast<uintptr_t>(aa_state) & 255) || total_pixels <= 0))
        return bfail("batch: aa_state must be 256-byte aligned, with total_pixels > 0");
    carve_aa_state(a, aa_state, total_pixels);
    a.emit_out = out != nullptr;
    a.aa_records = out != nullptr;  // raster only: no antialias pass, no records
    drp::launch_batch_forward(a, workspace, L, static_cast<cudaStream_t>(stream));
    return drp_check_launch("drp_batch_forward");
}

DRP_API int drp_batch_forward_l1(void* workspace, size_t workspace_bytes, const drp_batch_item* items, int num_items,
                                 const int* prim_block_map, long long prim_blocks, const int* pixel_block_map,
                                 long long pixel_blocks, long long total_prims, long long total_tiles,
                                 const float* pos, const int* tri, const float* attr, const int* nbr, int tile_log2,
                                 int threads_per_tri, unsigned long long list_capacity, unsigned bin_depth,
                                 float* rast, float* color, float* out, void* aa_state, long long total_pixels,
                                 const float* target, float scale, float* grad, float* block_loss, float* loss,
                                 void* stream) {
    drp::BatchArgs a;
    drp::BatchLayout L;
    int st = batch_common(workspace, workspace_bytes, items, num_items, prim_block_map, prim_blocks, pixel_block_map,
                          pixel_blocks, total_prims, total_tiles, list_capacity, pos, tri, attr, a, L);
    if (st) return st;
    if (tile_log2 < 3 || tile_log2 > 5) return bfail("batch: tile_log2 must be 3, 4 or 5");
    if (threads_per_tri < 0 || threads_per_tri > 32 || (threads_per_tri & (threads_per_tri - 1)))
        return bfail("batch: threads_per_tri must be 0 or a power of two <= 32");
    if (!rast || !color || !target || !grad || !loss || (pixel_blocks > 0 && !block_loss) ||
        (reinterpret_cast<uintptr_t>(rast) & 15))
        return bfail("batch: bad outputs");
    if (bin_depth && (unsigned long long)total_tiles * bin_depth > list_capacity)
        return bfail("batch: list_capacity below total_tiles * bin_depth");
    a.nbr = nbr;
    a.tile_log2 = tile_log2;
    a.tpt = threads_per_tri;
    a.bin_depth = bin_depth;
    a.rast = rast;
    a.color = color;
    a.out = out;
    if (aa_state && ((reinterpret_cast<uintptr_t>(aa_state) & 255) || total_pixels <= 0))
        return bfail("batch: aa_state must be 256-byte aligned, with total_pixels > 0");
    carve_aa_state(a, aa_state, total_pixels);
    a.emit_out = false;  // the fused antialias + loss pass writes every output pixel
    a.aa_records = true;
    a.target = target;
    a.l1_scale = scale;
    a.l1_grad = grad;
    a.block_loss = block_loss;
    a.loss = loss;
    drp::launch_batch_forward(a, workspace, L, static_cast<cudaStream_t>(stream));
    return drp_check_launch("drp_batch_forward_l1");
}

DRP_API int drp_batch_forward_l1_grad(void* workspace, size_t workspace_bytes, const drp_batch_item* items,
                                      int num_items, const int* prim_block_map, long long prim_blocks,
                                      const int* pixel_block_map, long long pixel_blocks, long long total_prims,
                                      long long total_tiles, const float* pos, const int* tri, const float* attr,
                                      const int* nbr, int tile_log2, int threads_per_tri,
                                      unsigned long long list_capacity, unsigned bin_depth, float* rast, float* color,
                                      float* out, void* aa_state, long long total_pixels, const float* target,
                                      float scale, float* block_loss, float* loss, float* grad_pos, float* grad_attr,
                                      float* zero_first, long long zero_floats, void* stream) {
    drp::BatchArgs a;
    drp::BatchLayout L;
    int st = batch_common(workspace, workspace_bytes, items, num_items, prim_block_map, prim_blocks, pixel_block_map,
                          pixel_blocks, total_prims, total_tiles, list_capacity, pos, tri, attr, a, L);
    if (st) return st;
    if (tile_log2 < 3 || tile_log2 > 5) return bfail("batch: tile_log2 must be 3, 4 or 5");
    if (threads_per_tri < 0 || threads_per_tri > 32 || (threads_per_tri & (threads_per_tri - 1)))
        return bfail("batch: threads_per_tri must be 0 or a power of two <= 32");
    if (!rast || !color || !out || !target || !loss || (pixel_blocks > 0 && !block_loss) ||
        (reinterpret_cast<uintptr_t>(rast) & 15))
        return bfail("batch: bad outputs");
    if (!grad_pos || !grad_attr || (reinterpret_cast<uintptr_t>(grad_pos) & 15))
        return bfail("batch: bad gradient buffers");
    if (!aa_state || (reinterpret_cast<uintptr_t>(aa_state) & 255) || total_pixels <= 0)
        return bfail("batch: the gradient pass needs the antialias state (256-byte aligned, total_pixels > 0)");
    if (bin_depth && (unsigned long long)total_tiles * bin_depth > list_capacity)
        return bfail("batch: list_capacity below total_tiles * bin_depth");
    a.nbr = nbr;
    a.tile_log2 = tile_log2;
    a.tpt = threads_per_tri;
    a.bin_depth = bin_depth;
    a.rast = rast;
    a.color = color;
    a.out = out;
    carve_aa_state(a, aa_state, total_pixels);
    a.emit_out = false;  // the fused antialias + loss pass writes every output pixel
    a.aa_records = true;
    a.target = target;
    a.l1_scale = scale;
    a.l1_grad = nullptr;
    a.block_loss = block_loss;
    a.loss = loss;
    a.l1_grads = true;
    a.grad_pos = grad_pos;
    a.grad_attr = grad_attr;
    if (zero_floats < 0 || (zero_floats > 0 && !zero_first) || (reinterpret_cast<uintptr_t>(zero_first) & 3))
        return bfail("batch: bad zero region");
    a.zero_first = zero_floats > 0 ? zero_first : nullptr;
    a.zero_floats = zero_floats;
    drp::launch_batch_forward(a, workspace, L, static_cast<cudaStream_t>(stream));
    return drp_check_launch("drp_batch_forward_l1_grad");
}

DRP_API int drp_batch_backward(void* workspace, size_t workspace_bytes, const drp_batch_item* items, int num_items,
                               const int* prim_block_map, long long prim_blocks, const int* pixel_block_map,
                               long long pixel_blocks, long long total_prims, long long total_tiles,
                               const float* pos, const int* tri, const float* attr, const int* nbr,
                               const float* rast, const float* color, const void* aa_state, long long total_pixels,
                               float* aa_grad,
                               const float* grad_out, float* grad_pos, float* grad_attr, const float* grad_scale,
                               int flags, void* stream) {
    drp::BatchArgs a;
    drp::BatchLayout L;
    int st = batch_common(workspace, workspace_bytes, items, num_items, prim_block_map, prim_blocks, pixel_block_map,
                          pixel_blocks, total_prims, total_tiles, 0, pos, tri, attr, a, L);
    if (st) return st;
    if (!rast || !color || !grad_out || !grad_pos || !grad_attr || (reinterpret_cast<uintptr_t>(grad_pos) & 15))
        return bfail("batch: bad gradient buffers");
    a.nbr = nbr;
    a.rast = const_cast<float*>(rast);
    a.color = const_cast<float*>(color);
    (void)aa_grad;  // no longer used: the listed pixels' backward is fused into their kernel
    if (aa_state && ((reinterpret_cast<uintptr_t>(aa_state) & 255) || total_pixels <= 0))
        return bfail("batch: aa_state needs 256-byte alignment and total_pixels > 0");
    carve_aa_state(a, const_cast<void*>(aa_state), total_pixels);
    a.grad_out = grad_out;
    a.grad_pos = grad_pos;
    a.grad_attr = grad_attr;
    a.grad_scale = grad_scale;
    if (flags & ~DRP_BATCH_REUSE_AA_RECORDS) return bfail("batch: unknown flags");
    drp::launch_batch_backward(a, workspace, L, (flags & DRP_BATCH_REUSE_AA_RECORDS) != 0,
                               static_cast<cudaStream_t>(stream));
    return drp_check_launch("drp_batch_backward");
}
