/*
 * diffrp_gb300.h -- C ABI of the GB300 (sm_103a) differentiable rasterisation
 * library libdiffrp_gb300.so.
 *
 * The entry points replace the native calls diffrp makes into nvdiffrast
 * (package diffrp-nvdiffrast, setup.py:39 of the reference):
 *
 *   dr.RasterizeCudaContext()                 diffrp/rendering/surface_deferred.py:225
 *   dr.DepthPeeler(...).rasterize_next_layer() diffrp/rendering/surface_deferred.py:260-262
 *   dr.interpolate(attr, rast, tri)           diffrp/rendering/interpolator.py:83
 *   dr.antialias(color, rast, pos, tri)       diffrp/rendering/surface_deferred.py:775
 *   polyfill_interpolate (torch gather + FMA) diffrp/rendering/interpolator.py:32-65
 *
 * Conventions
 *   - Every pointer argument is a device pointer unless stated otherwise;
 *     arrays are dense, row-major, float32 / int32 as typed.  float4-typed
 *     rows (pos, rast, rast_db, grad_rast) must be 16-byte aligned.
 *   - `stream` is a cudaStream_t passed as void*; NULL is the legacy stream.
 *     Every call only enqueues work; nothing synchronises the host.
 *   - The library allocates no device memory.  Scratch comes from
 *     caller-provided workspaces whose sizes are queried first.
 *   - rast layout (B, H, W, 4) = (u, v, z/w, tri_id + 1); row 0 is NDC y = -1.
 *     tri ids above 2^24 are stored as the float with bit pattern
 *     0x4a800000 + id (diffrp/rendering/interpolator.py:24-29).
 *   - Return value: DRP_STATUS_*; drp_last_error() gives a message for the
 *     calling thread.
 *   - Gradient outputs marked "accumulated" are added into (caller zeroes).
 */
#ifndef DIFFRP_GB300_H
#define DIFFRP_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DRP_ABI_VERSION 1

#define DRP_STATUS_OK 0
#define DRP_STATUS_INVALID_ARGUMENT 1
#define DRP_STATUS_WORKSPACE_TOO_SMALL 2
#define DRP_STATUS_CUDA_ERROR 3

/* Largest supported raster width / height. */
#define DRP_MAX_RESOLUTION 16384

/* Device error bits in the rasterisation workspace's stats block. */
#define DRP_DEVERR_BAD_INDEX 1u
#define DRP_DEVERR_LIST_OVERFLOW 2u
/* drp_batch_forward_l1_grad: an item has more than 32 channels (its gradient was not formed). */
#define DRP_DEVERR_CHANNELS 4u

int drp_abi_version(void);
const char* drp_status_string(int status);
const char* drp_last_error(void);

/* Kernel launches this library has enqueued since it was loaded, all threads
 * and streams (launches recorded into a CUDA graph count once, at capture).
 * No counterpart in the reference: a diagnostic for counting the kernels of a
 * step. */
unsigned long long drp_kernel_launches(void);

/* ------------------------------------------------------------------------ */
/* Rasterisation                                                             */
/* ------------------------------------------------------------------------ */

/*
 * Workspace bytes for drp_rasterize_fwd.  The first 16 bytes of the workspace
 * are a stats block written by every call: bytes [0, 8) = tile-list entries the
 * call needed (uint64), bytes [8, 12) = DRP_DEVERR_* bits, bytes [12, 16) =
 * the largest per-tile entry count (uint32).  Callers grow
 * list_capacity from the first field; a call whose lists overflow is still
 * exact (overflowing tiles fall back to scanning the view's primitives).
 */
int drp_raster_workspace_size(int num_views, long long max_view_tris, int height, int width, int tile_log2,
                              unsigned long long list_capacity, size_t* bytes);

/*
 * Rasterise num_views views.  Replaces dr.DepthPeeler(ctx, pos, tri, (h, w),
 * ranges).rasterize_next_layer() (diffrp/rendering/surface_deferred.py:260-262)
 * and dr.rasterize.
 *   pos              clip-space vertices, float4 rows; view b reads
 *                    pos + b * pos_view_stride (floats); stride 0 = shared
 *                    vertices (range mode).
 *   ranges           device int32 [num_views][2] = (first triangle, count), or
 *                    NULL for all triangles in every view (instanced mode).
 *   max_view_tris    max over views of the triangle count.
 *   tile_log2        3, 4 or 5 (8, 16, 32 pixel tiles).
 *   threads_per_tri  0: every thread owns pixels of the tile and tests them
 *                    against each primitive (no atomics); 1, 2, 4, 8, 16 or
 *                    32: that many threads walk one primitive's bounding box
 *                    and resolve depth with shared-memory atomics.
 *   bin_depth        0: exact tile lists (count, scan, fill passes);
 *                    > 0: one setup pass appends into fixed-depth bins
 *                    (list_capacity >= num_views * tiles * bin_depth); a
 *                    tile with more entries stays exact (it scans the view's
 *                    primitives), sets DRP_DEVERR_LIST_OVERFLOW and raises
 *                    the largest-count field to its count.
 *   prev_key         previous layer's keys (depth peeling) or NULL.
 *   rast             out (B, H, W, 4); rast_db out (B, H, W, 4) or NULL;
 *   out_key          out (B, H, W) uint64 visibility keys or NULL.
 */
int drp_rasterize_fwd(void* workspace, size_t workspace_bytes, const float* pos, long long pos_view_stride,
                      long long num_vertices, const int* tri, long long num_triangles, int num_views,
                      const int* ranges, long long max_view_tris, int height, int width, int tile_log2,
                      int threads_per_tri, unsigned long long list_capacity, unsigned bin_depth,
                      const unsigned long long* prev_key, float* rast, float* rast_db, unsigned long long* out_key,
                      void* stream);

/*
 * Backward of rasterisation: grad_rast (B, H, W, 4) on (u, v, z/w, -) and
 * optional grad_db (B, H, W, 4) -> grad_pos (accumulated, layout of pos).
 * The gradient path of dr.rasterize under autograd
 * (diffrp/rendering/surface_deferred.py:260-262).
 */
int drp_rasterize_bwd(const float* pos, long long pos_view_stride, long long num_vertices, const int* tri,
                      long long num_triangles, int num_views, int height, int width, const float* rast,
                      const float* grad_rast, const float* grad_db, float* grad_pos, void* stream);

/* ------------------------------------------------------------------------ */
/* Interpolation                                                             */
/* ------------------------------------------------------------------------ */

/*
 * dr.interpolate(attr, rast, tri, rast_db, diff_attrs)
 * (diffrp/rendering/interpolator.py:83).  attr (V, C) shared
 * (attr_view_stride 0) or (B, V, C).  diff_idx: device int32[num_diff] channel
 * indices for screen-space derivatives (da (B, H, W, 2 * num_diff)), NULL when
 * num_diff == 0.
 */
int drp_interpolate_fwd(const float* attr, long long attr_view_stride, long long num_vertices, int channels,
                        const float* rast, const float* rast_db, const int* tri, long long num_triangles,
                        int num_views, int height, int width, const int* diff_idx, int num_diff, float* out,
                        float* da, void* stream);

/* Backward of drp_interpolate_fwd.  grad_attr accumulated; grad_rast
 * (B, H, W, 4) and grad_db (B, H, W, 4, may be NULL) overwritten. */
int drp_interpolate_bwd(const float* attr, long long attr_view_stride, long long num_vertices, int channels,
                        const float* rast, const float* rast_db, const int* tri, long long num_triangles,
                        int num_views, int height, int width, const int* diff_idx, int num_diff,
                        const float* grad_out, const float* grad_da, float* grad_attr, float* grad_rast,
                        float* grad_db, void* stream);

/*
 * Stencil-masked interpolation of n pixel rows: polyfill_interpolate /
 * _interpolate_impl (diffrp/rendering/interpolator.py:32-65).
 * vi_data (n, 4) rast rows, tri_idx (n, 3) int64 vertex indices.
 */
int drp_interpolate_sparse_fwd(const float* vertex_buffer, long long num_vertices, int channels,
                               const float* vi_data, const long long* tri_idx, long long n, float* out,
                               void* stream);

/* Backward: grad_vb accumulated, grad_vi (n, 4) overwritten (u, v, 0, 0). */
int drp_interpolate_sparse_bwd(const float* vertex_buffer, long long num_vertices, int channels,
                               const float* vi_data, const long long* tri_idx, long long n, const float* grad_out,
                               float* grad_vb, float* grad_vi, void* stream);

/* ------------------------------------------------------------------------ */
/* Antialiasing                                                              */
/* ------------------------------------------------------------------------ */

/* Workspace bytes for drp_antialias_topology. */
int drp_topology_workspace_size(long long num_triangles, size_t* bytes);

/*
 * dr.antialias_construct_topology_hash(tri) (implicit in the dr.antialias call
 * at diffrp/rendering/surface_deferred.py:775): nbr (F, 3) int32; for edge k
 * of triangle t (vertices k+1, k+2), when exactly two triangles share that
 * vertex pair, the other triangle's vertex opposite the edge, else -1.  (The
 * table is opaque to diffrp, like nvdiffrast's topology hash; the
 * silhouette test only needs the opposite vertex.)
 */
int drp_antialias_topology(void* workspace, size_t workspace_bytes, const int* tri, long long num_triangles,
                           int* nbr, void* stream);

/* Workspace bytes for drp_antialias_fwd / drp_antialias_bwd (32 bytes per
 * view and triangle: screen-space vertices and silhouette-edge mask). */
int drp_antialias_workspace_size(int num_views, long long num_triangles, size_t* bytes);

/* Bytes of the optional pixel-list state of drp_antialias_fwd / _bwd. */
int drp_antialias_state_size(int num_views, int height, int width, size_t* bytes);

/*
 * dr.antialias(color, rast, pos, tri) (diffrp/rendering/surface_deferred.py:775).
 * color (B, H, W, C); nbr from drp_antialias_topology or NULL (every edge
 * is treated as a silhouette).  The workspace is scratch for this call only.
 * aa_state (may be NULL; drp_antialias_state_size bytes, 256-byte aligned)
 * receives the list of pixels a blending pair touches; handing it to the
 * matching drp_antialias_bwd lets the backward evaluate only those pixels.
 */
int drp_antialias_fwd(void* workspace, size_t workspace_bytes, const float* color, int channels, const float* rast,
                      const float* pos, long long pos_view_stride, long long num_vertices, const int* tri,
                      long long num_triangles, const int* nbr, int num_views, int height, int width, float* out,
                      void* aa_state, void* stream);

/* Most num_views * num_triangles that drp_antialias_fwd_noalloc accepts
 * (its fixed scratch holds 32 bytes per triangle and view: 8 MiB). */
#define DRP_NOALLOC_AA_MAX_TRIANGLE_VIEWS 262144

/*
 * drp_antialias_fwd without a workspace argument, for callers that cannot
 * allocate device memory: a host whose GPU memory is handed out by someone
 * else's allocator or reserved up front (an engine or plugin host with a
 * fixed budget), or code that must not allocate at the call site.  It
 * allocates nothing: the per-triangle scratch is a fixed array inside this
 * library (8 MiB per GPU, held until the process exits), so the call rejects
 * num_views * num_triangles above DRP_NOALLOC_AA_MAX_TRIANGLE_VIEWS with
 * DRP_STATUS_INVALID_ARGUMENT.  Same arguments and output as
 * drp_antialias_fwd, except that num_views above 65535 and num_views *
 * height * width above 2^31 - 1 are rejected the same way.  The first call
 * on each device looks up the array's device address (cudaGetSymbolAddress)
 * -- make that first call before any stream capture.  The address is kept
 * with the id of the CUDA context it was found in; a call in a new context
 * (after cudaDeviceReset, say) looks it up again, so make the first call
 * after a reset before any capture too.  All calls share the one array: calls whose GPU work
 * overlaps (different streams, or threads without ordering) race on it.
 * No counterpart in the reference: dr.antialias always allocates its own
 * buffers.
 */
int drp_antialias_fwd_noalloc(const float* color, int channels, const float* rast, const float* pos,
                              long long pos_view_stride, long long num_vertices, const int* tri,
                              long long num_triangles, const int* nbr, int num_views, int height, int width,
                              float* out, void* stream);

/* Backward: grad_color overwritten, grad_pos accumulated (times
 * pos_gradient_boost); grad_pos may be NULL.  aa_state: NULL, or the state
 * the forward on the same color / rast / pos filled. */
int drp_antialias_bwd(void* workspace, size_t workspace_bytes, const float* color, int channels, const float* rast,
                      const float* pos, long long pos_view_stride, long long num_vertices, const int* tri,
                      long long num_triangles, const int* nbr, int num_views, int height, int width,
                      const float* grad_out, float pos_gradient_boost, float* grad_color, float* grad_pos,
                      const void* aa_state, void* stream);

/* ------------------------------------------------------------------------ */
/* Edge-gradient visibility operator                                         */
/* ------------------------------------------------------------------------ */

/*
 * Backward of _EdgeGradient (diffrp/rendering/surface_deferred.py:126-169),
 * the operator behind SurfaceDeferredRenderSession.edge_gradient
 * (:777-804).  All buffers are in the bottom-up rast frame: frag_xy (H, W, 2)
 * fragment NDC positions, tris_xy (F, 3, 2) triangle NDC vertices, rast
 * (H, W, 4), rgb and grad_out (H, W, C).  grad_frag_xy (H, W, 2) is
 * overwritten.
 */
int drp_edge_gradient_bwd(const float* frag_xy, const float* tris_xy, long long num_triangles, const float* rast,
                          const float* rgb, int channels, const float* grad_out, int height, int width,
                          float* grad_frag_xy, void* stream);

/* ------------------------------------------------------------------------ */
/* Fused image loss                                                          */
/* ------------------------------------------------------------------------ */

/* Workspace bytes for drp_l1_loss_fwd over n elements. */
int drp_l1_loss_workspace_size(long long n, size_t* bytes);

/*
 * loss = scale * sum |pred - target| and grad = scale * sign(pred - target)
 * (0 at ties) in one pass over n elements; loss is one device float.  The
 * mean-absolute-error image loss the benchmark fits renders with (no
 * counterpart in the reference, which leaves losses to the user).
 */
int drp_l1_loss_fwd(void* workspace, size_t workspace_bytes, const float* pred, const float* target, long long n,
                    float scale, float* loss, float* grad, void* stream);

/* ------------------------------------------------------------------------ */
/* Clip-space transform                                                     */
/* ------------------------------------------------------------------------ */

/*
 * out[b * V + i] = M_b [v_i, 1] for V float32 xyz vertices and num_views
 * (<= 65535) row-major 4x4 matrices; out is 16-byte aligned float4 rows.
 * Replaces SurfaceDeferredRenderSession.clip_space
 * (diffrp/rendering/surface_deferred.py:229-238) through transform_point
 * (diffrp/utils/shader_ops.py:123-136), one small GEMM per view there.
 */
int drp_transform_points_fwd(const float* verts, long long num_vertices, const float* mats, int num_views,
                             float* out, void* stream);

/*
 * grad_verts[i] = sum over b (in view order) of M_b[:, :3]^T grad_out[b * V + i]:
 * writes (does not accumulate) V x 3 floats; grad_out as out above.
 */
int drp_transform_points_bwd(const float* grad_out, long long num_vertices, const float* mats, int num_views,
                             float* grad_verts, void* stream);

/* ------------------------------------------------------------------------ */
/* Mip-mapped texture sampling: the consumer of interpolate's screen-space  */
/* derivatives (uv_da), nvdiffrast's dr.texture as this project fixes it,   */
/* for the texture lookups of diffrp's materials (reference:                */
/* diffrp/materials/gltf_material.py:47-48 through                          */
/* diffrp/utils/shader_ops.py:224 sample2d, which samples without mipmaps). */
/* ------------------------------------------------------------------------ */
/*
 * Texture tex (num_tex, height, width, channels) float32; level 0 is tex
 * itself, levels 1 .. levels-1 live in a caller buffer `pyr` of
 * drp_texture_pyramid_floats() floats, level-major (level k: (num_tex, H_k,
 * W_k, channels), H_k = max(1, H_{k-1} >> 1)), filled by
 * drp_texture_mip_build (2x2 box average, indices clamped).
 * Sampling: uv (num_views, out_height, out_width, 2), texel (x, y) centred
 * at ((x + 0.5) / W, (y + 0.5) / H); uv_da (num_views, out_height,
 * out_width, 4) = (du/dX, du/dY, dv/dX, dv/dY), 16-byte aligned, or NULL.
 * mip_level_bias (num_views, out_height, out_width), or NULL: added to
 * the level of detail (alone, it sets it).  num_tex is 1 (shared) or
 * num_views.  filter_mode: 0 nearest, 1 linear, 2 linear-mipmap-nearest,
 * 3 linear-mipmap-linear (level of detail 0.5 log2 of the larger squared
 * footprint in level-0 texels, plus the bias, clamped to the pyramid).  boundary_mode: 0 wrap, 1 clamp, 2 zero, 3 mirror (mirrored
 * repeat: period 2 x size, the second half reversed).  Textures of at most
 * 32768 x 32768.
 */
int drp_texture_levels(int height, int width, int max_mip_level, int* levels);
int drp_texture_pyramid_floats(int num_tex, int height, int width, int channels, int levels, long long* floats);
int drp_texture_mip_build(const float* tex, int num_tex, int height, int width, int channels, int levels,
                          float* pyr, void* stream);
int drp_texture_fwd(const float* tex, const float* pyr, int num_tex, int height, int width, int channels,
                    int levels, const float* uv, const float* uv_da, const float* mip_level_bias, int num_views,
                    int out_height, int out_width, int filter_mode, int boundary_mode, float* out, void* stream);
/*
 * Backward of drp_texture_fwd (and of the pyramid): grad_tex (tex layout) is
 * accumulated (caller zeroes); grad_pyr is scratch of the pyramid's size
 * (zeroed and consumed by the call); grad_uv (uv layout) is written;
 * grad_uv_da (uv_da layout, may be NULL) and grad_mip_level_bias
 * (mip_level_bias layout, may be NULL) are written -- nonzero only for
 * linear-mipmap-linear where the level of detail is not clamped.
 */
int drp_texture_bwd(const float* tex, const float* pyr, int num_tex, int height, int width, int channels,
                    int levels, const float* uv, const float* uv_da, const float* mip_level_bias, int num_views,
                    int out_height, int out_width, int filter_mode, int boundary_mode, const float* grad_out,
                    float* grad_tex, float* grad_pyr, float* grad_uv, float* grad_uv_da,
                    float* grad_mip_level_bias, void* stream);

/* ------------------------------------------------------------------------ */
/* Host transport (no counterpart in the reference, which leaves transfers  */
/* to torch)                                                                */
/* ------------------------------------------------------------------------ */

/* Device address of mapped pinned host memory (cudaHostAlloc /
 * cudaHostRegister memory; every such allocation is mapped under unified
 * addressing).  DRP_STATUS_INVALID_ARGUMENT, and *device = NULL, for memory
 * that is not. */
int drp_host_device_pointer(const void* host, void** device);

/* Copy `bytes` bytes between non-overlapping buffers with a kernel (16-byte
 * vectors when both ends are 16-byte aligned), stream-ordered.  Either end may be device memory or the
 * device address of mapped pinned host memory: on a coherent host link the
 * SMs move a few hundred kilobytes faster than a copy engine transfer. */
int drp_copy_async(void* dst, const void* src, size_t bytes, void* stream);

/* ------------------------------------------------------------------------ */
/* Batching form: many (mesh, view, resolution) items per launch             */
/* ------------------------------------------------------------------------ */

/*
 * One item = one render of a mesh from one view at its own resolution.  The
 * caller fills the first group of fields; drp_batch_plan fills the rest.
 * Packed buffers: pos (rows of float4 clip vertices, the item's vertex 0 at
 * row pos_offset), tri (int32 triples, the item's mesh triangles at
 * [tri_first, tri_first + tri_count), vertex indices local to the item),
 * attr (floats, the mesh's V x channels attributes from attr_offset), and the
 * per-item outputs at pixel_offset (rast rows) / image_offset (floats).
 * No counterpart in the reference: diffrp renders one session (one view) per
 * call; this is the batched form of the same rasterize -> interpolate ->
 * antialias chain (rast, interpolated colour and antialiased output per item
 * are identical to the per-item calls).
 */
typedef struct drp_batch_item {
    long long pos_offset;   /* in float4 rows */
    long long attr_offset;  /* in floats */
    int tri_first, tri_count, num_vertices, height, width, channels;
    /* filled by drp_batch_plan: */
    int tiles_x, tiles_y;
    long long prim_offset, tile_offset, pixel_offset, image_offset;
} drp_batch_item;

/* Fill the derived fields of items[] (in place, host memory) for the given
 * tile size; totals[6] = {primitives, tiles, pixels, image floats,
 * primitive blocks, pixel blocks}. */
int drp_batch_plan(drp_batch_item* items, int num_items, int tile_log2, long long* totals);

/* Host-side block maps (int pairs: item, block within the item) of 256
 * triangle slots / 256 pixels; sizes from totals[4] / totals[5].  The
 * launches take at most (2^31 - 1) / 4 triangle blocks (each is set up by
 * four CTAs) and 2^31 - 1 pixel blocks. */
int drp_batch_block_maps(const drp_batch_item* items, int num_items, int* prim_block_map, int* pixel_block_map);

int drp_batch_workspace_size(long long total_prims, long long total_tiles, unsigned long long list_capacity,
                             size_t* bytes);

/*
 * Forward of every item: rasterise (persistent CTAs over an (item, tile)
 * work queue), interpolate attr into colour (fused), antialias into out.
 * items / block maps are device copies.  nbr: per-mesh topology from
 * drp_antialias_topology at the mesh's triangle offset, or NULL.  out may be
 * NULL: then only rast and colour are written (the antialias pass and its
 * triangle records are skipped), which is how a backward without stored
 * per-pixel buffers regenerates them.
 * bin_depth 0: exact tile lists (count, scan, fill; list_capacity entries);
 * the workspace's stats then hold the total list entries (u64 at byte 0) and
 * the largest tile count (u32 at byte 12).  bin_depth > 0: one setup pass
 * appends to fixed-depth bins (list_capacity >= total_tiles * bin_depth);
 * a tile with more entries is still rasterised exactly (by scanning all of
 * its item's triangles), sets DRP_DEVERR_LIST_OVERFLOW (u32 at byte 8) and
 * raises the u32 at byte 12 to its count.
 * aa_state (may be NULL; drp_batch_aa_state_size(total_pixels) bytes,
 * 256-byte aligned): the antialias pass records there which pixels a
 * blending pair touches (a flag per pixel and a list of them), so that
 * drp_batch_backward evaluates the antialias terms of those pixels only.
 */
int drp_batch_forward(void* workspace, size_t workspace_bytes, const drp_batch_item* items, int num_items,
                      const int* prim_block_map, long long prim_blocks, const int* pixel_block_map,
                      long long pixel_blocks, long long total_prims, long long total_tiles, const float* pos,
                      const int* tri, const float* attr, const int* nbr, int tile_log2, int threads_per_tri,
                      unsigned long long list_capacity, unsigned bin_depth, float* rast, float* color, float* out,
                      void* aa_state, long long total_pixels, void* stream);

/* Bytes of the antialias state block of drp_batch_forward (total_pixels =
 * totals[2] of drp_batch_plan). */
int drp_batch_aa_state_size(long long total_pixels, size_t* bytes);

/*
 * drp_batch_forward with the mean-absolute-error loss against target (image
 * floats, item layout) fused into the antialias pass: out (may be NULL) gets
 * the antialiased images, grad = sign(out - target) * scale, loss (one
 * float, device) = scale * sum |out - target|, reduced through block_loss
 * (pixel_blocks floats of scratch) in a fixed order.  The other arguments and
 * the workspace are those of drp_batch_forward.  No counterpart in the
 * reference: its L1 objective is separate PyTorch code after the render.
 */
int drp_batch_forward_l1(void* workspace, size_t workspace_bytes, const drp_batch_item* items, int num_items,
                         const int* prim_block_map, long long prim_blocks, const int* pixel_block_map,
                         long long pixel_blocks, long long total_prims, long long total_tiles, const float* pos,
                         const int* tri, const float* attr, const int* nbr, int tile_log2, int threads_per_tri,
                         unsigned long long list_capacity, unsigned bin_depth, float* rast, float* color, float* out,
                         void* aa_state, long long total_pixels, const float* target, float scale, float* grad,
                         float* block_loss, float* loss, void* stream);

/*
 * drp_batch_forward_l1 that also forms the gradient of the loss in the same
 * pass: grad_pos (pos layout) and grad_attr (attr layout), both accumulated
 * (caller zeroes), receive d loss / d pos and d loss / d attr -- the
 * gradients drp_batch_backward gives for grad_out = sign(out - target) *
 * scale.  The pixels no blending pair touches get their backward inside the
 * antialias + loss kernel (their rast row and signs at hand, no gradient
 * image written); the listed ones in a second kernel that forms the sign from
 * out and target and whose last block also forms the loss, the next launch
 * on the caller's stream.  block_loss holds pixel_blocks floats.  out and
 * aa_state are required; no sign-gradient image
 * is written.  At most 32 channels per item (an item with more sets
 * DRP_DEVERR_CHANNELS in the stats block and gets no gradient).  A caller
 * whose loss is the only consumer of the images can then skip the backward
 * pass entirely: multiply the two gradients by the loss's upstream gradient
 * (drp_scale_floats).  zero_first / zero_floats (may be NULL / 0): floats
 * the call zeroes before anything is accumulated -- the gradient buffers,
 * when the caller wants them started at zero (in its first kernel, instead
 * of a separate fill).  No counterpart in the reference.
 */
int drp_batch_forward_l1_grad(void* workspace, size_t workspace_bytes, const drp_batch_item* items, int num_items,
                              const int* prim_block_map, long long prim_blocks, const int* pixel_block_map,
                              long long pixel_blocks, long long total_prims, long long total_tiles, const float* pos,
                              const int* tri, const float* attr, const int* nbr, int tile_log2, int threads_per_tri,
                              unsigned long long list_capacity, unsigned bin_depth, float* rast, float* color,
                              float* out, void* aa_state, long long total_pixels, const float* target, float scale,
                              float* block_loss, float* loss, float* grad_pos, float* grad_attr, float* zero_first,
                              long long zero_floats, void* stream);

/*
 * dst[i] = src[i] * scale[0] for n floats (scale: one device float), dst and
 * src 4-byte aligned, the same buffer or disjoint: the backward of a loss
 * whose gradient drp_batch_forward_l1_grad formed, scaled by the loss's
 * upstream gradient without a host read.  No counterpart in the reference.
 */
int drp_scale_floats(float* dst, const float* src, long long n, const float* scale, void* stream);

/* drp_batch_backward flag: the workspace still holds the antialias triangle
 * records of the last drp_batch_forward, which ran on the same positions
 * (nothing else used the workspace since): they are not recomputed. */
#define DRP_BATCH_REUSE_AA_RECORDS 1

/* Fused backward: grad_out (image floats) -> grad_pos (accumulated, pos
 * layout) and grad_attr (accumulated, attr layout).  aa_state: NULL, or the
 * block the forward filled for this rast; then the listed pixels get their
 * whole backward (antialias terms, interpolation, rasterisation) in one
 * kernel, forked onto a library-owned side stream (one per host thread and
 * device, joined back before the call's work ends on `stream`; inside a
 * stream capture the fork and join are graph edges), while the other pixels,
 * which have no antialias terms, run the fused backward on `stream`.  aa_grad
 * is ignored (may be NULL).  grad_scale: NULL, or a device float every
 * grad_out value is multiplied by as it is read (the upstream gradient of
 * drp_batch_forward_l1's loss).  flags: 0 or DRP_BATCH_REUSE_AA_RECORDS. */
int drp_batch_backward(void* workspace, size_t workspace_bytes, const drp_batch_item* items, int num_items,
                       const int* prim_block_map, long long prim_blocks, const int* pixel_block_map,
                       long long pixel_blocks, long long total_prims, long long total_tiles, const float* pos,
                       const int* tri, const float* attr, const int* nbr, const float* rast, const float* color,
                       const void* aa_state, long long total_pixels, float* aa_grad, const float* grad_out,
                       float* grad_pos, float* grad_attr, const float* grad_scale, int flags, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* DIFFRP_GB300_H */
