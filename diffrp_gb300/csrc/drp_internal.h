// drp_internal.h -- argument blocks passed from the C-ABI layer to the kernel
// launchers.  Not part of the public interface (see include/diffrp_gb300.h).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace drp {

// Launch `kernel` on `s` with programmatic stream serialisation allowed: it
// may start before the previous kernel in the stream ends, and waits for it
// with pdl_wait() (drp_common.cuh) before touching memory.  Only for kernels
// that call pdl_wait() first.  After a non-kernel operation (memset, event,
// copy) the launch serialises as usual.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Tile-count scan: chunks of kScanChunk tiles, one block of kScanThreads each.
constexpr int kScanThreads = 256;
constexpr int kScanPerThread = 16;
constexpr int kScanChunk = kScanThreads * kScanPerThread;
__host__ __device__ inline long long scan_chunks(long long n) { return (n + kScanChunk - 1) / kScanChunk; }

// Device scratch carved out of the caller-provided rasterisation workspace.
struct RasterWs {
    void* prims;            // B * max_view_tris * 48 bytes
    uint32_t* tile_count;   // B * tiles
    uint32_t* tile_offset;  // B * tiles
    uint32_t* tile_cursor;  // B * tiles
    uint32_t* tile_list;    // list_capacity entries
    unsigned long long* chunk_sums;  // tile-scan chunk sums, ceil(B * tiles / 4096)
    uint32_t* stats;        // [0..1] total list entries (u64), [2] device error bits, [3] largest tile count
};

struct RasterArgs {
    const float* pos;
    long long pos_view_stride;  // floats between views, 0 = shared vertices
    long long num_vertices;
    const int* tri;
    long long num_triangles;
    const int* ranges;  // device [B][2] (first, count) or null = all triangles
    int B;
    long long max_view_tris;
    int H, W;
    int tiles_x, tiles_y, tile_log2, threads_per_tri;
    unsigned long long list_capacity;
    uint32_t bin_depth;  // 0: exact tile lists (count, scan, fill); > 0: fixed-depth bins (one pass)
    const unsigned long long* prev_key;
    float* rast;
    float* rast_db;
    unsigned long long* out_key;
    RasterWs ws;
    const uint32_t* tile_order = nullptr;  // fine-raster block -> tile (null: identity)
};

struct RasterBwdArgs {
    const float* pos;
    long long pos_view_stride;
    long long num_vertices;
    long long num_triangles;
    const int* tri;
    const float* rast;
    const float* grad_rast;
    const float* grad_db;
    int B, H, W;
    float* grad_pos;
};

struct InterpArgs {
    const float* attr;
    long long attr_view_stride;  // floats between views, 0 = shared attributes
    long long num_vertices;
    int C;
    const float* rast;
    const float* rast_db;
    const int* tri;
    long long num_triangles;
    int B, H, W;
    const int* diff_idx;  // device, nd entries
    int nd;
    float* out;
    float* da;
    // backward
    const float* grad_out;
    const float* grad_da;
    float* grad_attr;
    float* grad_rast;
    float* grad_db;
};

struct SparseInterpArgs {
    const float* vb;
    long long V;
    int C;
    const float* vi;          // N x 4
    const long long* tri_idx; // N x 3
    long long N;
    float* out;
    const float* grad_out;
    float* grad_vb;
    float* grad_vi;
};

struct AAArgs {
    const float* color;
    int C;
    const float* rast;
    const float* pos;
    long long pos_view_stride;
    long long num_vertices;
    long long num_triangles;
    const int* tri;
    const int* nbr;  // F x 3 neighbour table or null (every edge a silhouette)
    void* tri_rec;   // workspace: B x F x 32-byte per-triangle records
    int B, H, W;
    float* out;
    const float* grad_out;
    float* grad_color;
    float* grad_pos;
    float boost;
    // optional pixel list (forward appends every pixel a blending pair
    // touches; the backward then evaluates the antialias terms of those only)
    unsigned* list_count;
    int* list;
};

// Bytes of the drp_antialias_fwd / _bwd pixel-list state for B views of H x W.
size_t aa_state_bytes(int B, int H, int W);

int launch_rasterize(const RasterArgs& a, cudaStream_t s);
int launch_raster_bwd(const RasterBwdArgs& a, cudaStream_t s);
int launch_interp_fwd(const InterpArgs& a, cudaStream_t s);
int launch_interp_bwd(const InterpArgs& a, cudaStream_t s);
int launch_interp_sparse_fwd(const SparseInterpArgs& a, cudaStream_t s);
int launch_interp_sparse_bwd(const SparseInterpArgs& a, cudaStream_t s);
int launch_topology(const int* tri, long long F, void* ws, size_t ws_bytes, int* nbr, cudaStream_t s);
size_t topology_ws_bytes(long long F);
size_t aa_ws_bytes(int B, long long F);
int launch_aa_fwd(const AAArgs& a, cudaStream_t s);
int launch_aa_bwd(const AAArgs& a, cudaStream_t s);

// loss = scale * (sum of nblocks partial sums).  One block of kFinalThreads
// adds the partials as (sum, error) float pairs with TwoSum, in a fixed order
// (per thread, then by shuffles, then across warps; l1_final_block), so the
// result is reproducible from run to run.
void launch_l1_final(const float* partial, long long nblocks, float scale, float* loss, cudaStream_t s);

}  // namespace drp

// Thread-local error message of the C ABI (capi.cu).
void drp_set_last_error(const char* msg);
// DRP_STATUS_OK, or DRP_STATUS_CUDA_ERROR with the message set, after a launch.
int drp_check_launch(const char* what);
// Count one kernel launch enqueued by this library (drp_kernel_launches).
void drp_note_launch();
// Multiprocessors of the current device, cached per device (0 without one).
int drp_current_sm_count();
