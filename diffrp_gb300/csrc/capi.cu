// capi.cu -- extern "C" entry points declared in include/diffrp_gb300.h.
// Host-side validation (sizes, null pointers, alignment, workspace size) and
// the launch of the kernels in raster.cu / interp.cu / antialias.cu.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "../../include/diffrp_gb300.h"
#include "drp_common.cuh"
#include "drp_internal.h"

#define DRP_API extern "C" __attribute__((visibility("default")))

namespace {

thread_local char g_last_error[512] = "";

int fail(int status, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return status;
}

int check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(DRP_STATUS_CUDA_ERROR, "%s: %s", what, cudaGetErrorString(e));
    g_last_error[0] = 0;
    return DRP_STATUS_OK;
}

bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

bool res_ok(int h, int w) { return h > 0 && w > 0 && h <= DRP_MAX_RESOLUTION && w <= DRP_MAX_RESOLUTION; }

struct RasterLayout {
    size_t stats, prims, count, offset, cursor, chunks, list, total;
};

RasterLayout raster_layout(int B, long long maxT, int H, int W, int tile_log2, unsigned long long cap) {
    const long long tx = (W + (1 << tile_log2) - 1) >> tile_log2;
    const long long ty = (H + (1 << tile_log2) - 1) >> tile_log2;
    const size_t ntiles = (size_t)B * (size_t)(tx * ty);
    RasterLayout L;
    L.stats = 0;
    L.prims = 256;
    L.count = align_up(L.prims + (size_t)B * (size_t)maxT * 48, 256);
    L.offset = align_up(L.count + ntiles * 4, 256);
    L.cursor = align_up(L.offset + ntiles * 4, 256);
    L.chunks = align_up(L.cursor + ntiles * 4, 256);
    L.list = align_up(L.chunks + (size_t)drp::scan_chunks((long long)ntiles) * 8, 256);
    L.total = align_up(L.list + (size_t)cap * 4, 256);
    return L;
}

}  // namespace

void drp_set_last_error(const char* msg) { snprintf(g_last_error, sizeof(g_last_error), "%s", msg); }

int drp_check_launch(const char* what) { return check_launch(what); }

namespace {
std::atomic<unsigned long long> g_kernel_launches{0};
}

void drp_note_launch() { g_kernel_launches.fetch_add(1, std::memory_order_relaxed); }

namespace {
constexpr int kSmCacheDevices = 64;
std::atomic<int> g_sm_count[kSmCacheDevices];
}

int drp_current_sm_count() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 0;
    if (dev < kSmCacheDevices) {
        const int v = g_sm_count[dev].load(std::memory_order_relaxed);
        if (v > 0) return v;
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (dev < kSmCacheDevices && sms > 0) g_sm_count[dev].store(sms, std::memory_order_relaxed);
    return sms;
}

DRP_API unsigned long long drp_kernel_launches(void) { return g_kernel_launches.load(std::memory_order_relaxed); }

DRP_API int drp_abi_version(void) { return DRP_ABI_VERSION; }

DRP_API const char* drp_status_string(int status) {
    switch (status) {
    case DRP_STATUS_OK: return "ok";
    case DRP_STATUS_INVALID_ARGUMENT: return "invalid argument";
    case DRP_STATUS_WORKSPACE_TOO_SMALL: return "workspace too small";
    case DRP_STATUS_CUDA_ERROR: return "CUDA error";
    default: return "unknown status";
    }
}

DRP_API const char* drp_last_error(void) { return g_last_error; }

// ---------------------------------------------------------------------------
// Rasterisation
// ---------------------------------------------------------------------------
DRP_API int drp_raster_workspace_size(int num_views, long long max_view_tris, int height, int width, int tile_log2,
                                      unsigned long long list_capacity, size_t* bytes) {
    if (!bytes) return fail(DRP_STATUS_INVALID_ARGUMENT, "bytes is null");
    if (num_views < 0 || max_view_tris < 0) return fail(DRP_STATUS_INVALID_ARGUMENT, "negative size");
    if (!res_ok(height, width)) return fail(DRP_STATUS_INVALID_ARGUMENT, "resolution %dx%d out of range", height, width);
    if (tile_log2 < 3 || tile_log2 > 5) return fail(DRP_STATUS_INVALID_ARGUMENT, "tile_log2 must be 3, 4 or 5");
    if (list_capacity > 0x7fffffffull) return fail(DRP_STATUS_INVALID_ARGUMENT, "list_capacity above 2^31 - 1");
    *bytes = raster_layout(num_views, max_view_tris, height, width, tile_log2, list_capacity).total;
    return DRP_STATUS_OK;
}

DRP_API int drp_rasterize_fwd(void* workspace, size_t workspace_bytes, const float* pos, long long pos_view_stride,
                              long long num_vertices, const int* tri, long long num_triangles, int num_views,
                              const int* ranges, long long max_view_tris, int height, int width, int tile_log2,
                              int threads_per_tri, unsigned long long list_capacity, unsigned bin_depth,
                              const unsigned long long* prev_key, float* rast, float* rast_db,
                              unsigned long long* out_key, void* stream) {
    if (num_views <= 0) return fail(DRP_STATUS_INVALID_ARGUMENT, "num_views must be positive");
    if (!res_ok(height, width)) return fail(DRP_STATUS_INVALID_ARGUMENT, "resolution %dx%d out of range", height, width);
    if (tile_log2 < 3 || tile_log2 > 5) return fail(DRP_STATUS_INVALID_ARGUMENT, "tile_log2 must be 3, 4 or 5");
    if (threads_per_tri < 0 || threads_per_tri > 32 || (threads_per_tri & (threads_per_tri - 1)))
        return fail(DRP_STATUS_INVALID_ARGUMENT, "threads_per_tri must be 0 or a power of two in [1, 32]");
    if (num_vertices < 0 || num_triangles < 0 || max_view_tris < 0 || pos_view_stride < 0)
        return fail(DRP_STATUS_INVALID_ARGUMENT, "negative size");
    // The rast w channel encodes id + 1 as the float with bits 0x4a800000 + id + 1
    // above 2^24; it stays a finite positive float below id + 1 = 0x35000000.
    if (num_triangles >= 0x34ffffffll || num_vertices > 0x7fffffffll)
        return fail(DRP_STATUS_INVALID_ARGUMENT, "more than %lld triangles or 2^31 - 1 vertices", 0x34fffffell);
    if (!ranges && max_view_tris != num_triangles)
        return fail(DRP_STATUS_INVALID_ARGUMENT, "without ranges max_view_tris must equal num_triangles");
    if (max_view_tris > 0 && (!pos || !tri)) return fail(DRP_STATUS_INVALID_ARGUMENT, "pos / tri is null");
    if (!rast) return fail(DRP_STATUS_INVALID_ARGUMENT, "rast is null");
    if (!aligned(pos, 16) || !aligned(rast, 16) || !aligned(rast_db, 16) || !aligned(prev_key, 8) ||
        !aligned(out_key, 8) || (pos_view_stride % 4) != 0)
        return fail(DRP_STATUS_INVALID_ARGUMENT, "pos / rast / rast_db must be 16-byte aligned float4 rows");
    if (!workspace || !aligned(workspace, 256)) return fail(DRP_STATUS_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
    if (list_capacity > 0x7fffffffull) return fail(DRP_STATUS_INVALID_ARGUMENT, "list_capacity above 2^31 - 1");
    {
        const long long tiles = (long long)num_views * (((long long)width + (1 << tile_log2) - 1) >> tile_log2) *
                                (((long long)height + (1 << tile_log2) - 1) >> tile_log2);
        if (bin_depth && (unsigned long long)tiles * bin_depth > list_capacity)
            return fail(DRP_STATUS_INVALID_ARGUMENT, "list_capacity below tiles * bin_depth");
    }
    const RasterLayout L = raster_layout(num_views, max_view_tris, height, width, tile_log2, list_capacity);
    if (workspace_bytes < L.total)
        return fail(DRP_STATUS_WORKSPACE_TOO_SMALL, "raster workspace needs %zu bytes, got %zu", L.total, workspace_bytes);
    char* w = static_cast<char*>(workspace);
    drp::RasterArgs a;
    a.pos = pos;
    a.pos_view_stride = pos_view_stride;
    a.num_vertices = num_vertices;
    a.tri = tri;
    a.num_triangles = num_triangles;
    a.ranges = ranges;
    a.B = num_views;
    a.max_view_tris = max_view_tris;
    a.H = height;
    a.W = width;
    a.tile_log2 = tile_log2;
    a.tiles_x = (width + (1 << tile_log2) - 1) >> tile_log2;
    a.tiles_y = (height + (1 << tile_log2) - 1) >> tile_log2;
    a.threads_per_tri = threads_per_tri;
    a.list_capacity = list_capacity;
    a.bin_depth = bin_depth;
    a.prev_key = prev_key;
    a.rast = rast;
    a.rast_db = rast_db;
    a.out_key = out_key;
    a.ws.stats = reinterpret_cast<uint32_t*>(w + L.stats);
    a.ws.prims = w + L.prims;
    a.ws.tile_count = reinterpret_cast<uint32_t*>(w + L.count);
    a.ws.tile_offset = reinterpret_cast<uint32_t*>(w + L.offset);
    a.ws.tile_cursor = reinterpret_cast<uint32_t*>(w + L.cursor);
    a.ws.tile_list = reinterpret_cast<uint32_t*>(w + L.list);
    a.ws.chunk_sums = reinterpret_cast<unsigned long long*>(w + L.chunks);
    drp::launch_rasterize(a, static_cast<cudaStream_t>(stream));
    return check_launch("drp_rasterize_fwd");
}

DRP_API int drp_rasterize_bwd(const float* pos, long long pos_view_stride, long long num_vertices, const int* tri,
                              long long num_triangles, int num_views, int height, int width, const float* rast,
                              const float* grad_rast, const float* grad_db, float* grad_pos, void* stream) {
    if (num_views <= 0 || !res_ok(height, width)) return fail(DRP_STATUS_INVALID_ARGUMENT, "bad views / resolution");
    if (!pos || !tri || !rast || !grad_rast || !grad_pos) return fail(DRP_STATUS_INVALID_ARGUMENT, "null pointer");
    if (!aligned(pos, 16) || !aligned(rast, 16) || !aligned(grad_rast, 16) || !aligned(grad_db, 16) ||
        !aligned(grad_pos, 16) || (pos_view_stride % 4) != 0)
        return fail(DRP_STATUS_INVALID_ARGUMENT, "float4 rows must be 16-byte aligned");
    drp::RasterBwdArgs a;
    a.pos = pos;
    a.pos_view_stride = pos_view_stride;
    a.num_vertices = num_vertices;
    a.num_triangles = num_triangles;
    a.tri = tri;
    a.rast = rast;
    a.grad_rast = grad_rast;
    a.grad_db = grad_db;
    a.B = num_views;
    a.H = height;
    a.W = width;
    a.grad_pos = grad_pos;
    drp::launch_raster_bwd(a, static_cast<cudaStream_t>(stream));
    return check_launch("drp_rasterize_bwd");
}

// ---------------------------------------------------------------------------
// Interpolation
// ---------------------------------------------------------------------------
static int interp_common(const float* attr, long long attr_view_stride, int channels, const float* rast,
                         const float* rast_db, const int* tri, int num_views, int height, int width,
                         const int* diff_idx, int num_diff) {
    if (num_views <= 0 || num_views > 65535 || !res_ok(height, width))
        return fail(DRP_STATUS_INVALID_ARGUMENT, "bad views / resolution");
    if (channels <= 0) return fail(DRP_STATUS_INVALID_ARGUMENT, "channels must be positive");
    if (!attr || !rast || !tri) return fail(DRP_STATUS_INVALID_ARGUMENT, "null pointer");
    if (attr_view_stride < 0) return fail(DRP_STATUS_INVALID_ARGUMENT, "negative stride");
    if (num_diff < 0 || (num_diff > 0 && (!diff_idx || !rast_db)))
        return fail(DRP_STATUS_INVALID_ARGUMENT, "derivatives need diff_idx and rast_db");
    if (!aligned(rast, 16) || !aligned(rast_db, 16)) return fail(DRP_STATUS_INVALID_ARGUMENT, "rast must be 16-byte aligned");
    if ((channels & 3) == 0 && (!aligned(attr, 16) || (attr_view_stride % 4) != 0))
        return fail(DRP_STATUS_INVALID_ARGUMENT, "attr rows must be 16-byte aligned when channels % 4 == 0");
    return DRP_STATUS_OK;
}

DRP_API int drp_interpolate_fwd(const float* attr, long long attr_view_stride, long long num_vertices, int channels,
                                const float* rast, const float* rast_db, const int* tri, long long num_triangles,
                                int num_views, int height, int width, const int* diff_idx, int num_diff, float* out,
                                float* da, void* stream) {
    int st = interp_common(attr, attr_view_stride, channels, rast, rast_db, tri, num_views, height, width, diff_idx,
                           num_diff);
    if (st) return st;
    if (!out || (num_diff > 0 && !da)) return fail(DRP_STATUS_INVALID_ARGUMENT, "null output");
    if ((channels & 3) == 0 && !aligned(out, 16)) return fail(DRP_STATUS_INVALID_ARGUMENT, "out must be 16-byte aligned");
    drp::InterpArgs a{};
    a.attr = attr;
    a.attr_view_stride = attr_view_stride;
    a.num_vertices = num_vertices;
    a.C = channels;
    a.rast = rast;
    a.rast_db = rast_db;
    a.tri = tri;
    a.num_triangles = num_triangles;
    a.B = num_views;
    a.H = height;
    a.W = width;
    a.diff_idx = diff_idx;
    a.nd = num_diff;
    a.out = out;
    a.da = num_diff > 0 ? da : nullptr;
    drp::launch_interp_fwd(a, static_cast<cudaStream_t>(stream));
    return check_launch("drp_interpolate_fwd");
}

DRP_API int drp_interpolate_bwd(const float* attr, long long attr_view_stride, long long num_vertices, int channels,
                                const float* rast, const float* rast_db, const int* tri, long long num_triangles,
                                int num_views, int height, int width, const int* diff_idx, int num_diff,
                                const float* grad_out, const float* grad_da, float* grad_attr, float* grad_rast,
                                float* grad_db, void* stream) {
    int st = interp_common(attr, attr_view_stride, channels, rast, rast_db, tri, num_views, height, width, diff_idx,
                           num_diff);
    if (st) return st;
    if (!grad_out || !grad_attr) return fail(DRP_STATUS_INVALID_ARGUMENT, "null gradient pointer");
    if (!aligned(grad_rast, 16) || !aligned(grad_db, 16) || ((channels & 3) == 0 && !aligned(grad_attr, 16)))
        return fail(DRP_STATUS_INVALID_ARGUMENT, "gradient buffers must be 16-byte aligned");
    drp::InterpArgs a{};
    a.attr = attr;
    a.attr_view_stride = attr_view_stride;
    a.num_vertices = num_vertices;
    a.C = channels;
    a.rast = rast;
    a.rast_db = rast_db;
    a.tri = tri;
    a.num_triangles = num_triangles;
    a.B = num_views;
    a.H = height;
    a.W = width;
    a.diff_idx = diff_idx;
    a.nd = num_diff;
    a.grad_out = grad_out;
    a.grad_da = num_diff > 0 ? grad_da : nullptr;
    a.grad_attr = grad_attr;
    a.grad_rast = grad_rast;
    a.grad_db = grad_db;
    drp::launch_interp_bwd(a, static_cast<cudaStream_t>(stream));
    return check_launch("drp_interpolate_bwd");
}

static int sparse_common(const float* vb, int channels, const float* vi, const long long* tri_idx, long long n) {
    if (channels <= 0 || n < 0) return fail(DRP_STATUS_INVALID_ARGUMENT, "bad channels / n");
    if (n > 0 && (!vb || !vi || !tri_idx)) return fail(DRP_STATUS_INVALID_ARGUMENT, "null pointer");
    if (!aligned(vi, 16)) return fail(DRP_STATUS_INVALID_ARGUMENT, "vi_data must be 16-byte aligned");
    if ((channels & 3) == 0 && !aligned(vb, 16))
        return fail(DRP_STATUS_INVALID_ARGUMENT, "vertex_buffer must be 16-byte aligned when channels % 4 == 0");
    return DRP_STATUS_OK;
}

DRP_API int drp_interpolate_sparse_fwd(const float* vertex_buffer, long long num_vertices, int channels,
                                       const float* vi_data, const long long* tri_idx, long long n, float* out,
                                       void* stream) {
    int st = sparse_common(vertex_buffer, channels, vi_data, tri_idx, n);
    if (st) return st;
    if (n > 0 && !out) return fail(DRP_STATUS_INVALID_ARGUMENT, "null output");
    if ((channels & 3) == 0 && !aligned(out, 16)) return fail(DRP_STATUS_INVALID_ARGUMENT, "out must be 16-byte aligned");
    drp::SparseInterpArgs a{};
    a.vb = vertex_buffer;
    a.V = num_vertices;
    a.C = channels;
    a.vi = vi_data;
    a.tri_idx = tri_idx;
    a.N = n;
    a.out = out;
    drp::launch_interp_sparse_fwd(a, static_cast<cudaStream_t>(stream));
    return check_launch("drp_interpolate_sparse_fwd");
}

DRP_API int drp_interpolate_sparse_bwd(const float* vertex_buffer, long long num_vertices, int channels,
                                       const float* vi_data, const long long* tri_idx, long long n,
                                       const float* grad_out, float* grad_vb, float* grad_vi, void* stream) {
    int st = sparse_common(vertex_buffer, channels, vi_data, tri_idx, n);
    if (st) return st;
    if (n > 0 && (!grad_out || !grad_vb)) return fail(DRP_STATUS_INVALID_ARGUMENT, "null gradient pointer");
    if (!aligned(grad_vi, 16)) return fail(DRP_STATUS_INVALID_ARGUMENT, "grad_vi must be 16-byte aligned");
    drp::SparseInterpArgs a{};
    a.vb = vertex_buffer;
    a.V = num_vertices;
    a.C = channels;
    a.vi = vi_data;
    a.tri_idx = tri_idx;
    a.N = n;
    a.grad_out = grad_out;
    a.grad_vb = grad_vb;
    a.grad_vi = grad_vi;
    drp::launch_interp_sparse_bwd(a, static_cast<cudaStream_t>(stream));
    return check_launch("drp_interpolate_sparse_bwd");
}

// ---------------------------------------------------------------------------
// Antialiasing
// ---------------------------------------------------------------------------
DRP_API int drp_topology_workspace_size(long long num_triangles, size_t* bytes) {
    if (!bytes || num_triangles < 0) return fail(DRP_STATUS_INVALID_ARGUMENT, "bad arguments");
    *bytes = drp::topology_ws_bytes(num_triangles);
    return DRP_STATUS_OK;
}

DRP_API int drp_antialias_topology(void* workspace, size_t workspace_bytes, const int* tri, long long num_triangles,
                                   int* nbr, void* stream) {
    if (num_triangles < 0 || num_triangles > 0x2aaaaaa9ll)
        return fail(DRP_STATUS_INVALID_ARGUMENT, "num_triangles out of range");
    if (num_triangles == 0) return DRP_STATUS_OK;
    if (!workspace || !tri || !nbr) return fail(DRP_STATUS_INVALID_ARGUMENT, "null pointer");
    if (workspace_bytes < drp::topology_ws_bytes(num_triangles))
        return fail(DRP_STATUS_WORKSPACE_TOO_SMALL, "topology workspace needs %zu bytes",
                    drp::topology_ws_bytes(num_triangles));
    drp::launch_topology(tri, num_triangles, workspace, workspace_bytes, nbr, static_cast<cudaStream_t>(stream));
    return check_launch("drp_antialias_topology");
}

static int aa_common(const float* color, int channels, const float* rast, const float* pos, long long stride,
                     const int* tri, int num_views, int height, int width) {
    if (num_views <= 0 || num_views > 65535 || !res_ok(height, width))
        return fail(DRP_STATUS_INVALID_ARGUMENT, "bad views / resolution");
    if (channels <= 0) return fail(DRP_STATUS_INVALID_ARGUMENT, "channels must be positive");
    if (!color || !rast || !pos || !tri) return fail(DRP_STATUS_INVALID_ARGUMENT, "null pointer");
    if (!aligned(rast, 16) || !aligned(pos, 16) || stride < 0 || (stride % 4) != 0)
        return fail(DRP_STATUS_INVALID_ARGUMENT, "rast / pos must be 16-byte aligned float4 rows");
    return DRP_STATUS_OK;
}

DRP_API int drp_antialias_workspace_size(int num_views, long long num_triangles, size_t* bytes) {
    if (!bytes || num_views < 0 || num_triangles < 0) return fail(DRP_STATUS_INVALID_ARGUMENT, "bad arguments");
    *bytes = drp::aa_ws_bytes(num_views, num_triangles);
    return DRP_STATUS_OK;
}

static int aa_ws_check(void* workspace, size_t workspace_bytes, int num_views, long long num_triangles) {
    if (!workspace || !aligned(workspace, 16)) return fail(DRP_STATUS_INVALID_ARGUMENT, "workspace must be 16-byte aligned");
    if (workspace_bytes < drp::aa_ws_bytes(num_views, num_triangles))
        return fail(DRP_STATUS_WORKSPACE_TOO_SMALL, "antialias workspace needs %zu bytes",
                    drp::aa_ws_bytes(num_views, num_triangles));
    if ((long long)num_views * num_triangles * 2 > 0x7fffffffll * 16)
        return fail(DRP_STATUS_INVALID_ARGUMENT, "too many triangles x views");
    return DRP_STATUS_OK;
}

DRP_API int drp_antialias_state_size(int num_views, int height, int width, size_t* bytes) {
    if (num_views <= 0 || !res_ok(height, width) || !bytes) return fail(DRP_STATUS_INVALID_ARGUMENT, "bad arguments");
    *bytes = drp::aa_state_bytes(num_views, height, width);
    return DRP_STATUS_OK;
}

DRP_API int drp_antialias_fwd(void* workspace, size_t workspace_bytes, const float* color, int channels,
                              const float* rast, const float* pos, long long pos_view_stride, long long num_vertices,
                              const int* tri, long long num_triangles, const int* nbr, int num_views, int height,
                              int width, float* out, void* aa_state, void* stream) {
    int st = aa_common(color, channels, rast, pos, pos_view_stride, tri, num_views, height, width);
    if (st) return st;
    st = aa_ws_check(workspace, workspace_bytes, num_views, num_triangles);
    if (st) return st;
    if (!out) return fail(DRP_STATUS_INVALID_ARGUMENT, "null output");
    if (!aligned(aa_state, 256)) return fail(DRP_STATUS_INVALID_ARGUMENT, "aa_state must be 256-byte aligned");
    if ((long long)num_views * height * width > 0x7fffffffll)
        return fail(DRP_STATUS_INVALID_ARGUMENT, "num_views * height * width above 2^31 - 1");
    drp::AAArgs a{};
    a.color = color;
    a.C = channels;
    a.rast = rast;
    a.pos = pos;
    a.pos_view_stride = pos_view_stride;
    a.num_vertices = num_vertices;
    a.num_triangles = num_triangles;
    a.tri = tri;
    a.nbr = nbr;
    a.tri_rec = workspace;
    a.B = num_views;
    a.H = height;
    a.W = width;
    a.out = out;
    if (aa_state) {
        a.list_count = static_cast<unsigned*>(aa_state);
        a.list = reinterpret_cast<int*>(static_cast<char*>(aa_state) + 256);
    }
    drp::launch_aa_fwd(a, static_cast<cudaStream_t>(stream));
    return check_launch("drp_antialias_fwd");
}

DRP_API int drp_antialias_bwd(void* workspace, size_t workspace_bytes, const float* color, int channels,
                              const float* rast, const float* pos, long long pos_view_stride, long long num_vertices,
                              const int* tri, long long num_triangles, const int* nbr, int num_views, int height,
                              int width, const float* grad_out, float pos_gradient_boost, float* grad_color,
                              float* grad_pos, const void* aa_state, void* stream) {
    int st = aa_common(color, channels, rast, pos, pos_view_stride, tri, num_views, height, width);
    if (st) return st;
    st = aa_ws_check(workspace, workspace_bytes, num_views, num_triangles);
    if (st) return st;
    if (!grad_out || !grad_color) return fail(DRP_STATUS_INVALID_ARGUMENT, "null gradient pointer");
    if (!aligned(grad_pos, 16)) return fail(DRP_STATUS_INVALID_ARGUMENT, "grad_pos must be 16-byte aligned");
    drp::AAArgs a{};
    a.color = color;
    a.C = channels;
    a.rast = rast;
    a.pos = pos;
    a.pos_view_stride = pos_view_stride;
    a.num_vertices = num_vertices;
    a.num_triangles = num_triangles;
    a.tri = tri;
    a.nbr = nbr;
    a.tri_rec = workspace;
    a.B = num_views;
    a.H = height;
    a.W = width;
    a.grad_out = grad_out;
    a.grad_color = grad_color;
    a.grad_pos = grad_pos;
    a.boost = pos_gradient_boost;
    if (aa_state) {
        if (!aligned(aa_state, 256)) return fail(DRP_STATUS_INVALID_ARGUMENT, "aa_state must be 256-byte aligned");
        a.list_count = const_cast<unsigned*>(static_cast<const unsigned*>(aa_state));
        a.list = reinterpret_cast<int*>(static_cast<char*>(const_cast<void*>(aa_state)) + 256);
    }
    drp::launch_aa_bwd(a, static_cast<cudaStream_t>(stream));
    return check_launch("drp_antialias_bwd");
}
