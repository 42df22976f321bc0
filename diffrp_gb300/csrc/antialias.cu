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
// atomics, one pair per owner pixel.  A per-triangle setup pass first stores
// each triangle's screen-space vertices and silhouette-edge mask (32 bytes).
#include "aa_core.cuh"
#include "drp_internal.h"

namespace drp {

// ---------------------------------------------------------------------------
// Topology: open-addressing hash of undirected edges -> the (at most two)
// triangle edges that use it.  When exactly two distinct triangles share the
// edge k of triangle t (between its vertices k+1 and k+2), opp[3t + k] is the
// other triangle's vertex opposite that edge -- tri[e'] for the other
// triangle edge e' = 3t' + k', since vertex k' is opposite edge k' -- else -1.
// The silhouette test needs only that vertex, so the per-view triangle setup
// reads one index per edge instead of the neighbour's three.
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
                    if (other / 3 != (int)t) out = tri[other];
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
    drp_note_launch();
    topo_resolve_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(tri, F, keys, cnt, slots, cap - 1, nbr);
    drp_note_launch();
    return 0;
}

__global__ void __launch_bounds__(256) aa_setup_kernel(AAArgs a) {
    const int b = blockIdx.y;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.num_triangles) return;
    float4* rec = reinterpret_cast<float4*>(a.tri_rec) + ((long long)b * a.num_triangles + t) * 2;
    const float4* P = reinterpret_cast<const float4*>(a.pos + (long long)b * a.pos_view_stride);
    aa_tri_record(P, a.tri, a.nbr, t, a.num_triangles, a.num_vertices, a.W, a.H, rec);
}

__global__ void __launch_bounds__(256) aa_fwd_kernel(AAArgs a) {
    const int b = blockIdx.y;
    const int npix = a.H * a.W;
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = pix < npix;
    unsigned bits = 0;
    if (in) {
        const float4* R = reinterpret_cast<const float4*>(a.rast) + (long long)b * npix;
        const float* Cc = a.color + (long long)b * npix * a.C;
        const float4* rec = reinterpret_cast<const float4*>(a.tri_rec) + (long long)b * a.num_triangles * 2;
        aa_fwd_pixel<true>(R, Cc, rec, a.num_triangles, a.W, a.H, a.C, pix,
                           a.out + ((long long)b * npix + pix) * a.C, &bits);
    }
    if (!a.list) return;
    // warp-aggregated append of the pixels some blending pair touches
    const bool need = in && bits != 0u;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (!m) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(a.list_count, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (need) a.list[base + __popc(m & ((1u << lane) - 1u))] = b * npix + pix;
}

// With the forward's pixel list the colour gradient is the incoming one
// everywhere (this pass) except at the listed pixels (aa_bwd_list_kernel,
// launched after it, overwrites them).
__global__ void __launch_bounds__(256) aa_grad_copy_kernel(AAArgs a) {
    const long long n = (long long)a.B * a.H * a.W * a.C;
    const long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 4;
    if ((((uintptr_t)a.grad_out | (uintptr_t)a.grad_color) & 15) == 0) {
        if (i + 4 <= n) {
            *reinterpret_cast<float4*>(a.grad_color + i) = *reinterpret_cast<const float4*>(a.grad_out + i);
            return;
        }
    }
    for (long long k = i; k < i + 4 && k < n; ++k) a.grad_color[k] = a.grad_out[k];
}

// One quad of lanes per listed pixel: lane q evaluates pair slot q (and
// scatters its edge gradient when it owns the pair); the quad exchanges the
// slot terms by shuffles and shares the channels (c = q, q + 4, ...).
__global__ void __launch_bounds__(256) aa_bwd_list_kernel(AAArgs a) {
    const unsigned n = *a.list_count;
    const int npix = a.H * a.W, W = a.W, H = a.H, C = a.C;
    const int lane = threadIdx.x & 31, q = lane & 3, qbase = lane & ~3;
    const long long quads = ((long long)gridDim.x * blockDim.x) >> 2;
    for (long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 2;; i += quads) {
        const bool active = i < n;
        if (!__any_sync(0xffffffffu, active)) break;  // warp-uniform exit (quads step together)
        int role = 0, tgt = 0, b = 0, pix = 0;
        float wt = 0.f;
        if (active) {
            const int g = a.list[i];
            b = g / npix;
            pix = g - b * npix;
            const int py = pix / W, px = pix - py * W;
            int A, B, ax, ay;
            bool vert;
            if (pair_slot(q, pix, px, py, W, H, A, B, ax, ay, vert)) {
                const float4* R = reinterpret_cast<const float4*>(a.rast) + (long long)b * npix;
                const float4 rs = R[pix], ro = R[A == pix ? B : A];
                if (ro.w != rs.w) {
                    AAPair p;
                    const float4* rec = reinterpret_cast<const float4*>(a.tri_rec) + (long long)b * a.num_triangles * 2;
                    aa_pair(rec, a.num_triangles, A, B, ax, ay, vert, A == pix ? rs : ro, A == pix ? ro : rs, p);
                    if (p.valid) {
                        role = p.target == pix ? 1 : 2;
                        tgt = p.target;
                        wt = p.w;
                        if (a.grad_pos && A == pix && !p.clamped)
                            aa_edge_grad(p, a.color + (long long)b * npix * C, a.grad_out + (long long)b * npix * C, C,
                                         reinterpret_cast<const float4*>(a.pos + (long long)b * a.pos_view_stride),
                                         a.tri, reinterpret_cast<float4*>(a.grad_pos + (long long)b * a.pos_view_stride),
                                         a.boost, 1.0f, W, H);
                    }
                }
            }
        }
        AATerms at;
        at.any = false;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            at.role[k] = __shfl_sync(0xffffffffu, role, qbase | k);
            at.tgt[k] = __shfl_sync(0xffffffffu, tgt, qbase | k);
            at.wt[k] = __shfl_sync(0xffffffffu, wt, qbase | k);
            at.any = at.any || at.role[k] != 0;
        }
        if (active) {
            const float* Gd = a.grad_out + (long long)b * npix * C;
            float* gc = a.grad_color + ((long long)b * npix + pix) * C;
            for (int c = q; c < C; c += 4) gc[c] = aa_bwd_channel(at, Gd, C, pix, c);
        }
    }
}

__global__ void __launch_bounds__(256) aa_bwd_kernel(AAArgs a) {
    const int b = blockIdx.y;
    const int npix = a.H * a.W;
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    const int C = a.C;
    const float4* R = reinterpret_cast<const float4*>(a.rast) + (long long)b * npix;
    const float* Cc = a.color + (long long)b * npix * C;
    const float* Gd = a.grad_out + (long long)b * npix * C;
    const float4* P = reinterpret_cast<const float4*>(a.pos + (long long)b * a.pos_view_stride);
    float4* GP = a.grad_pos ? reinterpret_cast<float4*>(a.grad_pos + (long long)b * a.pos_view_stride) : nullptr;
    const float4* rec = reinterpret_cast<const float4*>(a.tri_rec) + (long long)b * a.num_triangles * 2;
    float* gc = a.grad_color + ((long long)b * npix + pix) * C;
    const float* gs = Gd + (long long)pix * C;
    AATerms at;
    aa_bwd_terms(R, Cc, Gd, rec, a.num_triangles, a.W, a.H, C, P, a.tri, GP, a.boost, pix, at);
    if (!at.any) {
        if ((C & 3) == 0 && (((uintptr_t)gs | (uintptr_t)gc) & 15) == 0) {
            for (int c = 0; c < C; c += 4)
                *reinterpret_cast<float4*>(gc + c) = *reinterpret_cast<const float4*>(gs + c);
        } else {
            for (int c = 0; c < C; ++c) gc[c] = gs[c];
        }
        return;
    }
    for (int c = 0; c < C; ++c) gc[c] = aa_bwd_channel(at, Gd, C, pix, c);
}

size_t aa_ws_bytes(int B, long long F) { return (size_t)B * (size_t)F * 32 + 256; }

size_t aa_state_bytes(int B, int H, int W) { return 256 + (size_t)B * (size_t)H * (size_t)W * 4; }

static void launch_aa_setup(const AAArgs& a, cudaStream_t s) {
    if (a.num_triangles <= 0) return;
    dim3 grid((unsigned)((a.num_triangles + 255) / 256), (unsigned)a.B);
    aa_setup_kernel<<<grid, 256, 0, s>>>(a);
    drp_note_launch();
}

int launch_aa_fwd(const AAArgs& a, cudaStream_t s) {
    const int npix = a.H * a.W;
    if (npix == 0) return 0;
    if (a.list_count) cudaMemsetAsync(a.list_count, 0, sizeof(unsigned), s);
    launch_aa_setup(a, s);
    dim3 grid((unsigned)((npix + 255) / 256), (unsigned)a.B);
    aa_fwd_kernel<<<grid, 256, 0, s>>>(a);
    drp_note_launch();
    return 0;
}

int launch_aa_bwd(const AAArgs& a, cudaStream_t s) {
    const int npix = a.H * a.W;
    if (npix == 0) return 0;
    launch_aa_setup(a, s);
    if (a.list_count) {
        const long long n4 = ((long long)a.B * npix * a.C + 3) / 4;
        aa_grad_copy_kernel<<<(unsigned)((n4 + 255) / 256), 256, 0, s>>>(a);
        drp_note_launch();
        const int sms = drp_current_sm_count();
        aa_bwd_list_kernel<<<(sms > 0 ? sms : 1) * 4, 256, 0, s>>>(a);
        drp_note_launch();
        return 0;
    }
    dim3 grid((unsigned)((npix + 255) / 256), (unsigned)a.B);
    aa_bwd_kernel<<<grid, 256, 0, s>>>(a);
    drp_note_launch();
    return 0;
}

}  // namespace drp

// ---------------------------------------------------------------------------
// drp_antialias_fwd_noalloc: the antialias forward for callers that cannot
// allocate device memory.  Its per-triangle scratch (the 32-byte screen-space
// records that drp_antialias_fwd keeps in a caller workspace) lives in the
// fixed array below, which every GPU that loads this library keeps for the
// life of the process.
// ---------------------------------------------------------------------------
#include <mutex>

#include "../../include/diffrp_gb300.h"

static __device__ __align__(256) float4 g_aa_noalloc_scratch[2 * DRP_NOALLOC_AA_MAX_TRIANGLE_VIEWS];

namespace {
std::mutex g_noalloc_mutex;
constexpr int kMaxDevices = 64;
struct NoallocAddr {
    unsigned long long ctx_id;  // the CUDA context the address belongs to (0: none cached)
    void* addr;
};
NoallocAddr g_noalloc_scratch_addr[kMaxDevices] = {};

// Unique id of the calling thread's current CUDA context, through the driver
// entry points the runtime hands out (no link-time dependency on libcuda).
// False when there is no current context or the entry points are missing.
bool current_context_id(unsigned long long* id) {
    typedef int (*GetCurrentFn)(void**);
    typedef int (*GetIdFn)(void*, unsigned long long*);
    static GetCurrentFn get_current = nullptr;
    static GetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetIdFn>(f);
    });
    if (!get_current || !get_id) return false;
    void* ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx) return false;
    return get_id(ctx, id) == 0 && *id != 0;
}

// Device address of the scratch array in the current device's context (host
// code may not use the array's name as a device address).  Looked up on the
// first call in each context and cached with that context's id: after a
// cudaDeviceReset the runtime makes a new primary context, the module is
// loaded again, and the address is looked up again.  Without context ids
// (driver entry points unavailable) it is looked up on every call.
int noalloc_scratch(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        drp_set_last_error("drp_antialias_fwd_noalloc: cudaGetDevice failed");
        return DRP_STATUS_CUDA_ERROR;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        drp_set_last_error("drp_antialias_fwd_noalloc: device ordinal out of range");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    unsigned long long id = 0;
    const bool have_id = current_context_id(&id);
    if (have_id && g_noalloc_scratch_addr[dev].ctx_id == id && g_noalloc_scratch_addr[dev].addr) {
        *out = g_noalloc_scratch_addr[dev].addr;
        return DRP_STATUS_OK;
    }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_aa_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        drp_set_last_error("drp_antialias_fwd_noalloc: cudaGetSymbolAddress of the scratch array failed");
        return DRP_STATUS_CUDA_ERROR;
    }
    // the lookup made the primary context current if it was not yet
    unsigned long long id_after = 0;
    if (current_context_id(&id_after)) g_noalloc_scratch_addr[dev] = NoallocAddr{id_after, p};
    else g_noalloc_scratch_addr[dev] = NoallocAddr{0, nullptr};
    *out = p;
    return DRP_STATUS_OK;
}
}  // namespace

extern "C" __attribute__((visibility("default"))) int drp_antialias_fwd_noalloc(
    const float* color, int channels, const float* rast, const float* pos, long long pos_view_stride,
    long long num_vertices, const int* tri, long long num_triangles, const int* nbr, int num_views, int height,
    int width, float* out, void* stream) {
    if (num_views <= 0 || height <= 0 || width <= 0 || height > DRP_MAX_RESOLUTION || width > DRP_MAX_RESOLUTION) {
        drp_set_last_error("drp_antialias_fwd_noalloc: bad views / resolution");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    if (channels <= 0 || num_triangles < 0 || num_vertices < 0 || pos_view_stride < 0 || (pos_view_stride % 4)) {
        drp_set_last_error("drp_antialias_fwd_noalloc: bad channels, sizes or stride");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    if (num_views > 65535) {
        drp_set_last_error("drp_antialias_fwd_noalloc: num_views above 65535");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    if ((long long)num_views * height * width > 0x7fffffffll) {
        drp_set_last_error("drp_antialias_fwd_noalloc: num_views * height * width above 2^31 - 1");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    if ((long long)num_views * num_triangles > DRP_NOALLOC_AA_MAX_TRIANGLE_VIEWS) {
        drp_set_last_error("drp_antialias_fwd_noalloc: num_views * num_triangles exceeds "
                           "DRP_NOALLOC_AA_MAX_TRIANGLE_VIEWS (262144); use drp_antialias_fwd with a workspace");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    if (!color || !rast || !pos || !tri || !out || (reinterpret_cast<uintptr_t>(rast) & 15) ||
        (reinterpret_cast<uintptr_t>(pos) & 15)) {
        drp_set_last_error("drp_antialias_fwd_noalloc: null or misaligned pointer");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    void* scratch = nullptr;
    const int st = noalloc_scratch(&scratch);
    if (st != DRP_STATUS_OK) return st;
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
    a.tri_rec = scratch;  // every record read by the pixel pass is written by the setup pass first
    a.B = num_views;
    a.H = height;
    a.W = width;
    a.out = out;
    drp::launch_aa_fwd(a, static_cast<cudaStream_t>(stream));
    return drp_check_launch("drp_antialias_fwd_noalloc");
}
