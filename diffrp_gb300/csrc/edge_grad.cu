// edge_grad.cu -- backward of the edge-gradient visibility operator
// (_EdgeGradient.backward, diffrp/rendering/surface_deferred.py:126-169;
// "Rasterized Edge Gradients: Handling Discontinuities Differentiably").
//
// Forward is the identity on the image.  Backward, per pixel boundary whose
// triangle ids differ (horizontal and vertical neighbours of the bottom-up
// rast frame):
//   grad_edge = s * 0.5 * dot(g[a] + g[b], rgb[a] - rgb[b])   (s = +1 for x, -1 for y)
//   a receives grad_edge when its fragment lies in b's screen triangle (or b
//   is background); b receives it when its fragment lies in a's triangle (or a
//   is background).  The per-pixel sums are scaled by (W / 2, H / 2) into the
//   gradient of the fragment's NDC position.  One thread per pixel gathers
//   its (up to four) boundaries, so no atomics are needed.
#include "drp_common.cuh"
#include "drp_internal.h"

namespace drp {

// sign2d / point_in_tri2d of diffrp/utils/geometry.py:69-91, same operation order.
__device__ __forceinline__ float sign2d(float2 p1, float2 p2, float2 p3) {
    return (p1.x - p3.x) * (p2.y - p3.y) - (p2.x - p3.x) * (p1.y - p3.y);
}

__device__ __forceinline__ bool point_in_tri2d(float2 pt, float2 v1, float2 v2, float2 v3) {
    const float d1 = sign2d(pt, v1, v2), d2 = sign2d(pt, v2, v3), d3 = sign2d(pt, v3, v1);
    const bool neg = (d1 < 0.0f) || (d2 < 0.0f) || (d3 < 0.0f);
    const bool pos = (d1 > 0.0f) || (d2 > 0.0f) || (d3 > 0.0f);
    return !(neg && pos);
}

struct EdgeGradArgs {
    const float2* frag_xy;  // H x W
    const float2* tris_xy;  // F x 3
    long long num_triangles;
    const float4* rast;     // H x W
    const float* rgb;       // H x W x C
    const float* grad;      // H x W x C
    int C, H, W;
    float2* out;            // H x W
};

// Triangle index the reference forms with rast.w.int() - 1 (background -> the
// last triangle, as negative indexing does; its result is masked out).
__device__ __forceinline__ long long eg_tri(float w, long long F) {
    const long long id = (long long)(int)w;
    long long t = id - 1;
    if (t < 0) t += F;
    return (t >= 0 && t < F) ? t : -1;
}

__device__ __forceinline__ bool eg_inside(const EdgeGradArgs& a, int frag_pix, long long tri) {
    if (tri < 0) return false;
    const float2 p = a.frag_xy[frag_pix];
    return point_in_tri2d(p, a.tris_xy[3 * tri], a.tris_xy[3 * tri + 1], a.tris_xy[3 * tri + 2]);
}

__device__ __forceinline__ float eg_dot(const EdgeGradArgs& a, int pa, int pb) {
    float s = 0.0f;
    for (int c = 0; c < a.C; ++c) {
        const float gs = a.grad[(long long)pa * a.C + c] + a.grad[(long long)pb * a.C + c];
        const float dr = a.rgb[(long long)pa * a.C + c] - a.rgb[(long long)pb * a.C + c];
        s = fmaf(gs, dr, s);
    }
    return s;
}

// Contribution of the boundary (A, B), A the left / lower pixel, to pixel
// `self` (A or B); sign +1 horizontal, -1 vertical.
__device__ __forceinline__ float eg_pair(const EdgeGradArgs& a, int A, int B, int self, float sign) {
    const float4 rA = a.rast[A], rB = a.rast[B];
    const int idA = (int)rA.w, idB = (int)rB.w;
    if (idA == idB) return 0.0f;
    bool take;
    if (self == A) take = (idB == 0) || eg_inside(a, A, eg_tri(rB.w, a.num_triangles));
    else take = (idA == 0) || eg_inside(a, B, eg_tri(rA.w, a.num_triangles));
    if (!take) return 0.0f;
    return sign * 0.5f * eg_dot(a, A, B);
}

__global__ void __launch_bounds__(256) edge_grad_bwd_kernel(EdgeGradArgs a) {
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= a.H * a.W) return;
    const int py = pix / a.W, px = pix - py * a.W;
    float gx = 0.0f, gy = 0.0f;
    if (px > 0) gx += eg_pair(a, pix - 1, pix, pix, 1.0f);
    if (px < a.W - 1) gx += eg_pair(a, pix, pix + 1, pix, 1.0f);
    if (py > 0) gy += eg_pair(a, pix - a.W, pix, pix, -1.0f);
    if (py < a.H - 1) gy += eg_pair(a, pix, pix + a.W, pix, -1.0f);
    a.out[pix] = make_float2(gx * ((float)a.W / 2.0f), gy * ((float)a.H / 2.0f));
}

}  // namespace drp

extern "C" __attribute__((visibility("default"))) int drp_edge_gradient_bwd(
    const float* frag_xy, const float* tris_xy, long long num_triangles, const float* rast, const float* rgb,
    int channels, const float* grad_out, int height, int width, float* grad_frag_xy, void* stream) {
    if (height <= 0 || width <= 0 || height > DRP_MAX_RES || width > DRP_MAX_RES || channels <= 0 ||
        num_triangles < 0) {
        drp_set_last_error("drp_edge_gradient_bwd: bad sizes");
        return 1;
    }
    if (!frag_xy || !rast || !rgb || !grad_out || !grad_frag_xy || (num_triangles > 0 && !tris_xy) ||
        (reinterpret_cast<uintptr_t>(rast) & 15) || (reinterpret_cast<uintptr_t>(frag_xy) & 7) ||
        (reinterpret_cast<uintptr_t>(tris_xy) & 7) || (reinterpret_cast<uintptr_t>(grad_frag_xy) & 7)) {
        drp_set_last_error("drp_edge_gradient_bwd: null or misaligned pointer");
        return 1;
    }
    drp::EdgeGradArgs a;
    a.frag_xy = reinterpret_cast<const float2*>(frag_xy);
    a.tris_xy = reinterpret_cast<const float2*>(tris_xy);
    a.num_triangles = num_triangles;
    a.rast = reinterpret_cast<const float4*>(rast);
    a.rgb = rgb;
    a.grad = grad_out;
    a.C = channels;
    a.H = height;
    a.W = width;
    a.out = reinterpret_cast<float2*>(grad_frag_xy);
    const int n = height * width;
    drp::edge_grad_bwd_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(a);
    drp_note_launch();
    return drp_check_launch("drp_edge_gradient_bwd");
}
