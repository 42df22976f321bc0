// transform.cu -- clip-space transform of shared vertices by per-view
// matrices: out[b, i] = M_b [v_i, 1] (SurfaceDeferredRenderSession.clip_space,
// diffrp/rendering/surface_deferred.py:229-238, through transform_point,
// diffrp/utils/shader_ops.py:123-136: one small GEMM per view there).  The
// backward sums the views' contributions per vertex in view order, so it
// needs no atomics and is reproducible.
#include "../../include/diffrp_gb300.h"
#include "drp_common.cuh"
#include "drp_internal.h"

namespace drp {

// M: B row-major 4x4 matrices (16 floats each).
__global__ void __launch_bounds__(256) transform_fwd_kernel(const float* __restrict__ verts, long long V,
                                                            const float* __restrict__ M, int B,
                                                            float4* __restrict__ out) {
    __shared__ float m[16];
    pdl_wait();
    pdl_launch_dependents();
    const int b = blockIdx.y;
    if (threadIdx.x < 16) m[threadIdx.x] = M[16 * b + threadIdx.x];
    __syncthreads();
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    const float x = verts[3 * i], y = verts[3 * i + 1], z = verts[3 * i + 2];
    float r[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) r[k] = fmaf(m[4 * k + 2], z, fmaf(m[4 * k + 1], y, fmaf(m[4 * k], x, m[4 * k + 3])));
    out[(long long)b * V + i] = make_float4(r[0], r[1], r[2], r[3]);
}

// grad_verts[i] = sum over b (view order) of M_b[:, :3]^T grad_out[b, i].
__global__ void __launch_bounds__(256) transform_bwd_kernel(const float4* __restrict__ grad_out, long long V,
                                                            const float* __restrict__ M, int B,
                                                            float* __restrict__ grad_verts) {
    pdl_wait();
    pdl_launch_dependents();
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    float gx = 0.f, gy = 0.f, gz = 0.f;
    for (int b = 0; b < B; ++b) {
        const float4 g = grad_out[(long long)b * V + i];
        const float* m = M + 16 * b;
        gx = fmaf(g.w, m[12], fmaf(g.z, m[8], fmaf(g.y, m[4], fmaf(g.x, m[0], gx))));
        gy = fmaf(g.w, m[13], fmaf(g.z, m[9], fmaf(g.y, m[5], fmaf(g.x, m[1], gy))));
        gz = fmaf(g.w, m[14], fmaf(g.z, m[10], fmaf(g.y, m[6], fmaf(g.x, m[2], gz))));
    }
    grad_verts[3 * i] = gx;
    grad_verts[3 * i + 1] = gy;
    grad_verts[3 * i + 2] = gz;
}

}  // namespace drp

#define DRP_API extern "C" __attribute__((visibility("default")))

DRP_API int drp_transform_points_fwd(const float* verts, long long num_vertices, const float* mats, int num_views,
                                     float* out, void* stream) {
    if (num_vertices < 0 || num_views <= 0 || num_views > 65535 || (num_vertices > 0 && (!verts || !out)) || !mats ||
        (reinterpret_cast<uintptr_t>(out) & 15)) {
        drp_set_last_error("drp_transform_points_fwd: bad arguments (out must be 16-byte aligned float4 rows)");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    if (num_vertices == 0) return DRP_STATUS_OK;
    const dim3 grid((unsigned)((num_vertices + 255) / 256), (unsigned)num_views);
    drp::launch_pdl(drp::transform_fwd_kernel, grid, dim3(256), static_cast<cudaStream_t>(stream), verts,
                    num_vertices, mats, num_views, reinterpret_cast<float4*>(out));
    drp_note_launch();
    return drp_check_launch("drp_transform_points_fwd");
}

DRP_API int drp_transform_points_bwd(const float* grad_out, long long num_vertices, const float* mats, int num_views,
                                     float* grad_verts, void* stream) {
    if (num_vertices < 0 || num_views <= 0 || num_views > 65535 || (num_vertices > 0 && (!grad_out || !grad_verts)) || !mats ||
        (reinterpret_cast<uintptr_t>(grad_out) & 15)) {
        drp_set_last_error("drp_transform_points_bwd: bad arguments (grad_out must be 16-byte aligned float4 rows)");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    if (num_vertices == 0) return DRP_STATUS_OK;
    drp::launch_pdl(drp::transform_bwd_kernel, dim3((unsigned)((num_vertices + 255) / 256)), dim3(256),
                    static_cast<cudaStream_t>(stream), reinterpret_cast<const float4*>(grad_out), num_vertices, mats,
                    num_views, grad_verts);
    drp_note_launch();
    return drp_check_launch("drp_transform_points_bwd");
}
