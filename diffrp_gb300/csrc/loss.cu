// loss.cu -- fused mean-absolute-error loss for image fitting: one pass reads
// prediction and target, writes the per-element gradient sign(p - t) * scale
// and per-block partial sums; a second single-block pass adds the partials in
// a fixed order (deterministic loss).
#include "drp_common.cuh"
#include "drp_internal.h"

namespace drp {

constexpr int kLossThreads = 256;
constexpr int kLossItems = 8;  // elements per thread per block pass

__global__ void __launch_bounds__(kLossThreads) l1_partial_kernel(const float* p, const float* t, long long n,
                                                                  float scale, float* grad, float* partial) {
    __shared__ float warp_sum[kLossThreads / 32];
    const long long base = (long long)blockIdx.x * kLossThreads * kLossItems;
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < kLossItems; ++k) {
        const long long i = base + (long long)k * kLossThreads + threadIdx.x;
        if (i < n) {
            const float d = p[i] - t[i];
            s += fabsf(d);
            grad[i] = d > 0.0f ? scale : (d < 0.0f ? -scale : 0.0f);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = threadIdx.x < kLossThreads / 32 ? warp_sum[threadIdx.x] : 0.0f;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}

__global__ void __launch_bounds__(1024) l1_final_kernel(const float* partial, long long nblocks, float scale,
                                                        float* loss) {
    __shared__ double warp_sum[32];
    double s = 0.0;
    for (long long i = threadIdx.x; i < nblocks; i += blockDim.x) s += (double)partial[i];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (int)(blockDim.x >> 5) ? warp_sum[threadIdx.x] : 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (threadIdx.x == 0) *loss = (float)(v * (double)scale);
    }
}

}  // namespace drp

extern "C" __attribute__((visibility("default"))) int drp_l1_loss_workspace_size(long long n, size_t* bytes) {
    if (!bytes || n < 0) {
        drp_set_last_error("drp_l1_loss_workspace_size: bad arguments");
        return 1;
    }
    const long long per = (long long)drp::kLossThreads * drp::kLossItems;
    *bytes = (size_t)((n + per - 1) / per) * sizeof(float) + 256;
    return 0;
}

extern "C" __attribute__((visibility("default"))) int drp_l1_loss_fwd(void* workspace, size_t workspace_bytes,
                                                                      const float* pred, const float* target,
                                                                      long long n, float scale, float* loss,
                                                                      float* grad, void* stream) {
    const long long per = (long long)drp::kLossThreads * drp::kLossItems;
    const long long nblocks = (n + per - 1) / per;
    if (n <= 0 || !pred || !target || !loss || !grad || !workspace ||
        workspace_bytes < (size_t)nblocks * sizeof(float) || nblocks > 0x7fffffffll) {
        drp_set_last_error("drp_l1_loss_fwd: bad arguments or workspace too small");
        return 1;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    float* partial = static_cast<float*>(workspace);
    drp::l1_partial_kernel<<<(unsigned)nblocks, drp::kLossThreads, 0, s>>>(pred, target, n, scale, grad, partial);
    drp::l1_final_kernel<<<1, 1024, 0, s>>>(partial, nblocks, scale, loss);
    return drp_check_launch("drp_l1_loss_fwd");
}
