// loss.cu -- fused mean-absolute-error loss for image fitting: one pass reads
// prediction and target, writes the per-element gradient sign(p - t) * scale
// and per-block partial sums (compensated float sums over a grid of a few
// blocks per SM); a second single-block pass adds the partials in a fixed
// order with compensated float-pair sums (reproducible loss).
#include "drp_common.cuh"
#include "drp_internal.h"

namespace drp {

constexpr int kLossThreads = 256;
constexpr int kLossBlocksPerSM = 8;

// Kahan step: s + x with the lost low part carried in c.
__device__ inline void kahan_add(float& s, float& c, float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

__device__ inline float l1_grad(float d, float scale) { return d > 0.0f ? scale : (d < 0.0f ? -scale : 0.0f); }

// Grid-stride pass over float4 groups (scalar head/tail when the three
// pointers are not 16-byte aligned alike); one partial per block.  The grid is
// fixed per device, so the summation order -- and the loss -- is reproducible.
__global__ void __launch_bounds__(kLossThreads) l1_partial_kernel(const float* p, const float* t, long long n,
                                                                  float scale, float* grad, float* partial) {
    __shared__ float warp_sum[kLossThreads / 32];
    const long long stride = (long long)gridDim.x * kLossThreads;
    const long long tid = (long long)blockIdx.x * kLossThreads + threadIdx.x;
    float s = 0.0f, c = 0.0f;
    const bool vec = ((reinterpret_cast<uintptr_t>(p) | reinterpret_cast<uintptr_t>(t) |
                       reinterpret_cast<uintptr_t>(grad)) & 15) == 0;
    long long done = 0;
    if (vec) {
        const long long n4 = n >> 2;
        const float4* p4 = reinterpret_cast<const float4*>(p);
        const float4* t4 = reinterpret_cast<const float4*>(t);
        float4* g4 = reinterpret_cast<float4*>(grad);
        for (long long i = tid; i < n4; i += stride) {
            const float4 a = p4[i], b = t4[i];
            const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z, dw = a.w - b.w;
            kahan_add(s, c, (fabsf(dx) + fabsf(dy)) + (fabsf(dz) + fabsf(dw)));
            g4[i] = make_float4(l1_grad(dx, scale), l1_grad(dy, scale), l1_grad(dz, scale), l1_grad(dw, scale));
        }
        done = n4 << 2;
    }
    for (long long i = done + tid; i < n; i += stride) {
        const float d = p[i] - t[i];
        kahan_add(s, c, fabsf(d));
        grad[i] = l1_grad(d, scale);
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

// Fixed-order compensated sum of the partials (l1_final_block,
// drp_common.cuh) in one block.
__global__ void __launch_bounds__(kFinalThreads) l1_final_kernel(const float* partial, long long nblocks, float scale,
                                                                 float* loss) {
    pdl_wait();
    pdl_launch_dependents();
    l1_final_block<kFinalThreads>(partial, nblocks, scale, loss);
}

void launch_l1_final(const float* partial, long long nblocks, float scale, float* loss, cudaStream_t s) {
    launch_pdl(l1_final_kernel, dim3(1), dim3(kFinalThreads), s, partial, nblocks, scale, loss);
    drp_note_launch();
}

// dst = src * scale[0]: 16-byte groups from the first aligned float, scalar
// head and tail (grid-stride).
__global__ void __launch_bounds__(256) scale_floats_kernel(float* dst, const float* src, long long n,
                                                           const float* scale) {
    pdl_wait();
    pdl_launch_dependents();
    const float k = *scale;
    const long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const bool same_phase = ((reinterpret_cast<uintptr_t>(dst) ^ reinterpret_cast<uintptr_t>(src)) & 15) == 0;
    long long h = same_phase ? (long long)(((16 - (reinterpret_cast<uintptr_t>(dst) & 15)) & 15) >> 2) : n;
    if (h > n) h = n;
    for (long long i = i0; i < h; i += stride) dst[i] = src[i] * k;
    const long long n4 = (n - h) >> 2;
    float4* d4 = reinterpret_cast<float4*>(dst + h);
    const float4* s4 = reinterpret_cast<const float4*>(src + h);
    for (long long i = i0; i < n4; i += stride) {
        const float4 v = s4[i];
        d4[i] = make_float4(v.x * k, v.y * k, v.z * k, v.w * k);
    }
    const long long t0 = h + 4 * n4;
    if (i0 < n - t0) dst[t0 + i0] = src[t0 + i0] * k;
}

// Blocks for n elements: enough to fill every SM, never more than one
// float4 group per thread.
static long long l1_blocks(long long n) {
    const int sms = drp_current_sm_count();
    if (sms <= 0) return 1;  // no device: callers fail at launch
    const long long max_blocks = (long long)sms * kLossBlocksPerSM;
    const long long need = ((n + 3) / 4 + kLossThreads - 1) / kLossThreads;
    return need < max_blocks ? (need > 0 ? need : 1) : max_blocks;
}

}  // namespace drp

extern "C" __attribute__((visibility("default"))) int drp_l1_loss_workspace_size(long long n, size_t* bytes) {
    if (!bytes || n < 0) {
        drp_set_last_error("drp_l1_loss_workspace_size: bad arguments");
        return 1;
    }
    // the most blocks any device uses: one float4 group per thread (the grid
    // is capped below that by the SM count), so the size is device-independent
    const long long most = ((n + 3) / 4 + drp::kLossThreads - 1) / drp::kLossThreads;
    *bytes = (size_t)(most > 0 ? most : 1) * sizeof(float) + 256;
    return 0;
}

extern "C" __attribute__((visibility("default"))) int drp_l1_loss_fwd(void* workspace, size_t workspace_bytes,
                                                                      const float* pred, const float* target,
                                                                      long long n, float scale, float* loss,
                                                                      float* grad, void* stream) {
    const long long nblocks = drp::l1_blocks(n);
    if (n <= 0 || !pred || !target || !loss || !grad || !workspace ||
        workspace_bytes < (size_t)nblocks * sizeof(float) || nblocks > 0x7fffffffll) {
        drp_set_last_error("drp_l1_loss_fwd: bad arguments or workspace too small");
        return 1;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    float* partial = static_cast<float*>(workspace);
    drp::l1_partial_kernel<<<(unsigned)nblocks, drp::kLossThreads, 0, s>>>(pred, target, n, scale, grad, partial);
    drp_note_launch();
    drp::launch_l1_final(partial, nblocks, scale, loss, s);
    return drp_check_launch("drp_l1_loss_fwd");
}

extern "C" __attribute__((visibility("default"))) int drp_scale_floats(float* dst, const float* src, long long n,
                                                                      const float* scale, void* stream) {
    if (n < 0 || (n > 0 && (!dst || !src || !scale)) || ((reinterpret_cast<uintptr_t>(dst) |
                                                        reinterpret_cast<uintptr_t>(src)) & 3)) {
        drp_set_last_error("drp_scale_floats: bad arguments");
        return 1;
    }
    if (n == 0) return 0;
    const int sms = drp_current_sm_count();
    long long blocks = (n / 4 + 255) / 256;
    const long long cap = (long long)(sms > 0 ? sms : 1) * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    drp::launch_pdl(drp::scale_floats_kernel, dim3((unsigned)blocks), dim3(256), static_cast<cudaStream_t>(stream),
                    dst, src, n, scale);
    drp_note_launch();
    return drp_check_launch("drp_scale_floats");
}
