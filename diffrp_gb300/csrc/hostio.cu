// hostio.cu -- moving a step's inputs and results between pinned host memory
// and the device with the SMs instead of a copy engine.  On a coherent
// host link (NVLink-C2C) a kernel can load and store mapped pinned host
// memory directly; for the few hundred kilobytes of a fitting step's
// parameters and gradients that beats a DMA transfer, whose set-up latency
// dominates at this size.  No counterpart in the reference, which leaves
// transfers to torch.
#include "../../include/diffrp_gb300.h"
#include "drp_common.cuh"
#include "drp_internal.h"

namespace drp {

constexpr int kCopyThreads = 256;

// 16-byte vectors when both ends are 16-byte aligned, then the tail bytes.
__global__ void __launch_bounds__(kCopyThreads) copy_kernel(unsigned char* __restrict__ dst,
                                                            const unsigned char* __restrict__ src, size_t bytes,
                                                            bool vec) {
    const size_t stride = (size_t)gridDim.x * kCopyThreads;
    const size_t tid = (size_t)blockIdx.x * kCopyThreads + threadIdx.x;
    size_t done = 0;
    if (vec) {
        const size_t n16 = bytes >> 4;
        const uint4* s = reinterpret_cast<const uint4*>(src);
        uint4* d = reinterpret_cast<uint4*>(dst);
        for (size_t i = tid; i < n16; i += stride) d[i] = s[i];
        done = n16 << 4;
    }
    for (size_t i = done + tid; i < bytes; i += stride) dst[i] = src[i];
}

}  // namespace drp

#define DRP_API extern "C" __attribute__((visibility("default")))

DRP_API int drp_host_device_pointer(const void* host, void** device) {
    if (!host || !device) {
        drp_set_last_error("drp_host_device_pointer: null argument");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    *device = nullptr;
    void* p = nullptr;
    const cudaError_t e = cudaHostGetDevicePointer(&p, const_cast<void*>(host), 0);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();  // not sticky: clear it
        drp_set_last_error("drp_host_device_pointer: memory is not mapped pinned host memory");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    *device = p;
    return DRP_STATUS_OK;
}

DRP_API int drp_copy_async(void* dst, const void* src, size_t bytes, void* stream) {
    if (bytes == 0) return DRP_STATUS_OK;
    if (!dst || !src) {
        drp_set_last_error("drp_copy_async: null pointer");
        return DRP_STATUS_INVALID_ARGUMENT;
    }
    const bool vec = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0;
    // one 16-byte unit per thread up to eight blocks per SM (grid-stride
    // beyond): as many loads in flight across the link as the size allows
    const size_t units = vec ? (bytes + 15) >> 4 : bytes;
    const int sms = drp_current_sm_count();
    const size_t most = (size_t)(sms > 0 ? sms : 1) * 8;
    size_t blocks = (units + drp::kCopyThreads - 1) / drp::kCopyThreads;
    blocks = blocks < 1 ? 1 : (blocks > most ? most : blocks);
    drp::copy_kernel<<<(unsigned)blocks, drp::kCopyThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<unsigned char*>(dst), static_cast<const unsigned char*>(src), bytes, vec);
    drp_note_launch();
    return drp_check_launch("drp_copy_async");
}
