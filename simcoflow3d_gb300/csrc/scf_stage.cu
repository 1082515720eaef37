// scf_stage.cu -- host<->device staging by SM loads and stores through the
// device-mapped address of page-locked host buffers (the reasons are in
// scf_stage.h).
#include "scf_stage.h"

#include <stdint.h>

namespace {

constexpr int kThreads = 512;
constexpr int kFullGrid = 152 * 8;   // four resident blocks per SM, the rest queued

// 16-byte words while both sides allow them, then 4-byte words for the tail.
__global__ void __launch_bounds__(kThreads) k_stage16(const uint4 *__restrict__ src, uint4 *__restrict__ dst,
                                                      size_t n16, const unsigned *__restrict__ src_tail,
                                                      unsigned *__restrict__ dst_tail, int n4_tail)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n16; t += stride) dst[t] = src[t];
    if (blockIdx.x == 0 && (int)threadIdx.x < n4_tail) dst_tail[threadIdx.x] = src_tail[threadIdx.x];
}

__global__ void __launch_bounds__(kThreads) k_stage4(const unsigned *__restrict__ src, unsigned *__restrict__ dst,
                                                     size_t n4)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n4; t += stride) dst[t] = src[t];
}

// The device-mapped address of a page-locked host pointer, or null.
void *mapped_host(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();   // not a pointer the runtime knows: the copy engine path
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// `bytes` (a multiple of 4) from `src` to `dst`, both device-addressable.
cudaError_t copy_kernel(void *dst, const void *src, size_t bytes, cudaStream_t st, int max_blocks, int *launches)
{
    const int grid_cap = max_blocks > 0 && max_blocks < kFullGrid ? max_blocks : kFullGrid;
    const uintptr_t s = (uintptr_t)src, d = (uintptr_t)dst;
    if (((s | d) & 15u) == 0) {
        const size_t n16 = bytes / 16;
        const int n4_tail = (int)((bytes % 16) / 4);
        const size_t want = (n16 + kThreads - 1) / kThreads;
        const int grid = (int)(want < 1 ? 1 : want < (size_t)grid_cap ? want : (size_t)grid_cap);
        k_stage16<<<grid, kThreads, 0, st>>>((const uint4 *)src, (uint4 *)dst, n16,
                                            (const unsigned *)(s + n16 * 16), (unsigned *)(d + n16 * 16), n4_tail);
    } else {
        const size_t n4 = bytes / 4;
        const size_t want = (n4 + kThreads - 1) / kThreads;
        const int grid = (int)(want < 1 ? 1 : want < (size_t)grid_cap ? want : (size_t)grid_cap);
        k_stage4<<<grid, kThreads, 0, st>>>((const unsigned *)src, (unsigned *)dst, n4);
    }
    if (launches) *launches += 1;
    return cudaGetLastError();
}

}  // namespace

cudaError_t stage_h2d(void *dst, const void *src, size_t bytes, cudaStream_t st, int max_blocks, int *launches,
                      StageHow *how)
{
    if (how) *how = STAGE_COPY_ENGINE;
    if (bytes == 0) return cudaSuccess;
    const void *dsrc = bytes % 4 == 0 ? mapped_host(src) : nullptr;
    if (!dsrc) return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    if (how) *how = STAGE_KERNEL;
    return copy_kernel(dst, dsrc, bytes, st, max_blocks, launches);
}

cudaError_t stage_d2h(void *dst, const void *src, size_t bytes, cudaStream_t st, int max_blocks, int *launches,
                      StageHow *how)
{
    if (how) *how = STAGE_COPY_ENGINE;
    if (bytes == 0) return cudaSuccess;
    void *ddst = bytes % 4 == 0 ? mapped_host(dst) : nullptr;
    if (!ddst) return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st);
    if (how) *how = STAGE_KERNEL;
    return copy_kernel(ddst, src, bytes, st, max_blocks, launches);
}
