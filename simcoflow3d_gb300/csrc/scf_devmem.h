// scf_devmem.h -- every device buffer of the library is allocated and freed
// through these two functions.  They count the buffers held, and a test can
// make the n-th allocation from now fail as cudaMalloc would on a full GPU:
// the failure is injected on the host, no cudaMalloc is called for it, so
// the test exercises each context's clean-up path without touching the
// device's memory.  (scf_debug_fail_device_alloc / scf_debug_device_buffers
// in scf_projection.h.)
#pragma once

#include <cuda_runtime.h>

#include <atomic>

namespace scf_mem {

extern std::atomic<long long> fail_countdown;   // > 0: allocations left until the injected failure
extern std::atomic<long long> live;             // device buffers currently held

inline cudaError_t dev_malloc(void **p, size_t bytes)
{
    long long c = fail_countdown.load();
    while (c > 0) {
        if (fail_countdown.compare_exchange_weak(c, c - 1)) {
            if (c == 1) {
                *p = nullptr;
                return cudaErrorMemoryAllocation;
            }
            break;
        }
    }
    const cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) live.fetch_add(1);
    return e;
}

inline cudaError_t dev_free(void *p)
{
    if (!p) return cudaSuccess;
    live.fetch_sub(1);
    return cudaFree(p);
}

}  // namespace scf_mem
