// scf_tma.cuh -- Tensor Memory Accelerator staging shared by the stencil
// kernels: mbarrier waits with a bound, 3-D tiled TMA loads, and the host
// side that encodes tensor maps of the padded level layout.
//
// Row pairs.  TMA wants every global stride to be a multiple of 16 bytes.
// A row of an FP32 array in the padded layout (sy = n0 + 2 floats) is one
// only when sy is a multiple of 4, but with n0 even two consecutive rows
// are: an FP32 array is viewed as (2 sy, (n1 + 2) / 2, n2 + 2) floats --
// row pair, row pairs, planes -- and a tile arrives as two boxes, one over
// the even rows of its row pairs (x = i) and one over the odd rows
// (x = sy + i), each box's first x rounded down to a multiple of 4 floats.
// Conditions: n0 even and sy (n1 + 2) a multiple of 4 (the plane stride in
// 16-byte units); a last unpaired row (n1 odd) reads as 0.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include "scf_common.cuh"

// polls of an mbarrier before a wait gives up (each poll may suspend the
// thread for a while; together well over a second, far beyond any copy)
constexpr unsigned TMA_WAIT_POLLS = 1u << 22;

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}

// make the initialised barriers visible to the copy engine and the block
__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase of the given parity; false if it gave up.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity)
{
    for (unsigned it = 0; it < TMA_WAIT_POLLS; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 3-D tiled TMA load of one box into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load3(unsigned dst, const CUtensorMap *map, int x, int y, int z, unsigned bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

// Host side (defined in k_solver.cu).
// cuTensorMapEncodeTiled from the driver, found through the runtime (no
// link-time dependence on the driver library); nullptr if unavailable.
PFN_cuTensorMapEncodeTiled_v12000 tma_encode_fn();
// The level's shape allows the row-pair view of its FP32 arrays.
bool tma_pair_shape_ok(int n0, int n1, int sy);
// Tensor map of one FP32 array of a level (n0 x n1 x n2, row length sy,
// plane size sz) in the row-pair view, box w floats x h row pairs x 1 plane.
bool tma_encode_f32_pairs(CUtensorMap *m, const float *base, int n0, int n1, int n2, int sy, int sz, int w, int h);
