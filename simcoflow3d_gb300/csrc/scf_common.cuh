// scf_common.cuh -- shared definitions of the GB300 projection library.
//
// Layout conventions (the reference's, kept on the device so that every
// host array moves with one contiguous copy):
//   ghosted   (0:I+1, 0:J+1, 0:K+1), i fastest: g = i + gx*(j + gy*k)
//   interior  (1:I, 1:J, 1:K):                  n = (i-1) + I*((j-1) + J*(k-1))
//   PoCoef    (1:I, 1:J, 1:K, 1:6):             n + N*(f-1), faces W,S,B,E,N,T
// Solver arrays of the fine level use the ghosted layout with a zero ghost
// layer; coarse levels use the same padded layout for their own sizes.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define SCF_HD __host__ __device__ __forceinline__

struct Dims {
    int I, J, K;
    int gx, gy, gz;     // I+2, J+2, K+2
    int ng;             // ghosted cell count
    int n;              // interior cell count
};

SCF_HD int gidx(const Dims &d, int i, int j, int k) { return i + d.gx * (j + d.gy * k); }
SCF_HD int nidx(const Dims &d, int i, int j, int k) { return (i - 1) + d.I * ((j - 1) + d.J * (k - 1)); }

// Device error flags (bitwise OR into ctx->flags[0]).
enum ScfFlag : unsigned {
    FLAG_BAD_POSNU = 1u,          // PosNu == -1 differs from Cell_Type == 2, or out of range
    FLAG_STALE_OVERFLOW = 2u,     // stale-coefficient list full
    FLAG_STALE_LIMIT = 4u,        // stale search hit its step limit
    FLAG_NONFINITE = 8u,          // NaN/Inf in the assembled system
    FLAG_BAD_DIAG = 16u,          // active row with diagonal <= 0
    FLAG_NEITHER_ACTIVE = 32u,    // active cell that is neither wet nor dry
    FLAG_WAIT_TIMEOUT = 64u,      // a kernel's bounded wait for its own copies gave up
};

// Scalars kept on the device during CG (no host round trip for alpha/beta).
enum ScfScalar {
    S_RZ = 0,      // (r, z) of the current iteration
    S_PQ,          // (p, A p)
    S_ALPHA,
    S_BETA,
    S_RR,          // (r, r)
    S_BB,          // (b, b)
    S_SUM,         // scratch sum (mean projection)
    S_COUNT,       // active cell count
    S_MEAN,
    S_RZ_NEW,
    S_MEANX,       // mean of x over the active cells (all-Neumann systems)
    S_JP,          // loss: pressure term
    S_JD,          // loss: divergence term
    S_QMEAN,       // mean of A p over the active cells (all-Neumann systems)
    S_NUM
};

// One multigrid level as the kernels see it (padded layout).
template <typename T>
struct LevelView {
    int n0, n1, n2;       // interior sizes
    int sy, sz;           // strides (n0+2, (n0+2)*(n1+2))
    const T *diag, *dinv, *cE, *cN, *cT;
};

// Jacobi scaling of the FP32 V-cycle levels: 1/diag by the hardware
// reciprocal (rcp.approx.ftz.f32, one instruction, within one unit in the
// last place), 0 on inactive cells (diag <= 0).  Every FP32 smoothing
// kernel uses it, so they agree bit for bit; the smoother needs no
// correctly rounded reciprocal.
__device__ __forceinline__ float jacobi_inv(float d)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d));
    return d > 0.0f ? r : 0.0f;
}

template <typename T>
__device__ __forceinline__ T apply_row(const LevelView<T> &L, const T *__restrict__ x, int c)
{
    return L.diag[c] * x[c] -
           (L.cE[c] * x[c + 1] + L.cE[c - 1] * x[c - 1] + L.cN[c] * x[c + L.sy] + L.cN[c - L.sy] * x[c - L.sy] +
            L.cT[c] * x[c + L.sz] + L.cT[c - L.sz] * x[c - L.sz]);
}

// Launch helpers -----------------------------------------------------------
struct Launch3 {
    dim3 grid, block;
};

inline Launch3 launch_interior(int n0, int n1, int n2)
{
    Launch3 l;
    l.block = dim3(32, 4, 2);
    l.grid = dim3((n0 + 31) / 32, (n1 + 3) / 4, (n2 + 1) / 2);
    return l;
}

inline unsigned nblocks(const Launch3 &l) { return l.grid.x * l.grid.y * l.grid.z; }

// Block-wide FP64 sum; result valid in thread 0.  blockDim.x*y*z <= 1024.
__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double warp_part[32];
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthreads = blockDim.x * blockDim.y * blockDim.z;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = tid & 31, w = tid >> 5;
    if (lane == 0) warp_part[w] = v;
    __syncthreads();
    const int nw = (nthreads + 31) >> 5;
    v = (tid < nw) ? warp_part[tid] : 0.0;
    if (w == 0)
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ int block_linear() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }
__device__ __forceinline__ int thread_linear() { return threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z); }

#if defined(__CUDACC__)
// ---- FP64 -> FP32 on the integer pipe ---------------------------------------
// FP64 arithmetic is this GPU's scarcest resource; these two conversions
// (used by the assembly and the mixed solver's double-float vectors) run on
// the integer pipe and match the IEEE conversions bit for bit.

// d - (double)hi rounded to FP32, where hi is d rounded to FP32: the lo part
// of the double-float form of d.  Computed on the integer pipe (the
// significands of d and hi aligned to d's exponent differ by less than
// 2^29 units of d's last place).  Zeros give +0; subnormals and non-finite
// values take the FP64 route.
__device__ __forceinline__ float scf_lo_part(double d, float hi)
{
    const long long db = __double_as_longlong(d);
    if (((unsigned long long)db << 1) == 0) return 0.0f;   // d - (double)hi = +0 for d = +-0
    const int ed = (int)((db >> 52) & 0x7ff);
    const int hb = __float_as_int(hi);
    const int eh8 = (hb >> 23) & 0xff;
    if (ed != 0 && ed != 0x7ff && eh8 != 0 && eh8 != 0xff) {
        const long long md = (db & 0xfffffffffffffLL) | (1LL << 52);
        const long long mh = (long long)((hb & 0x7fffff) | 0x800000) << 29;
        const int eh = eh8 - 127 + 1023;
        long long diff;
        bool ok = true;
        if (eh == ed) diff = md - mh;
        else if (eh == ed + 1) diff = md - (mh << 1);
        else { diff = 0; ok = false; }
        if (ok && diff > -(1LL << 30) && diff < (1LL << 30)) {
            if (diff == 0) return 0.0f;
            if (db < 0) diff = -diff;
            const int fb = __float_as_int(__int2float_rn((int)diff));
            const int ef = ((fb >> 23) & 0xff) + (ed - 1075);
            if (ef >= 1 && ef <= 254) return __int_as_float((fb & ~(0xff << 23)) | (ef << 23));
        }
    }
    return (float)(d - (double)hi);
}

// d rounded to FP32 (round to nearest even) on the integer pipe, for results
// in FP32's normal range, and of zeros; the rest (subnormal or out-of-range
// results, non-finite values) take the conversion instruction, which runs on
// the FP64 pipe.
__device__ __forceinline__ float scf_to_f32(double d)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const int e = (int)((b >> 52) & 0x7ff);
    if ((b << 1) == 0) return __uint_as_float((unsigned)(b >> 32));   // +-0
    if (e >= 1023 - 126 && e <= 1023 + 127) {
        const unsigned long long m = b & 0xfffffffffffffull;
        const unsigned hi = (unsigned)(m >> 29), rem = (unsigned)(m & 0x1fffffffu);
        unsigned r = ((unsigned)(e - 1023 + 127) << 23) | hi;
        if (rem > 0x10000000u || (rem == 0x10000000u && (hi & 1u))) r += 1u;   // a carry rounds into the exponent
        r |= (unsigned)(b >> 32) & 0x80000000u;
        return __uint_as_float(r);
    }
    return (float)d;
}
#endif
