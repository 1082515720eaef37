// k_cg_df.cu -- the CG of the mixed solver in double-float arithmetic.
//
// This GPU executes FP64 at 1/64 of its FP32 rate, and the FP64 CG kernels
// (operator apply, vector updates, dot products) were bound by that rate, not
// by memory.  In the mixed solver the CG vectors x, r, p, q therefore hold
// unevaluated sums hi + lo of two FP32 numbers (a "double-float", about 48
// significand bits), and the fine operator is split the same way (its FP32
// copy is the hi part; the assembly also writes the lo parts).  The
// arithmetic is the error-free transformations of Dekker and Knuth -- the
// two-sum and the FMA-based two-product -- with every FP32 operation an
// explicitly rounded intrinsic, so that no contraction changes them.  Each
// vector occupies the 8 bytes per cell of its FP64 counterpart (the FP64
// buffers are reused), so memory traffic is unchanged.  The dot products of
// the iteration -- (p, Ap), (r, z) and (r, r) -- are FP64: each cell's
// double-float values are widened to FP64 (the FP32 -> FP64 widening is done
// with integer operations, which are exact), multiplied with an FP64 FMA and
// accumulated in FP64 per thread, per block and across blocks.  That is two
// to four FP64 operations per cell and dot, which the memory-bound kernels
// hide.  The solution is converted back to FP64 at the end of a CG round and
// its residual is recomputed in FP64, so the stopping test on the true
// residual is unchanged.
#include "scf_kernels.h"

namespace {

__device__ __forceinline__ float2 two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return make_float2(s, e);
}
// |a| >= |b|
__device__ __forceinline__ float2 quick_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ float2 dadd(float2 x, float2 y)
{
    const float2 s = two_sum(x.x, y.x);
    return quick_two_sum(s.x, __fadd_rn(s.y, __fadd_rn(x.y, y.y)));
}
__device__ __forceinline__ float2 dneg(float2 x) { return make_float2(-x.x, -x.y); }
__device__ __forceinline__ float2 dmul(float2 x, float2 y)
{
    const float p = __fmul_rn(x.x, y.x);
    float e = __fmaf_rn(x.x, y.x, -p);
    e = __fmaf_rn(x.x, y.y, e);
    e = __fmaf_rn(x.y, y.x, e);
    return quick_two_sum(p, e);
}
// the double-float form of d: hi = d rounded to FP32, lo = d - hi rounded
// to FP32, both on the integer pipe (scf_common.cuh)
__device__ __forceinline__ float2 dfrom(double d)
{
    const float hi = scf_to_f32(d);
    return make_float2(hi, scf_lo_part(d, hi));
}
__device__ __forceinline__ double dto(float2 x) { return (double)x.x + (double)x.y; }

// FP32 -> FP64 widening on the integer pipe (exact: the exponent is rebiased
// and the significand shifted into place).  Zeros keep their sign; the rare
// subnormal inputs, Inf and NaN take the hardware conversion.
__device__ __forceinline__ double widen(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    if (e - 1u < 254u) {   // normal numbers
        const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3);
        return __hiloint2double((int)hi, (int)(u << 29));
    }
    if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
    return (double)f;
}
// the FP64 value of a double-float: one FP64 addition
__device__ __forceinline__ double dwide(float2 x) { return widen(x.x) + widen(x.y); }
__device__ __forceinline__ float2 ld(const float2 *__restrict__ v, int c) { return v[c]; }

#define DF_ZCHUNK(A)                                                   \
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;          \
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;          \
    const int k0 = blockIdx.z * DF_KZ + 1;                            \
    const int k1 = min(k0 + DF_KZ - 1, (A).hi.n2);                    \
    const bool in = i <= (A).hi.n0 && j <= (A).hi.n1;

constexpr int DF_KZ = 32;

// operator coefficient of cell c from its hi (FP32 copy) and lo parts
__device__ __forceinline__ float2 cf(const float *hi, const float *lo, int c) { return make_float2(hi[c], lo[c]); }

}  // namespace

Launch3 df_launch(const DfOp &A)
{
    Launch3 l;
    l.block = dim3(32, 4, 1);
    l.grid = dim3((A.hi.n0 + 31) / 32, (A.hi.n1 + 3) / 4, (A.hi.n2 + DF_KZ - 1) / DF_KZ);
    return l;
}

// q = A p, and the block partials of (p, q) (FP64 products and sums) and of
// the sum of q (for the mean of A p in all-Neumann systems, which is zero in
// exact arithmetic: double-float per thread, FP64 across threads)
__global__ void __launch_bounds__(128, 8) k_spmv_df(DfOp A, const float2 *__restrict__ p, float2 *__restrict__ q,
                                                 double *__restrict__ part, int n0)
{
    DF_ZCHUNK(A);
    double v = 0.0;
    float2 sq = make_float2(0.f, 0.f);
    if (in) {
        const int sy = A.hi.sy, sz = A.hi.sz;
        int c = i + sy * j + sz * k0;
        float2 xm = ld(p, c - sz), x0 = ld(p, c), tb = cf(A.hi.cT, A.tlo, c - sz);
        // the six neighbour products are summed as a tree (short dependency
        // chains: the kernel is latency-bound, not memory-bound, otherwise);
        // one accumulator each keeps the kernel within 64 registers, eight
        // blocks per SM
        for (int k = k0; k <= k1; ++k, c += sz) {
            const float2 xp = ld(p, c + sz), tt = cf(A.hi.cT, A.tlo, c);
            const float2 sx = dadd(dmul(cf(A.hi.cE, A.elo, c), ld(p, c + 1)),
                                   dmul(cf(A.hi.cE, A.elo, c - 1), ld(p, c - 1)));
            const float2 syy = dadd(dmul(cf(A.hi.cN, A.nlo, c), ld(p, c + sy)),
                                    dmul(cf(A.hi.cN, A.nlo, c - sy), ld(p, c - sy)));
            const float2 sz2 = dadd(dmul(tt, xp), dmul(tb, xm));
            const float2 s = dadd(dadd(sx, syy), sz2);
            const float2 y = dadd(dmul(cf(A.hi.diag, A.dlo, c), x0), dneg(s));
            q[c] = y;
            v = fma(dwide(x0), dwide(y), v);
            sq = dadd(sq, y);
            xm = x0; x0 = xp; tb = tt;
        }
    }
    double dv = block_sum(v);
    __syncthreads();
    double ds = block_sum(dto(sq));
    if (thread_linear() == 0) {
        part[block_linear()] = dv;
        part[n0 + block_linear()] = ds;
    }
}

// (r, z) for beta: r double-float, z the FP32 preconditioned residual; FP64
// products and sums
__global__ void __launch_bounds__(128) k_dot_rz_df(DfOp A, const float2 *__restrict__ r, const float *__restrict__ z,
                                                   double *__restrict__ part)
{
    DF_ZCHUNK(A);
    double v = 0.0;
    if (in) {
        const int sy = A.hi.sy, sz = A.hi.sz;
        int c = i + sy * j + sz * k0;
        for (int k = k0; k <= k1; ++k, c += sz) v = fma(dwide(ld(r, c)), widen(z[c]), v);
    }
    v = block_sum(v);
    if (thread_linear() == 0) part[block_linear()] = v;
}

// x += alpha p, r -= alpha (q - mean q), (r, r) in FP64; also the FP32 copy
// of r (its hi part) for the V-cycle and, when x0 is given, the first
// point-Jacobi smoothing step from a zero guess, x0 = first D^-1 r.
__global__ void __launch_bounds__(128) k_cg_update_df(DfOp A, float2 *__restrict__ x, float2 *__restrict__ r,
                                                      const float2 *__restrict__ p, const float2 *__restrict__ q,
                                                      float *__restrict__ rlow, float *__restrict__ x0, float first,
                                                      const double *__restrict__ scal, double *__restrict__ part)
{
    DF_ZCHUNK(A);
    double v = 0.0;
    if (in) {
        const float2 al = dfrom(scal[S_ALPHA]), mal = dneg(al), qm = dfrom(scal[S_QMEAN]);
        const int sy = A.hi.sy, sz = A.hi.sz;
        int c = i + sy * j + sz * k0;
        for (int k = k0; k <= k1; ++k, c += sz) {
            x[c] = dadd(ld(x, c), dmul(al, ld(p, c)));
            const float dg = A.hi.diag[c];
            float2 qq = ld(q, c);
            if (dg > 0.f) qq = dadd(qq, dneg(qm));
            const float2 rn = dadd(ld(r, c), dmul(mal, qq));
            r[c] = rn;
            rlow[c] = rn.x;
            if (x0) x0[c] = first * jacobi_inv(dg) * rn.x;
            const double rd = dwide(rn);
            v = fma(rd, rd, v);
        }
    }
    v = block_sum(v);
    if (thread_linear() == 0) part[block_linear()] = v;
}

// p = z + beta p (p = z on the first call)
__global__ void __launch_bounds__(128) k_pupdate_df(DfOp A, const float *__restrict__ z, float2 *__restrict__ p,
                                                    const double *__restrict__ scal, int first)
{
    DF_ZCHUNK(A);
    if (!in) return;
    const float2 be = dfrom(first ? 0.0 : scal[S_BETA]);
    const int sy = A.hi.sy, sz = A.hi.sz;
    int c = i + sy * j + sz * k0;
    for (int k = k0; k <= k1; ++k, c += sz) {
        const float2 zz = make_float2(z[c], 0.f);
        p[c] = first ? zz : dadd(zz, dmul(be, ld(p, c)));
    }
}

// element-wise conversions over the whole padded array (in place allowed)
__global__ void k_df_from_double(const double *src, float2 *dst, int n)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const double d = src[e];
        dst[e] = dfrom(d);
    }
}
// the residual at the start of a CG round: its double-float form in place
// and its FP32 copy (the hi part) for the V-cycle, in one pass
__global__ void k_df_round_start(double *r, float *rlow, int n)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const float2 v = dfrom(r[e]);
        ((float2 *)r)[e] = v;
        rlow[e] = v.x;
    }
}
__global__ void k_df_to_double(const float2 *src, double *dst, int n)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const float2 v = src[e];
        dst[e] = dwide(v);
    }
}

void df_spmv_dot(const DfOp &A, const float2 *p, float2 *q, Reducer &R, bool singular, cudaStream_t st,
                 int *launches, KTimer *kt)
{
    Launch3 l = df_launch(A);
    const int id = kt_begin(kt, KC_SPMV, st);
    k_spmv_df<<<l.grid, l.block, 0, st>>>(A, p, q, R.partials, R.max_blocks);
    kt_end(kt, id, st);
    *launches += 1;
    reduce_alpha(R, (int)nblocks(l), singular, st, launches);
}

void df_dot_rz(const DfOp &A, const float2 *r, const float *z, Reducer &R, cudaStream_t st, int *launches)
{
    Launch3 l = df_launch(A);
    k_dot_rz_df<<<l.grid, l.block, 0, st>>>(A, r, z, R.partials);
    *launches += 1;
    reduce_beta(R, (int)nblocks(l), st, launches);
}

void df_cg_update(const DfOp &A, float2 *x, float2 *r, const float2 *p, const float2 *q, float *rlow, float *x0,
                  double first, Reducer &R, cudaStream_t st, int *launches, KTimer *kt)
{
    Launch3 l = df_launch(A);
    const int id = kt_begin(kt, KC_CGUPDATE, st);
    k_cg_update_df<<<l.grid, l.block, 0, st>>>(A, x, r, p, q, rlow, x0, (float)first, R.scal, R.partials);
    kt_end(kt, id, st);
    *launches += 1;
    reduce_to(R, (int)nblocks(l), S_RR, st, launches);
}

void df_pupdate(const DfOp &A, const float *z, float2 *p, const double *scal, bool first, cudaStream_t st,
                int *launches)
{
    Launch3 l = df_launch(A);
    k_pupdate_df<<<l.grid, l.block, 0, st>>>(A, z, p, scal, first ? 1 : 0);
    *launches += 1;
}

void df_from_double(const double *src, float2 *dst, int n, cudaStream_t st, int *launches)
{
    k_df_from_double<<<152 * 8, 256, 0, st>>>(src, dst, n);
    *launches += 1;
}

void df_round_start(double *r, float *rlow, int n, cudaStream_t st, int *launches)
{
    k_df_round_start<<<152 * 8, 256, 0, st>>>(r, rlow, n);
    *launches += 1;
}

void df_to_double(const float2 *src, double *dst, int n, cudaStream_t st, int *launches)
{
    k_df_to_double<<<152 * 8, 256, 0, st>>>(src, dst, n);
    *launches += 1;
}
