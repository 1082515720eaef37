// k_bicgstab.cu -- BiCGStab (van der Vorst, SIAM J. Sci. Stat. Comput. 13,
// 1992) on the Jacobi-scaled momentum systems of the predictor, templated on
// the vector type (FP64, or FP32 inside FP64 iterative refinement).
//
// One iteration is four passes:
//   U: p = r + beta (p - omega v) in place (the first step of a run takes
//      p = r)
//   P: v = A p; r0.v; then alpha
//   S: s = r - alpha v, formed at the 7 points; t = A s; t.s, t.t; omega
//   X: s again, x += alpha p + omega s, r = s - omega t; r0.r, r.r; beta,
//      and the stopping test
// s is never stored.  Each thread marches KZ cells of one (i, j) column and
// keeps its share of the dot products in registers, so a block writes one
// partial sum per dot for 128 x KZ cells; after each of P, S and X one
// block of 1024 threads sums the partials in a fixed order (so every run is
// bitwise reproducible) and updates the scalars, which stay in device
// memory.  (Summing them in the last block of the pass instead was slower:
// 128 threads on one SM add 8192 partials.)  The reduction after X sets
// `done` when ||r||^2 <= target or on a breakdown, and every kernel after
// that returns at once, so the host enqueues several iterations and reads
// the scalars once per batch.
#include "pred_kernels.h"

namespace pred {
namespace {

constexpr int NT = 128;
constexpr int KZ = 16;

// Sum of up to 4 values over the block; thread 0 writes them to
// partials[4 * block + q].  The products and the warp sums are formed in A
// (FP32 for the FP32 iteration: this GPU runs FP64 at 1/64 of the FP32
// rate), the sums over the block's warps and over the blocks in FP64.
template <int Q, typename A>
__device__ __forceinline__ void block_partials(A (&v)[Q], double *partials)
{
    __shared__ double sh[NT / 32][4];
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        A a = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) sh[warp][q] = (double)a;
    }
    __syncthreads();
    if (tid == 0) {
        const long long blk = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            double a = 0.0;
            for (int w = 0; w < NT / 32; ++w) a += sh[w][q];
            partials[4 * blk + q] = a;
        }
    }
}

__device__ __forceinline__ bool finite_nonzero(double a) { return a != 0.0 && isfinite(a); }

template <typename T>
struct M6 {
    const T *w, *s, *b, *e, *n, *t;
};

// The column segment of a thread: cells (i, j, k0..k1); `in` is false for
// threads outside the grid (they still join the block reduction).
#define COLUMN                                                                \
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;                  \
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;                  \
    const int k0 = blockIdx.z * KZ + 1;                                       \
    const int k1 = min(k0 + KZ - 1, d.K);                                     \
    const bool in = i <= d.I && j <= d.J;                                     \
    const long long c0 = i + d.sy * j + d.sz * k0;

template <typename T, typename F>
__device__ __forceinline__ T apply_stencil(const M6<T> &m, const Dims &d, long long c, F X)
{
    return X(c) - (m.w[c] * X(c - 1) + m.s[c] * X(c - d.sy) + m.b[c] * X(c - d.sz) + m.e[c] * X(c + 1) +
                   m.n[c] * X(c + d.sy) + m.t[c] * X(c + d.sz));
}

template <typename T>
__global__ void __launch_bounds__(NT) k_bcg_u(Dims d, const T *__restrict__ r, T *__restrict__ p,
                                              const T *__restrict__ v, const BcgScalars *sc, int first)
{
    if (sc->done) return;
    COLUMN
    if (!in) return;
    const T beta = (T)sc->beta, omega = (T)sc->omega;
    long long c = c0;
    if (first)
        for (int k = k0; k <= k1; ++k, c += d.sz) p[c] = r[c];
    else
        for (int k = k0; k <= k1; ++k, c += d.sz) p[c] = r[c] + beta * (p[c] - omega * v[c]);
}

template <typename T>
__global__ void __launch_bounds__(NT) k_bcg_p(Dims d, M6<T> m, const T *__restrict__ p, const T *__restrict__ r0,
                                              T *__restrict__ v, const BcgScalars *sc, double *partials)
{
    if (sc->done) return;
    COLUMN
    T acc[1] = {T(0)};
    if (in) {
        auto P = [&](long long q) { return p[q]; };
        long long c = c0;
        for (int k = k0; k <= k1; ++k, c += d.sz) {
            const T y = apply_stencil(m, d, c, P);
            v[c] = y;
            acc[0] += r0[c] * y;
        }
    }
    block_partials<1, T>(acc, partials);
}

template <typename T>
__global__ void __launch_bounds__(NT) k_bcg_s(Dims d, M6<T> m, const T *__restrict__ r, const T *__restrict__ v,
                                              T *__restrict__ t, const BcgScalars *sc, double *partials)
{
    if (sc->done) return;
    COLUMN
    T acc[2] = {T(0), T(0)};
    if (in) {
        const T alpha = (T)sc->alpha;
        auto S = [&](long long q) { return r[q] - alpha * v[q]; };
        long long c = c0;
        for (int k = k0; k <= k1; ++k, c += d.sz) {
            const T y = apply_stencil(m, d, c, S);
            t[c] = y;
            acc[0] += y * S(c);
            acc[1] += y * y;
        }
    }
    block_partials<2, T>(acc, partials);
}

template <typename T>
__global__ void __launch_bounds__(NT) k_bcg_x(Dims d, T *__restrict__ x, T *__restrict__ r,
                                              const T *__restrict__ r0, const T *__restrict__ p,
                                              const T *__restrict__ v, const T *__restrict__ t, const BcgScalars *sc,
                                              double *partials)
{
    if (sc->done) return;
    COLUMN
    T acc[2] = {T(0), T(0)};
    if (in) {
        const T alpha = (T)sc->alpha, omega = (T)sc->omega;
        long long c = c0;
        for (int k = k0; k <= k1; ++k, c += d.sz) {
            const T s = r[c] - alpha * v[c];
            x[c] = x[c] + (alpha * p[c] + omega * s);
            const T rn = s - omega * t[c];
            r[c] = rn;
            acc[0] += r0[c] * rn;
            acc[1] += rn * rn;
        }
    }
    block_partials<2, T>(acc, partials);
}

// x += e (the FP32 correction of a refinement round), pointwise.
__global__ void __launch_bounds__(NT) k_xadd(Dims d, double *__restrict__ x, const float *__restrict__ e)
{
    COLUMN
    if (!in) return;
    long long c = c0;
    for (int k = k0; k <= k1; ++k, c += d.sz) x[c] = x[c] + (double)e[c];
}

// r = b - A x in FP64 (x = NULL stands for x = 0: r = b without the stencil
// pass); ||r||^2, ||r_T||^2 of the stored vector (r32 when given, summed in
// FP32) and, with want_bb, ||b||^2.
__global__ void __launch_bounds__(NT) k_resid64(Dims d, M6<double> m, const double *__restrict__ b,
                                                const double *__restrict__ x, double *__restrict__ r64,
                                                float *__restrict__ r32, int want_bb, double *partials)
{
    COLUMN
    double acc[3] = {0.0, 0.0, 0.0};
    if (in) {
        auto X = [&](long long q) { return x[q]; };
        float rt2 = 0.f;
        long long c = c0;
        for (int k = k0; k <= k1; ++k, c += d.sz) {
            const double r = x ? b[c] - apply_stencil(m, d, c, X) : b[c];
            if (r64) r64[c] = r;
            if (r32) {
                const float f = (float)r;
                r32[c] = f;
                rt2 += f * f;
            }
            acc[0] += r * r;
            if (want_bb) acc[2] += b[c] * b[c];
        }
        acc[1] = r32 ? (double)rt2 : acc[0];
    }
    block_partials<3, double>(acc, partials);
}

// Sums q columns of the partials (fixed order: thread-strided, then a tree).
template <int Q>
__device__ __forceinline__ void sum_partials(const double *partials, int nb, double (&out)[Q])
{
    __shared__ double sh[1024][Q];
    double a[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) a[q] = 0.0;
    for (int blk = threadIdx.x; blk < nb; blk += blockDim.x)
#pragma unroll
        for (int q = 0; q < Q; ++q) a[q] += partials[4 * (long long)blk + q];
#pragma unroll
    for (int q = 0; q < Q; ++q) sh[threadIdx.x][q] = a[q];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
#pragma unroll
            for (int q = 0; q < Q; ++q) sh[threadIdx.x][q] += sh[threadIdx.x + s][q];
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) out[q] = sh[0][q];
}

// after P: alpha = rho / (r0.v)
__global__ void __launch_bounds__(1024) k_red_alpha(const double *partials, int nb, BcgScalars *sc)
{
    if (sc->done) return;
    double s[1];
    sum_partials<1>(partials, nb, s);
    if (threadIdx.x == 0) {
        const double a = sc->rho / s[0];
        if (finite_nonzero(s[0]) && isfinite(a)) sc->alpha = a;
        else { sc->alpha = 0.0; sc->breakdown = 1; sc->done = 1; }
    }
}

// after S: omega = (t.s) / (t.t); t.t = 0 means s = 0 (omega = 0 finishes)
__global__ void __launch_bounds__(1024) k_red_omega(const double *partials, int nb, BcgScalars *sc)
{
    if (sc->done) return;
    double s[2];
    sum_partials<2>(partials, nb, s);
    if (threadIdx.x == 0) {
        const double w = s[1] > 0.0 ? s[0] / s[1] : 0.0;
        sc->omega = isfinite(w) ? w : 0.0;
    }
}

// after X: beta = (rho_new / rho) (alpha / omega), rho = rho_new, rr, and
// the stopping test
__global__ void __launch_bounds__(1024) k_red_rho(const double *partials, int nb, BcgScalars *sc)
{
    if (sc->done) return;
    double s[2];
    sum_partials<2>(partials, nb, s);
    if (threadIdx.x == 0) {
        sc->rr = s[1];
        sc->iters += 1;
        const double b = (s[0] / sc->rho) * (sc->alpha / sc->omega);
        if (finite_nonzero(s[0]) && sc->omega != 0.0 && isfinite(b)) sc->beta = b;
        else { sc->beta = 0.0; sc->breakdown = 1; sc->done = 1; }
        sc->rho = s[0];
        if (!(s[1] > sc->target)) sc->done = 1;   // converged (or NaN: the host checks)
    }
}

// after a residual: a fresh start (p = r on the next P)
__global__ void __launch_bounds__(1024) k_red_resid(const double *partials, int nb, BcgScalars *sc, int want_bb)
{
    double s[3];
    sum_partials<3>(partials, nb, s);
    if (threadIdx.x == 0) {
        sc->rr = s[0];
        sc->rho = s[1];
        if (want_bb) sc->bb = s[2];
        sc->alpha = 1.0;
        sc->omega = 1.0;
        sc->beta = 0.0;
        sc->breakdown = 0;
        sc->done = 0;
        sc->iters = 0;
    }
}

__global__ void k_set_target(BcgScalars *sc, double target)
{
    sc->target = target;
    sc->done = 0;
    sc->iters = 0;
}

template <typename T>
M6<T> m6(const T *const m[6])
{
    return M6<T>{m[0], m[1], m[2], m[3], m[4], m[5]};
}

}  // namespace

dim3 solver_block() { return dim3(32, 4, 1); }
dim3 solver_grid(const Dims &d) { return dim3((d.I + 31) / 32, (d.J + 3) / 4, (d.K + KZ - 1) / KZ); }

template <typename T>
void bcg_iteration(const Dims &d, const T *const m[6], BcgVecs<T> &V, bool first, Reduce &R,
                   BcgScalars *sc, cudaStream_t st, cudaEvent_t *ev)
{
    const dim3 g = solver_grid(d), b = solver_block();
    const M6<T> M = m6(m);
    T *p = V.p, *v = V.v;
    if (ev) cudaEventRecord(ev[0], st);
    k_bcg_u<T><<<g, b, 0, st>>>(d, V.r, p, v, sc, first ? 1 : 0);
    if (ev) cudaEventRecord(ev[1], st);
    k_bcg_p<T><<<g, b, 0, st>>>(d, M, p, V.r0, v, sc, R.partials);
    if (ev) cudaEventRecord(ev[2], st);
    k_red_alpha<<<1, 1024, 0, st>>>(R.partials, R.nblocks, sc);
    if (ev) cudaEventRecord(ev[3], st);
    k_bcg_s<T><<<g, b, 0, st>>>(d, M, V.r, v, V.t, sc, R.partials);
    if (ev) cudaEventRecord(ev[4], st);
    k_red_omega<<<1, 1024, 0, st>>>(R.partials, R.nblocks, sc);
    if (ev) cudaEventRecord(ev[5], st);
    k_bcg_x<T><<<g, b, 0, st>>>(d, V.x, V.r, V.r0, p, v, V.t, sc, R.partials);
    if (ev) cudaEventRecord(ev[6], st);
    k_red_rho<<<1, 1024, 0, st>>>(R.partials, R.nblocks, sc);
}

void resid64(const Dims &d, const double *const m[6], const double *b, const double *x, double *r64, float *r32,
             bool want_bb, Reduce &R, BcgScalars *sc, cudaStream_t st)
{
    k_resid64<<<solver_grid(d), solver_block(), 0, st>>>(d, m6(m), b, x, r64, r32, want_bb ? 1 : 0, R.partials);
    k_red_resid<<<1, 1024, 0, st>>>(R.partials, R.nblocks, sc, want_bb ? 1 : 0);
}

void set_target(BcgScalars *sc, double target, cudaStream_t st)
{
    k_set_target<<<1, 1, 0, st>>>(sc, target);
}

void xadd(const Dims &d, double *x, const float *e, cudaStream_t st)
{
    k_xadd<<<solver_grid(d), solver_block(), 0, st>>>(d, x, e);
}

template void bcg_iteration<double>(const Dims &, const double *const[6], BcgVecs<double> &, bool, Reduce &,
                                    BcgScalars *, cudaStream_t, cudaEvent_t *);
template void bcg_iteration<float>(const Dims &, const float *const[6], BcgVecs<float> &, bool, Reduce &,
                                   BcgScalars *, cudaStream_t, cudaEvent_t *);

}  // namespace pred
