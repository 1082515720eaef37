// k_solver.cu -- multigrid-preconditioned CG on the 7-point pressure operator.
//
// Fine level: FP64 CG (SpMV, vector updates, dot products) on the ghosted
// layout.  Preconditioner: one V-cycle, T = double (FP64 mode) or T = float
// (mixed mode), with Chebyshev smoothing of the Jacobi-preconditioned
// operator, sum restriction, piecewise-constant prolongation, and a dense
// FP64 inverse on the coarsest level.  Coarse operators: per coarse face, the
// fine face conductances summed over the face and divided by the coarsening
// factor along the normal (the cell-centre distance doubles); the coarse
// diagonal is the sum of the coarse couplings plus half the children's
// Dirichlet terms.  Dot products are reduced per block and then in one block
// in a fixed order, so results are bitwise reproducible.
#include <stdint.h>

#include <atomic>

#include "scf_kernels.h"
#include "scf_tma.cuh"

#define INTERIOR_IJK(L)                                       \
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1; \
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1; \
    const int k = blockIdx.z * blockDim.z + threadIdx.z + 1; \
    const bool in = i <= (L).n0 && j <= (L).n1 && k <= (L).n2; \
    const int c = i + (L).sy * j + (L).sz * k;

// ---------------------------------------------------------------------------
// Jacobi scaling.  FP32 levels compute 1/diag on the fly with the hardware
// reciprocal (one instruction, and it saves one array per pass); FP64 levels
// read a stored inverse (FP64 division is slow on this GPU).  Inactive cells carry diag = -1 and
// get no update and no coarse correction.
template <typename T>
__device__ __forceinline__ T dinv_at(const LevelView<T> &L, int c);
template <>
__device__ __forceinline__ float dinv_at<float>(const LevelView<float> &L, int c)
{
    return jacobi_inv(L.diag[c]);
}
template <>
__device__ __forceinline__ double dinv_at<double>(const LevelView<double> &L, int c)
{
    return L.dinv[c];
}
template <typename T>
__device__ __forceinline__ bool active_at(const LevelView<T> &L, int c);
template <>
__device__ __forceinline__ bool active_at<float>(const LevelView<float> &L, int c)
{
    return L.diag[c] > 0.0f;
}
template <>
__device__ __forceinline__ bool active_at<double>(const LevelView<double> &L, int c)
{
    return __double_as_longlong(L.dinv[c]) != 0;
}

// ---------------------------------------------------------------------------
// reductions

enum ReduceMode { RM_STORE = 0, RM_BETA = 2, RM_MEAN = 3 };

__global__ void __launch_bounds__(1024) k_reduce(const double *__restrict__ part, int n, double *scal, int slot,
                                                 int mode)
{
    double s = 0.0;
    for (int t = threadIdx.x; t < n; t += blockDim.x) s += part[t];
    s = block_sum(s);
    if (threadIdx.x == 0) {
        if (mode == RM_BETA) {
            const double old = scal[S_RZ];
            scal[S_BETA] = old != 0.0 ? s / old : 0.0;
            scal[S_RZ] = s;
        } else if (mode == RM_MEAN) {
            scal[S_SUM] = s;
            scal[S_MEAN] = scal[S_COUNT] > 0.0 ? s / scal[S_COUNT] : 0.0;
        } else {
            scal[slot] = s;
        }
    }
}

void reduce_to(Reducer &R, int nblocks, int slot, cudaStream_t st, int *launches)
{
    k_reduce<<<1, 1024, 0, st>>>(R.partials, nblocks, R.scal, slot, RM_STORE);
    *launches += 1;
}

// ---------------------------------------------------------------------------
// FP64 CG kernels on the fine level

// Fine-level FP64 kernels march KZ cells along k per thread: the k-neighbours
// stay in registers and the FP64 block reduction (costly on this GPU's FP64
// pipe) is paid once per KZ cells.
constexpr int KZ = 32;

inline Launch3 launch_zchunk(int n0, int n1, int n2)
{
    Launch3 l;
    l.block = dim3(32, 4, 1);
    l.grid = dim3((n0 + 31) / 32, (n1 + 3) / 4, (n2 + KZ - 1) / KZ);
    return l;
}

#define ZCHUNK_IJK(L)                                                  \
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;          \
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;          \
    const int k0 = blockIdx.z * KZ + 1;                               \
    const int k1 = min(k0 + KZ - 1, (L).n2);                          \
    const bool in = i <= (L).n0 && j <= (L).n1;

// q = A p and the block partials of (p, q) and of the sum of q (q is zero on
// inactive cells, whose p is zero and which couple to nothing).
__global__ void __launch_bounds__(128) k_spmv_dot(LevelView<double> A, const double *__restrict__ p,
                                                  double *__restrict__ q, double *__restrict__ part, int n0)
{
    ZCHUNK_IJK(A);
    double v = 0.0, sq = 0.0;
    if (in) {
        int c = i + A.sy * j + A.sz * k0;
        double xm = p[c - A.sz], x0 = p[c], tb = A.cT[c - A.sz];
        for (int k = k0; k <= k1; ++k, c += A.sz) {
            const double xp = p[c + A.sz], tt = A.cT[c];
            const double y = A.diag[c] * x0 - (A.cE[c] * p[c + 1] + A.cE[c - 1] * p[c - 1] + A.cN[c] * p[c + A.sy] +
                                               A.cN[c - A.sy] * p[c - A.sy] + tt * xp + tb * xm);
            q[c] = y;
            v += x0 * y;
            sq += y;
            xm = x0; x0 = xp; tb = tt;
        }
    }
    v = block_sum(v);
    __syncthreads();
    sq = block_sum(sq);
    if (thread_linear() == 0) {
        part[block_linear()] = v;
        part[n0 + block_linear()] = sq;
    }
}

// alpha = (r, z) / (p, q); for an all-Neumann system also the mean of q over
// the active cells.  That mean is zero in exact arithmetic (the constant is
// the null vector of the symmetric operator); the CG update subtracts the
// rounding that it carries, so that the recursive residual stays in the
// range of the operator instead of collecting a component that no iterate
// can remove.
__global__ void __launch_bounds__(1024) k_reduce_alpha(const double *__restrict__ part, int n, int n0,
                                                       double *scal, int singular)
{
    double s = 0.0, t = 0.0;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        s += part[q];
        t += part[n0 + q];
    }
    s = block_sum(s);
    __syncthreads();
    t = block_sum(t);
    if (threadIdx.x == 0) {
        scal[S_PQ] = s;
        scal[S_ALPHA] = s != 0.0 ? scal[S_RZ] / s : 0.0;
        scal[S_QMEAN] = (singular && scal[S_COUNT] > 0.0) ? t / scal[S_COUNT] : 0.0;
    }
}

void reduce_alpha(Reducer &R, int nblocks, bool singular, cudaStream_t st, int *launches)
{
    k_reduce_alpha<<<1, 1024, 0, st>>>(R.partials, nblocks, R.max_blocks, R.scal, singular ? 1 : 0);
    *launches += 1;
}

void cg_spmv_dot(const LevelView<double> &A, const double *p, double *q, Reducer &R, bool singular,
                 cudaStream_t st, int *launches, KTimer *kt)
{
    Launch3 l = launch_zchunk(A.n0, A.n1, A.n2);
    const int id = kt_begin(kt, KC_SPMV, st);
    k_spmv_dot<<<l.grid, l.block, 0, st>>>(A, p, q, R.partials, R.max_blocks);
    kt_end(kt, id, st);
    k_reduce_alpha<<<1, 1024, 0, st>>>(R.partials, (int)nblocks(l), R.max_blocks, R.scal, singular ? 1 : 0);
    *launches += 2;
}

// x += alpha p, r -= alpha (q - mean q), (r, r); also writes the preconditioner's
// level-0 rhs (FP32 copy of r in mixed mode) and the first Chebyshev step
// of the V-cycle from a zero guess, x0 = dinv * r / theta, which saves that
// pass in the V-cycle.
template <typename T>
__global__ void __launch_bounds__(128) k_cg_update(LevelView<double> A, double *__restrict__ x,
                                                   double *__restrict__ r, const double *__restrict__ p,
                                                   const double *__restrict__ q, T *__restrict__ rlow,
                                                   LevelView<T> L0, T *__restrict__ x0, T first,
                                                   const double *__restrict__ scal, double *__restrict__ part)
{
    ZCHUNK_IJK(A);
    double v = 0.0;
    if (in) {
        const double alpha = scal[S_ALPHA], qm = scal[S_QMEAN];
        int c = i + A.sy * j + A.sz * k0;
        for (int k = k0; k <= k1; ++k, c += A.sz) {
            x[c] = x[c] + alpha * p[c];
            const double rn = r[c] - alpha * (q[c] - (active_at(L0, c) ? qm : 0.0));
            r[c] = rn;
            const T rl = (T)rn;
            if (rlow) rlow[c] = rl;
            if (x0) x0[c] = first * dinv_at(L0, c) * rl;
            v += rn * rn;
        }
    }
    v = block_sum(v);
    if (thread_linear() == 0) part[block_linear()] = v;
}

template <typename T>
void cg_update(const LevelView<double> &A, double *x, double *r, const double *p, const double *q, T *rlow,
               const LevelView<T> &L0, T *x0, double first, Reducer &R, cudaStream_t st, int *launches,
               KTimer *kt)
{
    Launch3 l = launch_zchunk(A.n0, A.n1, A.n2);
    const int id = kt_begin(kt, KC_CGUPDATE, st);
    k_cg_update<T><<<l.grid, l.block, 0, st>>>(A, x, r, p, q, rlow, L0, x0, (T)first, R.scal, R.partials);
    kt_end(kt, id, st);
    *launches += 1;
    reduce_to(R, (int)nblocks(l), S_RR, st, launches);
}

// (r, z): in mixed mode r is taken from its FP32 copy (the V-cycle's rhs) and
// the products are formed in FP32, accumulated per thread in FP32 over KZ
// cells and across threads in FP64; z is an FP32 preconditioner output, so
// this loses nothing that matters for beta.  FP64 mode: FP64 throughout.
template <typename T>
__global__ void __launch_bounds__(128) k_dot_rz(LevelView<double> A, const double *__restrict__ r,
                                                const T *__restrict__ rlow, const T *__restrict__ z,
                                                double *__restrict__ part)
{
    ZCHUNK_IJK(A);
    double v = 0.0;
    if (in) {
        int c = i + A.sy * j + A.sz * k0;
        if (sizeof(T) == 4) {
            float acc = 0.f;
            for (int k = k0; k <= k1; ++k, c += A.sz) acc += (float)rlow[c] * (float)z[c];
            v = (double)acc;
        } else {
            for (int k = k0; k <= k1; ++k, c += A.sz) v += r[c] * (double)z[c];
        }
    }
    v = block_sum(v);
    if (thread_linear() == 0) part[block_linear()] = v;
}

template <typename T>
void cg_dot_rz(const LevelView<double> &A, const double *r, const T *rlow, const T *z, Reducer &R, cudaStream_t st,
               int *launches)
{
    Launch3 l = launch_zchunk(A.n0, A.n1, A.n2);
    k_dot_rz<T><<<l.grid, l.block, 0, st>>>(A, r, rlow, z, R.partials);
    k_reduce<<<1, 1024, 0, st>>>(R.partials, (int)nblocks(l), R.scal, 0, RM_BETA);
    *launches += 2;
}

void reduce_beta(Reducer &R, int nblocks, cudaStream_t st, int *launches)
{
    k_reduce<<<1, 1024, 0, st>>>(R.partials, nblocks, R.scal, 0, RM_BETA);
    *launches += 1;
}

template <typename T>
__global__ void __launch_bounds__(128) k_pupdate(LevelView<double> A, const T *__restrict__ z,
                                                 double *__restrict__ p, const double *__restrict__ scal, int first)
{
    ZCHUNK_IJK(A);
    if (!in) return;
    const double beta = first ? 0.0 : scal[S_BETA];
    int c = i + A.sy * j + A.sz * k0;
    for (int k = k0; k <= k1; ++k, c += A.sz) {
        const double zz = (double)z[c];
        p[c] = first ? zz : zz + beta * p[c];
    }
}

template <typename T>
void cg_pupdate(const LevelView<double> &A, const T *z, double *p, const double *scal, bool first, cudaStream_t st,
                int *launches)
{
    Launch3 l = launch_zchunk(A.n0, A.n1, A.n2);
    k_pupdate<T><<<l.grid, l.block, 0, st>>>(A, z, p, scal, first ? 1 : 0);
    *launches += 1;
}

// two-slot reduction: sums of part[0..n) and part[n0..n0+n)
__global__ void __launch_bounds__(1024) k_reduce2(const double *__restrict__ part, int n, int n0,
                                                  double *scal, int mode)
{
    double s = 0.0, t = 0.0;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        s += part[q];
        t += part[n0 + q];
    }
    s = block_sum(s);
    __syncthreads();
    t = block_sum(t);
    if (threadIdx.x == 0) {
        if (mode == 0) {           // sum of b, count
            scal[S_SUM] = s;
            scal[S_COUNT] = t;
            scal[S_MEAN] = t > 0.0 ? s / t : 0.0;
        } else if (mode == 1) {    // (r, r), sum of x
            scal[S_RR] = s;
            scal[S_MEANX] = scal[S_COUNT] > 0.0 ? t / scal[S_COUNT] : 0.0;
        } else {                   // loss terms
            scal[S_JP] = s;
            scal[S_JD] = t;
        }
    }
}

__global__ void __launch_bounds__(128) k_sum_count(LevelView<double> A, const unsigned char *__restrict__ act,
                                                   const double *__restrict__ v, double *__restrict__ part, int n0)
{
    ZCHUNK_IJK(A);
    double s = 0.0, cnt = 0.0;
    if (in) {
        int c = i + A.sy * j + A.sz * k0;
        for (int k = k0; k <= k1; ++k, c += A.sz)
            if (act[c]) { s += v[c]; cnt += 1.0; }
    }
    s = block_sum(s);
    __syncthreads();
    cnt = block_sum(cnt);
    if (thread_linear() == 0) {
        part[block_linear()] = s;
        part[n0 + block_linear()] = cnt;
    }
}

__global__ void __launch_bounds__(128) k_center_norm(LevelView<double> A, const unsigned char *__restrict__ act,
                                                     double *__restrict__ b, const double *__restrict__ scal,
                                                     int singular, double *__restrict__ part)
{
    ZCHUNK_IJK(A);
    double s = 0.0;
    if (in) {
        const double mu = singular ? scal[S_MEAN] : 0.0;
        int c = i + A.sy * j + A.sz * k0;
        for (int k = k0; k <= k1; ++k, c += A.sz) {
            double v = b[c];
            if (singular && act[c]) { v = v - mu; b[c] = v; }
            s += v * v;
        }
    }
    s = block_sum(s);
    if (thread_linear() == 0) part[block_linear()] = s;
}

void reduce2_to(Reducer &R, int nblocks, int mode, cudaStream_t st, int *launches)
{
    k_reduce2<<<1, 1024, 0, st>>>(R.partials, nblocks, R.max_blocks, R.scal, mode);
    *launches += 1;
}

void active_mean(const LevelView<double> &A, const unsigned char *active, const double *v, Reducer &R,
                 cudaStream_t st, int *launches)
{
    Launch3 l = launch_zchunk(A.n0, A.n1, A.n2);
    k_sum_count<<<l.grid, l.block, 0, st>>>(A, active, v, R.partials, R.max_blocks);
    *launches += 1;
    reduce2_to(R, (int)nblocks(l), 0, st, launches);
}

void rhs_prologue(const LevelView<double> &A, const unsigned char *active, double *b, bool singular, Reducer &R,
                  cudaStream_t st, int *launches)
{
    Launch3 l = launch_zchunk(A.n0, A.n1, A.n2);
    const int nb = (int)nblocks(l);
    if (singular) {
        k_sum_count<<<l.grid, l.block, 0, st>>>(A, active, b, R.partials, R.max_blocks);
        k_reduce2<<<1, 1024, 0, st>>>(R.partials, nb, R.max_blocks, R.scal, 0);
        *launches += 2;
    }
    k_center_norm<<<l.grid, l.block, 0, st>>>(A, active, b, R.scal, singular ? 1 : 0, R.partials);
    k_reduce<<<1, 1024, 0, st>>>(R.partials, nb, R.scal, S_BB, RM_STORE);
    *launches += 2;
}

__global__ void __launch_bounds__(128) k_final_residual(LevelView<double> A, const unsigned char *__restrict__ act,
                                                        const double *__restrict__ b, const double *__restrict__ x,
                                                        double *__restrict__ r, int singular,
                                                        double *__restrict__ part, int n0)
{
    ZCHUNK_IJK(A);
    double s = 0.0, sx = 0.0;
    if (in) {
        int c = i + A.sy * j + A.sz * k0;
        for (int k = k0; k <= k1; ++k, c += A.sz) {
            const double rr = b[c] - apply_row(A, x, c);
            r[c] = rr;
            s += rr * rr;
            if (singular && act[c]) sx += x[c];
        }
    }
    s = block_sum(s);
    __syncthreads();
    sx = block_sum(sx);
    if (thread_linear() == 0) {
        part[block_linear()] = s;
        part[n0 + block_linear()] = sx;
    }
}

void final_residual(const LevelView<double> &A, const unsigned char *active, const double *b, const double *x,
                    double *r, bool singular, Reducer &R, cudaStream_t st, int *launches)
{
    Launch3 l = launch_zchunk(A.n0, A.n1, A.n2);
    const int nb = (int)nblocks(l);
    k_final_residual<<<l.grid, l.block, 0, st>>>(A, active, b, x, r, singular ? 1 : 0, R.partials, R.max_blocks);
    k_reduce2<<<1, 1024, 0, st>>>(R.partials, nb, R.max_blocks, R.scal, 1);
    *launches += 2;
}

__global__ void __launch_bounds__(128) k_shift(LevelView<double> A, const unsigned char *__restrict__ act,
                                               double *__restrict__ x, const double *__restrict__ scal)
{
    ZCHUNK_IJK(A);
    if (!in) return;
    const double mu = scal[S_MEANX];
    int c = i + A.sy * j + A.sz * k0;
    for (int k = k0; k <= k1; ++k, c += A.sz)
        if (act[c]) x[c] = x[c] - mu;
}

void shift_solution(const LevelView<double> &A, const unsigned char *active, double *x, const double *scal,
                    cudaStream_t st, int *launches)
{
    Launch3 l = launch_zchunk(A.n0, A.n1, A.n2);
    k_shift<<<l.grid, l.block, 0, st>>>(A, active, x, scal);
    *launches += 1;
}

__global__ void __launch_bounds__(256) k_copy_low(LevelView<double> A, const double *__restrict__ s,
                                                  float *__restrict__ d)
{
    INTERIOR_IJK(A);
    if (in) d[c] = (float)s[c];
}

void copy_to_low(const LevelView<double> &A, const double *src, float *dst, cudaStream_t st, int *launches)
{
    Launch3 l = launch_interior(A.n0, A.n1, A.n2);
    k_copy_low<<<l.grid, l.block, 0, st>>>(A, src, dst);
    *launches += 1;
}

// ---------------------------------------------------------------------------
// V-cycle kernels

template <typename T>
__global__ void __launch_bounds__(256) k_cheb_first(LevelView<T> L, const T *__restrict__ b, T *__restrict__ x,
                                                    T coef)
{
    INTERIOR_IJK(L);
    if (in) x[c] = coef * dinv_at(L, c) * b[c];
}

// Arithmetic of one Chebyshev update with every operation spelled out (no
// contraction left to the compiler), so that the one-step kernel and the
// fused two-step kernel give the same bits: the six neighbour products
// summed by FMA in the order E, W, N, S, T, B; A x = diag x - s;
// r = b - A x; the update dn = (c2 dinv) r + c1 dprev.
__device__ __forceinline__ float fx_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double fx_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float fx_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fx_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fx_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double fx_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float fx_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double fx_add(double a, double b) { return __dadd_rn(a, b); }

// r = b - A x of one cell, the residual both the Chebyshev update and the
// restriction use, so a fused residual gives the bits of a separate one.
template <typename T>
__device__ __forceinline__ T cheb_residual(T b, T dg, T x0, T xe, T xw, T xn, T xs, T xt, T xb, T ce, T cw, T cn,
                                           T cs, T ct, T cb)
{
    T s = fx_mul(ce, xe);
    s = fx_fma(cw, xw, s);
    s = fx_fma(cn, xn, s);
    s = fx_fma(cs, xs, s);
    s = fx_fma(ct, xt, s);
    s = fx_fma(cb, xb, s);
    return fx_sub(b, fx_fma(dg, x0, -s));
}

template <typename T>
__device__ __forceinline__ T cheb_update(T b, T dg, T dinv, T x0, T xe, T xw, T xn, T xs, T xt, T xb, T ce, T cw,
                                         T cn, T cs, T ct, T cb, T dprev, T c1, T c2)
{
    const T r = cheb_residual(b, dg, x0, xe, xw, xn, xs, xt, xb, ce, cw, cn, cs, ct, cb);
    return fx_fma(fx_mul(c2, dinv), r, fx_mul(c1, dprev));
}

template <typename T>
__global__ void __launch_bounds__(256) k_cheb_step(LevelView<T> L, const T *__restrict__ b,
                                                   const T *__restrict__ xin, const T *dprev,
                                                   T *__restrict__ xout, T *dout, T c1, T c2)
{
    INTERIOR_IJK(L);
    if (!in) return;
    const int sy = L.sy, sz = L.sz;
    const T x0 = xin[c];
    const T dn = cheb_update(b[c], L.diag[c], dinv_at(L, c), x0, xin[c + 1], xin[c - 1], xin[c + sy], xin[c - sy],
                             xin[c + sz], xin[c - sz], L.cE[c], L.cE[c - 1], L.cN[c], L.cN[c - sy], L.cT[c],
                             L.cT[c - sz], dprev[c], c1, c2);
    xout[c] = fx_add(x0, dn);
    if (dout) dout[c] = dn;
}

// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// Two Chebyshev steps in one pass over a large FP32 level (2.5-D temporal
// blocking), with the inputs staged by the Tensor Memory Accelerator.
//
// A block of 256 threads owns a tile of 32 x 8 (i, j) columns and marches
// along k over `planes` planes.  Group P holds plane P's inputs on the tile
// and its halo (b, diag, cT and the previous update on 34 x 10 cells, cE one
// column wider to the west, cN one row wider to the south) and x of plane P
// with a two-cell halo.  For plane kk the block
//   1. has one thread issue the TMA copies of group kk + 2 into a four-slot
//      ring in shared memory; they complete on that slot's mbarrier;
//   2. waits for group kk + 1 (groups kk - 1 and kk landed earlier) and
//      applies the first step on the 34 x 10 cells of plane kk (ghost cells
//      give 0, the value the one-step kernel leaves there) into a four-plane
//      ring in shared memory;
//   3. after one block barrier, applies the second step on the 32 x 8 cells
//      of plane kk - 1.
// The first step's 84 halo cells go to the first three warps, so the other
// five carry no halo code path.  (Tiles of 32 x 16 with 512 threads, a 20%
// halo instead of 33%, measured slower: 0.158 against 0.155 ms per pair at
// 256^3.)
// The four-deep rings make that single barrier per plane enough: the slot a
// copy or a first step overwrites was last read before the previous
// plane's barrier.  Each array is read from DRAM about once per pass (halo
// columns come from L2), so two steps move about the bytes of one, and no
// thread spends instructions on copies.  Both steps go through cheb_update:
// the result is that of two k_cheb_step launches, bit for bit.  The output
// x must not be the input x, nor dout the previous update when both are
// given: neighbouring tiles read their halos from them.
//
// Row pairs.  TMA wants every global stride to be a multiple of 16 bytes; a
// row of the padded layout (n0 + 2 floats) is one only when n0 + 2 is a
// multiple of 4, but with n0 even two consecutive rows are.  So the tensor
// map views a level as (2 sy, (n1 + 2) / 2, n2 + 2) floats -- row pair, row
// pairs, planes -- and each array's tile arrives as two boxes: one over the
// even rows of its row pairs (x = i) and one over the odd rows (x = sy + i).
// A box's first x is rounded down to a multiple of 4 floats (16 bytes), as
// TMA requires; the tile's columns then start 0, 2 or 4 floats into it.
// Coordinates outside the tensor (the ghost ring's outside, a last unpaired
// row when n1 is odd, planes -1 and n2 + 2) read as 0.  Conditions: n0 even
// and sy (n1 + 2) a multiple of 4 (the plane stride in 16-byte units);
// other levels smooth with one-step launches.
constexpr int C2_TX = 32, C2_TY = 8, C2_THREADS = C2_TX * C2_TY;
constexpr int C2_BLOCKS_PER_SM = 4;
constexpr int C2_EX = C2_TX + 2, C2_EY = C2_TY + 2, C2_NE = C2_EX * C2_EY;  // first-step cells, from (i0-1, j0-1)
constexpr int C2_NH = C2_NE - C2_THREADS;                                // halo cells of step 1
// box widths (floats) and heights (row pairs): b, diag, cT, dprev and cN
// from column i0 - 1 (36 wide), cE and x from column i0 - 2 (40 wide); b,
// diag, cT, dprev and cE from row j0 - 1 (C2_TY/2 + 1 pairs), cN from row
// j0 - 3 (one pair more), x from row j0 - 3 (two pairs more)
constexpr int C2_WA = 36, C2_WE = 40, C2_HA = C2_TY / 2 + 1, C2_HN = C2_HA + 1, C2_HX = C2_HA + 2;
// one box per parity, each starting on a 128-byte boundary (floats)
constexpr int c2_round(int v) { return (v + 31) / 32 * 32; }
constexpr int C2_BA = c2_round(C2_WA * C2_HA), C2_BE = c2_round(C2_WE * C2_HA), C2_BN = c2_round(C2_WA * C2_HN),
              C2_BX = c2_round(C2_WE * C2_HX);
static_assert(C2_TY % 2 == 0, "tiles of whole row pairs");
static_assert(C2_WA * C2_HA <= C2_BA && C2_WE * C2_HA <= C2_BE && C2_WA * C2_HN <= C2_BN && C2_WE * C2_HX <= C2_BX,
              "boxes fit their slots");
static_assert(C2_BA % 32 == 0 && C2_BE % 32 == 0 && C2_BN % 32 == 0 && C2_BX % 32 == 0, "128-byte boxes");
// a group slot: b, diag, cT, dprev, cE, cN, x (two boxes each)
constexpr int C2_GB = 0, C2_GD = 2 * C2_BA, C2_GT = 4 * C2_BA, C2_GP = 6 * C2_BA, C2_GE = 8 * C2_BA,
              C2_GN = C2_GE + 2 * C2_BE, C2_GX = C2_GN + 2 * C2_BN, C2_SLOT = C2_GX + 2 * C2_BX;
constexpr int C2_DEPTH = 4;                                 // group slots (ring of planes)
constexpr int C2_R1 = 4;                                    // first-step result planes
constexpr int C2_R1N = ((C2_R1 * C2_NE + 31) / 32) * 32;    // floats, rounded to 128 bytes
// restriction mode: the second rows' residuals of a plane pair, handed to
// the first rows through shared memory (two buffers, by coarse plane parity)
constexpr int C2_XCH = 2 * (C2_TY / 2) * C2_TX;                  // float2 entries
constexpr size_t C2_SMEM = 128 + sizeof(float) * (C2_DEPTH * C2_SLOT + C2_R1N) + 8 * C2_DEPTH + 8 * C2_XCH;
constexpr int C2_PLANES = 32;
// bytes a group's copies deliver (full boxes, out-of-range parts as 0)
constexpr unsigned C2_TX_BYTES_NODP = 2u * 4u * (3 * C2_WA * C2_HA + C2_WE * C2_HA + C2_WA * C2_HN + C2_WE * C2_HX);
constexpr unsigned C2_TX_BYTES_DP = C2_TX_BYTES_NODP + 2u * 4u * C2_WA * C2_HA;
static_assert(C2_NH <= C2_THREADS, "one halo cell per thread at most");

// tensor maps of the pair kernel's inputs: b, diag, cT, dprev, cE, cN, x
struct PairMaps {
    CUtensorMap m[7];
};

struct PairArgs {
    LevelView<float> F;
    float *xout, *dout;          // dout nullptr: the second step's update is not kept
    unsigned *flags;             // FLAG_WAIT_TIMEOUT if a copy never landed
    float c1a, c2a, c1b, c2b;
    int planes;
    LevelView<float> C;          // restriction mode: the coarse level and its rhs
    float *bc;
    float *xc;                   // and, unless null, its first smoothing step (factor firstc)
    float firstc;
};

// Offsets in a group slot (floats) of one first-step cell (ex, ey) of the
// 34 x 10 tile: its b/diag/cT/dprev element (a), cE (e; cE of the west
// neighbour at e - 1), cN (n) and cN of the south neighbour (s), x (x; east
// and west at x +- 1) and x of the north and south neighbours (xn, xs).
// shA/shE: the column in a box of the tile's first column, per row parity.
struct C2Idx {
    int a, e, n, s, x, xn, xs;
};

__device__ __forceinline__ C2Idx c2_idx(int ex, int ey, const int shA[2], const int shE[2])
{
    const int p = ey & 1, q = p ^ 1;
    C2Idx t;
    t.a = p * C2_BA + (ey >> 1) * C2_WA + ex + shA[p];
    t.e = C2_GE + p * C2_BE + (ey >> 1) * C2_WE + ex + shE[p];
    t.n = C2_GN + p * C2_BN + ((ey + 2) >> 1) * C2_WA + ex + shA[p];
    t.s = C2_GN + q * C2_BN + ((ey + 1) >> 1) * C2_WA + ex + shA[q];
    t.x = C2_GX + p * C2_BX + ((ey + 2) >> 1) * C2_WE + ex + shE[p];
    t.xn = C2_GX + q * C2_BX + ((ey + 3) >> 1) * C2_WE + ex + shE[q];
    t.xs = C2_GX + q * C2_BX + ((ey + 1) >> 1) * C2_WE + ex + shE[q];
    return t;
}

struct C2Cell {
    float b, dg, dinv, ce, cw, cn, cs, ct, cb;
};

// First step on one cell: G, Gm, Gp the group slots of planes kk, kk - 1,
// kk + 1; x after the step written at o1[q]; `in` whether the cell is
// interior.  Returns the update and the cell's inputs.
template <bool DP>
__device__ __forceinline__ float c2_first(const PairArgs &a, const float *G, const float *Gm, const float *Gp,
                                          const C2Idx &t, float *o1, int q, bool in, C2Cell &k)
{
    if (!in) {
        o1[q] = 0.f;
        return 0.f;
    }
    k.b = G[C2_GB + t.a];
    k.dg = G[C2_GD + t.a];
    k.dinv = jacobi_inv(k.dg);
    k.ce = G[t.e];
    k.cw = G[t.e - 1];
    k.cn = G[t.n];
    k.cs = G[t.s];
    k.ct = G[C2_GT + t.a];
    k.cb = Gm[C2_GT + t.a];
    const float xc = G[t.x];
    const float dn = cheb_update(k.b, k.dg, k.dinv, xc, G[t.x + 1], G[t.x - 1], G[t.xn], G[t.xs], Gp[t.x],
                                 Gm[t.x], k.ce, k.cw, k.cn, k.cs, k.ct, k.cb, DP ? G[C2_GP + t.a] : xc, a.c1a,
                                 a.c2a);
    o1[q] = fx_add(xc, dn);
    return dn;
}

// RS (restriction mode, with DP and without DO): the first step is the last
// pre-smoothing step, written to xout, and the second phase forms its
// residual and restricts it to the coarse right-hand side a.bc, as
// k_restrict would (planes per block even, coarsening factors 2).
template <bool DP, bool DO, bool RS>
__global__ void __launch_bounds__(C2_THREADS, C2_BLOCKS_PER_SM) k_cheb_pair(const __grid_constant__ PairMaps tm,
                                                                          PairArgs a)
{
    extern __shared__ __align__(128) float c2_raw[];
    const unsigned raw = (unsigned)__cvta_generic_to_shared(c2_raw);
    const unsigned sb = (raw + 127u) & ~127u;            // 128-byte aligned start of the rings
    float *S = c2_raw + (sb - raw) / 4;
    float *R1 = S + C2_DEPTH * C2_SLOT;                  // first-step results, C2_R1 planes of 34 x 10
    const unsigned bar0 = sb + 4u * (C2_DEPTH * C2_SLOT + C2_R1N);
    const LevelView<float> &F = a.F;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + C2_TX * ty;
    const int bx = blockIdx.x * C2_TX, by = blockIdx.y * C2_TY;   // (i0 - 1, j0 - 1)
    const int i0 = bx + 1, j0 = by + 1;
    const int k0 = blockIdx.z * a.planes + 1, k1 = min(k0 + a.planes - 1, F.n2);
    // the tile's first column in each box, per row parity (box origins: x
    // rounded down to a multiple of 4 floats)
    int shA[2], shE[2];
#pragma unroll
    for (int p = 0; p < 2; ++p) {
        shA[p] = (p * F.sy + bx) & 3;
        shE[p] = p * F.sy + bx - ((p * F.sy + bx - 1) & ~3);
    }
    // this thread's column (tx + 1, ty + 1) of the 34 x 10 tile and its halo
    // cell (the ring around the 32 x 8 tile)
    const C2Idx t0 = c2_idx(tx + 1, ty + 1, shA, shE);
    const int q0 = (tx + 1) + C2_EX * (ty + 1);
    const bool in0 = i0 + tx <= F.n0 && j0 + ty <= F.n1;
    int hx = -1, hy = 0;
    if (tid < C2_EX) { hx = tid; hy = 0; }
    else if (tid < 2 * C2_EX) { hx = tid - C2_EX; hy = C2_EY - 1; }
    else if (tid < 2 * C2_EX + C2_TY) { hx = 0; hy = tid - 2 * C2_EX + 1; }
    else if (tid < C2_NH) { hx = C2_EX - 1; hy = tid - 2 * C2_EX - C2_TY + 1; }
    const bool halo = hx >= 0;
    const C2Idx th = c2_idx(halo ? hx : 0, hy, shA, shE);
    const int qh = (halo ? hx : 0) + C2_EX * hy;
    const bool inh = halo && bx + hx >= 1 && bx + hx <= F.n0 && by + hy >= 1 && by + hy <= F.n1;

    // restriction mode: this thread's row is the first (j odd) or second of
    // its row pair; the first rows finish a coarse cell one plane after its
    // last fine plane, from the second rows' residuals in xch
    float2 *xch = reinterpret_cast<float2 *>(S + C2_DEPTH * C2_SLOT + C2_R1N + 2 * C2_DEPTH);
    const bool row_ok = j0 + ty <= F.n1;
    const bool first_row = (ty & 1) == 0;
    const bool has_second = j0 + ty + 1 <= F.n1;
    float r0 = 0.f, sacc = 0.f;       // residual of the pair's first plane; the first row's partial sum
    int pendK = 0;                    // coarse plane awaiting completion (0: none)
    bool pend_two = false;            // it had two fine planes
    auto complete = [&]() {           // first rows: add the second row's residuals, then lanes i, i^1
        float sres = sacc;
        if (has_second) {
            const float2 v = xch[(pendK & 1) * (C2_TY / 2) * C2_TX + (ty >> 1) * C2_TX + tx];
            sres = fx_add(sres, v.x);
            if (pend_two) sres = fx_add(sres, v.y);
        }
        const float o = __shfl_xor_sync(0xffffffffu, sres, 1);
        const int i = i0 + tx;
        if ((tx & 1) == 0 && i <= F.n0) {
            sres = fx_add(sres, o);
            const int cc = (((i - 1) >> 1) + 1) + a.C.sy * (((j0 + ty - 1) >> 1) + 1) + a.C.sz * pendK;
            a.bc[cc] = sres;
            if (a.xc) a.xc[cc] = a.firstc * jacobi_inv(a.C.diag[cc]) * sres;
        }
    };

    const int g0 = k0 - 2, glast = k1 + 2;               // groups this block needs
    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < C2_DEPTH; ++s) mbar_init(bar0 + 8u * s, 1u);
        mbar_fence_init();
    }
    __syncthreads();
    // group P: slot (P - g0) mod 4, phase parity ((P - g0) / 4) mod 2
    // (thread 0 only; box origins recomputed here rather than held in
    // registers by every thread)
    auto issue = [&](int P) {
        const int s = (P - g0) & (C2_DEPTH - 1);
        const unsigned dst = sb + 4u * (unsigned)(s * C2_SLOT), bar = bar0 + 8u * s;
        const int bxi = blockIdx.x * C2_TX, yA = blockIdx.y * (C2_TY / 2), yN = yA - 1;
        mbar_expect_tx(bar, DP ? C2_TX_BYTES_DP : C2_TX_BYTES_NODP);
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            const int xA = (p * F.sy + bxi) & ~3, xE = (p * F.sy + bxi - 1) & ~3;
            tma_load3(dst + 4u * (C2_GB + p * C2_BA), &tm.m[0], xA, yA, P, bar);
            tma_load3(dst + 4u * (C2_GD + p * C2_BA), &tm.m[1], xA, yA, P, bar);
            tma_load3(dst + 4u * (C2_GT + p * C2_BA), &tm.m[2], xA, yA, P, bar);
            if (DP) tma_load3(dst + 4u * (C2_GP + p * C2_BA), &tm.m[3], xA, yA, P, bar);
            tma_load3(dst + 4u * (C2_GE + p * C2_BE), &tm.m[4], xE, yA, P, bar);
            tma_load3(dst + 4u * (C2_GN + p * C2_BN), &tm.m[5], xA, yN, P, bar);
            tma_load3(dst + 4u * (C2_GX + p * C2_BX), &tm.m[6], xE, yN, P, bar);
        }
    };
    // a block has at least five groups (g0 .. g0 + 4 <= glast)
    if (tid == 0)
        for (int P = g0; P <= g0 + 2; ++P) issue(P);
    bool gave_up = false;
    if (!mbar_wait(bar0, 0u)) gave_up = true;          // group g0
    if (!mbar_wait(bar0 + 8u, 0u)) gave_up = true;     // group g0 + 1
    float d1 = 0.f;             // first-step update of this thread's column, plane below
    C2Cell kc = {}, kp = {};
    const bool out_ok = in0;
    int c = (i0 + tx) + F.sy * (j0 + ty) + F.sz * (k0 - 2);   // output cell at plane kk - 1
    // iteration it handles plane kk = k0 - 1 + it; every ring index is a
    // function of it mod 4, so the unrolled copies address shared memory
    // with constant offsets: groups kk - 1, kk, kk + 1 in slots it, it + 1,
    // it + 2 (mod 4), first-step results of plane kk in R1 slot it mod 4
    const int nit = k1 - k0 + 3;
#pragma unroll 4
    for (int it = 0; it < nit; ++it, c += F.sz) {
        const int kk = k0 - 1 + it;
        if (tid == 0 && kk + 2 <= glast) issue(kk + 2);
        if (!mbar_wait(bar0 + 8u * ((it + 2) & (C2_DEPTH - 1)), (unsigned)((it + 2) >> 2) & 1u))
            gave_up = true;    // group kk + 1
        const float *G = S + ((it + 1) & (C2_DEPTH - 1)) * C2_SLOT;
        const float *Gm = S + (it & (C2_DEPTH - 1)) * C2_SLOT;
        const float *Gp = S + ((it + 2) & (C2_DEPTH - 1)) * C2_SLOT;
        float *o1 = R1 + (it & (C2_R1 - 1)) * C2_NE;
        const bool plane_in = kk >= 1 && kk <= F.n2;
        const float dn1 = c2_first<DP>(a, G, Gm, Gp, t0, o1, q0, in0 && plane_in, kc);
        if (halo) {
            C2Cell kh;
            c2_first<DP>(a, G, Gm, Gp, th, o1, qh, inh && plane_in, kh);
        }
        __syncthreads();
        if constexpr (RS) {
            // the smoothed x of plane kk - 1, its residual, and the restriction
            // of the plane pair it ends
            if (it >= 2 && row_ok) {
                if (pendK && first_row) complete();
                pendK = 0;
                const int pk = kk - 1;
                const float *y0 = R1 + ((it + 3) & (C2_R1 - 1)) * C2_NE;
                const float *ym = R1 + ((it + 2) & (C2_R1 - 1)) * C2_NE;
                const float *yp = o1;
                const int q = q0;
                float r = 0.f;
                if (out_ok) {
                    const float xc = y0[q];
                    a.xout[c] = xc;
                    r = cheb_residual(kp.b, kp.dg, xc, y0[q + 1], y0[q - 1], y0[q + C2_EX], y0[q - C2_EX], yp[q],
                                      ym[q], kp.ce, kp.cw, kp.cn, kp.cs, kp.ct, kp.cb);
                }
                const bool pfirst = (pk & 1) != 0;
                if (pfirst) r0 = r;
                if (!pfirst || pk == F.n2) {      // the pair ends at this plane
                    const int K = ((pk - 1) >> 1) + 1;
                    if (first_row) {
                        sacc = fx_add(0.f, r0);
                        if (!pfirst) sacc = fx_add(sacc, r);
                    } else {
                        xch[(K & 1) * (C2_TY / 2) * C2_TX + (ty >> 1) * C2_TX + tx] = make_float2(r0, r);
                    }
                    pendK = K;
                    pend_two = !pfirst;
                }
            }
        } else if (it >= 2 && out_ok) {
            // second step at plane kk - 1 from the first-step planes kk - 2 .. kk
            const float *y0 = R1 + ((it + 3) & (C2_R1 - 1)) * C2_NE;
            const float *ym = R1 + ((it + 2) & (C2_R1 - 1)) * C2_NE;
            const float *yp = o1;
            const int q = q0;
            const float xc = y0[q];
            const float dn = cheb_update(kp.b, kp.dg, kp.dinv, xc, y0[q + 1], y0[q - 1], y0[q + C2_EX],
                                         y0[q - C2_EX], yp[q], ym[q], kp.ce, kp.cw, kp.cn, kp.cs, kp.ct, kp.cb, d1,
                                         a.c1b, a.c2b);
            a.xout[c] = fx_add(xc, dn);
            if (DO) a.dout[c] = dn;
        }
        d1 = dn1;
        kp = kc;
    }
    if constexpr (RS) {
        __syncthreads();
        if (pendK && first_row && row_ok) complete();
    }
    if (gave_up) {
        atomicOr(a.flags, (unsigned)FLAG_WAIT_TIMEOUT);
        // no copy may still be writing into this block's shared memory when
        // it exits: wait once more (bounded) for the last groups issued
        if (tid == 0)
            for (int P = glast - (C2_DEPTH - 1) > g0 ? glast - (C2_DEPTH - 1) : g0; P <= glast; ++P)
                mbar_wait(bar0 + 8u * ((P - g0) & (C2_DEPTH - 1)), (unsigned)((P - g0) >> 2) & 1u);
    }
}

// Smoother pairing: 1 (the default) on the levels where the pair kernel
// measured faster than two one-step launches -- at least 2^22 cells, with
// at least two waves of blocks -- 2 on every FP32 level of at
// least 2^18 cells, 0 off; k-planes per block of the pair kernel (fewer
// when that fills the grid).
static int g_pairs = 1, g_pair_planes = C2_PLANES;
// launches of the TMA pair kernel, and pairs that ran as one-step launches
// because a tensor map did not encode (process-wide)
static std::atomic<long long> g_pair_tma{0}, g_pair_fallback{0};

void smoother_pair_counts(long long *tma, long long *fallback)
{
    *tma = g_pair_tma.load();
    *fallback = g_pair_fallback.load();
}

void set_smoother_pairs(int on, int planes)
{
    g_pairs = on < 0 ? 0 : (on > 2 ? 2 : on);
    g_pair_planes = planes > 0 ? planes : C2_PLANES;
}

int smoother_pairs_state() { return g_pairs + 3 * g_pair_planes; }

PFN_cuTensorMapEncodeTiled_v12000 tma_encode_fn()
{
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

bool tma_pair_shape_ok(int n0, int n1, int sy)
{
    return (n0 & 1) == 0 && ((long long)sy * (n1 + 2)) % 4 == 0;
}

bool tma_encode_f32_pairs(CUtensorMap *m, const float *base, int n0, int n1, int n2, int sy, int sz, int w, int h)
{
    const PFN_cuTensorMapEncodeTiled_v12000 fn = tma_encode_fn();
    if (!fn || !base || ((uintptr_t)base & 15u) || !tma_pair_shape_ok(n0, n1, sy)) return false;
    const cuuint64_t dim[3] = {(cuuint64_t)(2 * sy), (cuuint64_t)((n1 + 2) / 2), (cuuint64_t)(n2 + 2)};
    const cuuint64_t stride[2] = {(cuuint64_t)(2 * sy) * 4u, (cuuint64_t)sz * 4u};
    const cuuint32_t box[3] = {(cuuint32_t)w, (cuuint32_t)h, 1u};
    const cuuint32_t estride[3] = {1u, 1u, 1u};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dim, stride, box, estride,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

namespace {
// Tensor map of one FP32 array of level F in the row-pair view.
bool encode_pair_map(CUtensorMap *m, const float *base, const LevelView<float> &F, int w, int h)
{
    return tma_encode_f32_pairs(m, base, F.n0, F.n1, F.n2, F.sy, F.sz, w, h);
}
}  // namespace

// k-planes per block of the pair kernel on level F, 0: one-step kernels.
template <typename T>
int pair_planes(const MgLevel<T> &F)
{
    const long long cells = (long long)F.n0 * F.n1 * F.n2;
    if (sizeof(T) != 4 || g_pairs == 0 || cells < (1LL << 18) || !tma_pair_shape_ok(F.n0, F.n1, F.sy) ||
        !tma_encode_fn())
        return 0;
    if (g_pairs == 2) return g_pair_planes;
    if (cells < (1LL << 22)) return 0;
    const long long tiles = (long long)((F.n0 + C2_TX - 1) / C2_TX) * ((F.n1 + C2_TY - 1) / C2_TY);
    for (int planes = g_pair_planes; planes >= 8; planes /= 2)
        if (tiles * ((F.n2 + planes - 1) / planes) >= 2LL * C2_BLOCKS_PER_SM * 152) return planes;
    return 0;
}

template <typename T>
bool use_pairs(const MgLevel<T> &F)
{
    return pair_planes(F) > 0;
}

cudaError_t pair_smem_attr()
{
    static const cudaError_t rc = [] {
        cudaError_t e = cudaSuccess;
        const void *fns[5] = {(const void *)k_cheb_pair<false, false, false>,
                              (const void *)k_cheb_pair<false, true, false>, (const void *)k_cheb_pair<true, false, false>,
                              (const void *)k_cheb_pair<true, true, false>, (const void *)k_cheb_pair<true, false, true>};
        for (const void *f : fns) {
            const cudaError_t r = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C2_SMEM);
            if (r != cudaSuccess) e = r;
        }
        return e;
    }();
    return rc;
}

// Two Chebyshev steps (c1a, c2a) then (c1b, c2b) of FP32 level F from xin
// into xout; dprev nullptr means the first step's previous update is xin
// itself.  Callers check use_pairs(F) first.  Should a tensor map still not
// encode, the two steps run as one-step launches (xin is then overwritten,
// as the callers allow: it is their scratch buffer after the pair).
cudaError_t cheb_pair(const MgLevel<float> &F, const float *xin, const float *dprev, float *xout, float *dout,
                      double c1a, double c2a, double c1b, double c2b, cudaStream_t st)
{
    PairArgs a;
    a.F = F.view();
    a.xout = xout; a.dout = dout; a.flags = F.flags;
    a.c1a = (float)c1a; a.c2a = (float)c2a; a.c1b = (float)c1b; a.c2b = (float)c2b;
    a.planes = pair_planes(F) > 0 ? pair_planes(F) : g_pair_planes;
    PairMaps tm;
    const LevelView<float> v = a.F;
    bool ok = F.flags != nullptr && encode_pair_map(&tm.m[0], F.b, v, C2_WA, C2_HA) &&
              encode_pair_map(&tm.m[1], F.diag, v, C2_WA, C2_HA) && encode_pair_map(&tm.m[2], F.cT, v, C2_WA, C2_HA) &&
              (!dprev || encode_pair_map(&tm.m[3], dprev, v, C2_WA, C2_HA)) &&
              encode_pair_map(&tm.m[4], F.cE, v, C2_WE, C2_HA) && encode_pair_map(&tm.m[5], F.cN, v, C2_WA, C2_HN) &&
              encode_pair_map(&tm.m[6], xin, v, C2_WE, C2_HX);
    if (!dprev) tm.m[3] = tm.m[6];   // not read
    if (ok) ok = pair_smem_attr() == cudaSuccess;
    if (!ok) {
        g_pair_fallback.fetch_add(1);
        Launch3 lf = launch_interior(F.n0, F.n1, F.n2);
        float *x1 = xout, *x2 = const_cast<float *>(xin);
        k_cheb_step<float><<<lf.grid, lf.block, 0, st>>>(v, F.b, xin, dprev ? dprev : xin, x1, F.d, (float)c1a,
                                                         (float)c2a);
        k_cheb_step<float><<<lf.grid, lf.block, 0, st>>>(v, F.b, x1, F.d, x2, dout, (float)c1b, (float)c2b);
        return cudaMemcpyAsync(xout, x2, sizeof(float) * (size_t)F.tot, cudaMemcpyDeviceToDevice, st);
    }
    g_pair_tma.fetch_add(1);
    const dim3 blk(C2_TX, C2_TY, 1);
    const dim3 grd((F.n0 + C2_TX - 1) / C2_TX, (F.n1 + C2_TY - 1) / C2_TY, (F.n2 + a.planes - 1) / a.planes);
    if (dprev && dout) k_cheb_pair<true, true, false><<<grd, blk, C2_SMEM, st>>>(tm, a);
    else if (dprev) k_cheb_pair<true, false, false><<<grd, blk, C2_SMEM, st>>>(tm, a);
    else if (dout) k_cheb_pair<false, true, false><<<grd, blk, C2_SMEM, st>>>(tm, a);
    else k_cheb_pair<false, false, false><<<grd, blk, C2_SMEM, st>>>(tm, a);
    return cudaSuccess;
}

// The last pre-smoothing step fused with the restriction: one Chebyshev
// step (c1, c2) of FP32 level F from xin with the previous update F.d into
// xout, and the residual of the result restricted to C.b, with the bits of
// a k_cheb_step launch followed by k_restrict.  Needs coarsening factors 2
// and a level that takes the two-step kernel; returns false (launching
// nothing) otherwise.
bool cheb_restrict(const MgLevel<float> &F, const MgLevel<float> &C, const float *xin, float *xout, double c1,
                   double c2, float *xc, double first, cudaStream_t st)
{
    if (F.f0 != 2 || F.f1 != 2 || F.f2 != 2 || !use_pairs(F) || !F.flags) return false;
    PairArgs a;
    a.F = F.view();
    a.xout = xout; a.dout = nullptr; a.flags = F.flags;
    a.c1a = (float)c1; a.c2a = (float)c2; a.c1b = 0.f; a.c2b = 0.f;
    const int planes = pair_planes(F);
    a.planes = planes + (planes & 1);     // whole plane pairs per block
    a.C = C.view(); a.bc = C.b;
    a.xc = xc; a.firstc = (float)first;
    PairMaps tm;
    const LevelView<float> v = a.F;
    const bool ok = encode_pair_map(&tm.m[0], F.b, v, C2_WA, C2_HA) && encode_pair_map(&tm.m[1], F.diag, v, C2_WA, C2_HA) &&
                    encode_pair_map(&tm.m[2], F.cT, v, C2_WA, C2_HA) && encode_pair_map(&tm.m[3], F.d, v, C2_WA, C2_HA) &&
                    encode_pair_map(&tm.m[4], F.cE, v, C2_WE, C2_HA) && encode_pair_map(&tm.m[5], F.cN, v, C2_WA, C2_HN) &&
                    encode_pair_map(&tm.m[6], xin, v, C2_WE, C2_HX) && pair_smem_attr() == cudaSuccess;
    if (!ok) return false;
    g_pair_tma.fetch_add(1);
    const dim3 blk(C2_TX, C2_TY, 1);
    const dim3 grd((F.n0 + C2_TX - 1) / C2_TX, (F.n1 + C2_TY - 1) / C2_TY, (F.n2 + a.planes - 1) / a.planes);
    k_cheb_pair<true, false, true><<<grd, blk, C2_SMEM, st>>>(tm, a);
    return true;
}

// Chebyshev step with z-line Jacobi blocks: the preconditioner of the
// Chebyshev iteration is T^-1, T the block diagonal of A whose blocks are
// segments of LINE_SEG cells along k of one (i, j) column (the diagonal and
// the k-couplings inside the segment).  One thread owns one segment: it forms
// the residual cell by cell (k-neighbours in registers), eliminates forward
// (Thomas algorithm, pivots formed on the fly) and substitutes backward in
// registers, so the step moves the same arrays as the point step:
//   x <- x + (c1 d + c2 T^-1 (b - A x)).
// zero_guess: x = 0 on entry (the first pre-smoothing step); x and dprev are
// not read.  T is a diagonally dominant M-matrix block, so its eigenvalue
// bound for the Chebyshev interval is that of the point diagonal.
template <typename T>
__device__ __forceinline__ T rcp_of(T v);
template <>
__device__ __forceinline__ float rcp_of<float>(float v) { return __frcp_rn(v); }
template <>
__device__ __forceinline__ double rcp_of<double>(double v) { return 1.0 / v; }

template <typename T>
__global__ void __launch_bounds__(128) k_cheb_line(LevelView<T> L, const T *__restrict__ b, const T *x,
                                                   const T *dprev, T *__restrict__ xout, T *__restrict__ dout, T c1,
                                                   T c2, int zero_guess)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k0 = blockIdx.z * LINE_SEG + 1;
    if (i > L.n0 || j > L.n1) return;
    const int nk = min(LINE_SEG, L.n2 - k0 + 1);
    const int sy = L.sy, sz = L.sz;
    int c = i + sy * j + sz * k0;
    T y[LINE_SEG], cp[LINE_SEG], xo[LINE_SEG];
    T xm = zero_guess ? T(0) : x[c - sz];
    T xc = zero_guess ? T(0) : x[c];
    T ym = T(0), cpm = T(0);
#pragma unroll
    for (int s = 0; s < LINE_SEG; ++s) {
        y[s] = T(0); cp[s] = T(0); xo[s] = T(0);
        if (s < nk) {
            const T dg = L.diag[c];
            const T ct = L.cT[c], cb = L.cT[c - sz];
            T r;
            T xp = T(0);
            if (zero_guess) {
                r = b[c];
            } else {
                xp = x[c + sz];
                r = b[c] - (dg * xc - (L.cE[c] * x[c + 1] + L.cE[c - 1] * x[c - 1] + L.cN[c] * x[c + sy] +
                                       L.cN[c - sy] * x[c - sy] + ct * xp + cb * xm));
            }
            if (dg > T(0)) {
                const T a = s > 0 ? -cb : T(0);
                const T cc = s < nk - 1 ? -ct : T(0);
                const T inv = rcp_of<T>(dg - a * cpm);
                cp[s] = cc * inv;
                y[s] = (r - a * ym) * inv;
            }
            ym = y[s];
            cpm = cp[s];
            xo[s] = xc;
            xm = xc;
            xc = xp;
            c += sz;
        }
    }
    T zn = T(0);
#pragma unroll
    for (int s = LINE_SEG - 1; s >= 0; --s) {
        if (s < nk) {
            c -= sz;
            const T z = y[s] - cp[s] * zn;
            zn = z;
            const T dp = zero_guess ? T(0) : dprev[c];
            const T dn = c1 * dp + c2 * z;
            xout[c] = xo[s] + dn;
            if (dout) dout[c] = dn;
        }
    }
}

template <typename T>
void launch_cheb_line(const MgLevel<T> &F, const T *x, const T *dprev, T *xout, T *dout, double c1, double c2,
                      bool zero_guess, cudaStream_t st)
{
    dim3 blk(32, 4, 1);
    dim3 grd((F.n0 + 31) / 32, (F.n1 + 3) / 4, (F.n2 + LINE_SEG - 1) / LINE_SEG);
    k_cheb_line<T><<<grd, blk, 0, st>>>(F.view(), F.b, x, dprev, xout, dout, (T)c1, (T)c2, zero_guess ? 1 : 0);
}

// Residual of the fine level summed over each coarse cell's children (and,
// with xc given, the coarse level's first smoothing step x = D^-1 b / theta
// from that sum, which saves a launch per level and V-cycle).  One
// thread per fine i and coarse (J,K): it sums the residuals of its (up to
// 2x2) fine cells in j and k (j outer, k inner, from 0), then lanes i and
// i^1 add their sums with a shuffle (always in the order even + odd), so the
// result is reproducible; the fused smoothing step and restriction of the
// two-step kernel forms the same sums in the same order.
template <typename T>
__global__ void __launch_bounds__(128) k_restrict(LevelView<T> F, const T *__restrict__ b,
                                                  const T *__restrict__ x, LevelView<T> C, T *__restrict__ bc,
                                                  int f0, int f1, int f2, T *__restrict__ xc, T first)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int K = blockIdx.z + 1;
    const bool in = i <= F.n0 && J <= C.n1;
    T s = T(0);
    if (in) {
        const int j0 = (J - 1) * f1 + 1, j1 = min(j0 + f1 - 1, F.n1);
        const int k0 = (K - 1) * f2 + 1, k1 = min(k0 + f2 - 1, F.n2);
        for (int jj = j0; jj <= j1; ++jj)
            for (int kk = k0; kk <= k1; ++kk) {
                const int fc = i + F.sy * jj + F.sz * kk;
                const T r = cheb_residual(b[fc], F.diag[fc], x[fc], x[fc + 1], x[fc - 1], x[fc + F.sy],
                                          x[fc - F.sy], x[fc + F.sz], x[fc - F.sz], F.cE[fc], F.cE[fc - 1],
                                          F.cN[fc], F.cN[fc - F.sy], F.cT[fc], F.cT[fc - F.sz]);
                s = fx_add(s, r);
            }
    }
    if (f0 == 2) {
        const T o = __shfl_xor_sync(0xffffffffu, s, 1);
        if ((threadIdx.x & 1) == 0) s = fx_add(s, o);
        else return;
    }
    if (!in) return;
    const int I = f0 == 2 ? ((i - 1) >> 1) + 1 : i;
    const int cc = I + C.sy * J + C.sz * K;
    bc[cc] = s;
    // the coarse level's first Chebyshev step from a zero guess, as
    // k_cheb_first forms it (same operands, same order)
    if (xc) xc[cc] = first * dinv_at(C, cc) * s;
}

// prolongation (piecewise constant, active cells only) fused with the first
// post-smoothing Chebyshev step
template <typename T>
__global__ void __launch_bounds__(256) k_post_first(LevelView<T> F, const T *__restrict__ b,
                                                    const T *__restrict__ x, LevelView<T> C,
                                                    const T *__restrict__ e, T *__restrict__ xout,
                                                    T *__restrict__ dout, int f0, int f1, int f2, T coef)
{
    INTERIOR_IJK(F);
    if (!in) return;
    const int s0 = f0 - 1, s1 = f1 - 1, s2 = f2 - 1;   // factors are 1 or 2
    auto xc = [&](int ii, int jj, int kk) -> T {
        const int fc = ii + F.sy * jj + F.sz * kk;
        T v = x[fc];
        if (active_at(F, fc)) {
            const int I = ((ii - 1) >> s0) + 1, J = ((jj - 1) >> s1) + 1, K = ((kk - 1) >> s2) + 1;
            v += e[I + C.sy * J + C.sz * K];
        }
        return v;
    };
    const T x0 = xc(i, j, k);
    const T ax = F.diag[c] * x0 - (F.cE[c] * xc(i + 1, j, k) + F.cE[c - 1] * xc(i - 1, j, k) +
                                   F.cN[c] * xc(i, j + 1, k) + F.cN[c - F.sy] * xc(i, j - 1, k) +
                                   F.cT[c] * xc(i, j, k + 1) + F.cT[c - F.sz] * xc(i, j, k - 1));
    const T dn = coef * dinv_at(F, c) * (b[c] - ax);
    xout[c] = x0 + dn;
    if (dout) dout[c] = dn;
}

// x += e(parent) on the active cells (piecewise-constant prolongation of
// the coarse correction, in place); on large levels this and a plain first
// Chebyshev step replace k_post_first, whose seven recomputed neighbour
// prolongations cost more than one extra pass over x.  A thread owns
// PR_KZ cells of one (i, j) column and issues all their loads (mask, x and
// the parent's correction) before any store, so they are in flight
// together (one cell per thread, the load of x waiting on the mask, ran at
// a third of the HBM bandwidth).
constexpr int PR_KZ = 4;
template <typename T>
__global__ void __launch_bounds__(256) k_prolong(LevelView<T> F, const unsigned char *__restrict__ act,
                                                 T *__restrict__ x, LevelView<T> C, const T *__restrict__ e, int s0,
                                                 int s1, int s2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int kb = blockIdx.z * PR_KZ + 1;
    if (i > F.n0 || j > F.n1) return;
    const int c0 = i + F.sy * j;
    const int pc = (((i - 1) >> s0) + 1) + C.sy * (((j - 1) >> s1) + 1);
    unsigned char a[PR_KZ];
    T xv[PR_KZ], ev[PR_KZ];
#pragma unroll
    for (int m = 0; m < PR_KZ; ++m) {
        const int k = kb + m;
        a[m] = 0;
        if (k <= F.n2) {
            const int c = c0 + F.sz * k;
            a[m] = act[c];
            xv[m] = x[c];
            ev[m] = e[pc + C.sz * (((k - 1) >> s2) + 1)];
        }
    }
#pragma unroll
    for (int m = 0; m < PR_KZ; ++m)
        if (a[m]) x[c0 + F.sz * (kb + m)] = xv[m] + ev[m];
}

template <typename T>
void launch_prolong(const MgLevel<T> &F, const MgLevel<T> &C, T *x, const T *e, cudaStream_t st)
{
    const dim3 blk(32, 8, 1);
    const dim3 grd((F.n0 + 31) / 32, (F.n1 + 7) / 8, (F.n2 + PR_KZ - 1) / PR_KZ);
    k_prolong<T><<<grd, blk, 0, st>>>(F.view(), F.active, x, C.view(), e, F.f0 - 1, F.f1 - 1, F.f2 - 1);
}

// coarsest level: y = Ainv (b - mean) on the active cells (one block)
template <typename T>
__global__ void __launch_bounds__(128) k_coarse_solve(const T *__restrict__ b, T *__restrict__ x,
                                                      const unsigned char *__restrict__ act,
                                                      const double *__restrict__ ainv, const int *__restrict__ map,
                                                      int n, int singular)
{
    __shared__ double sb[128];
    __shared__ double red[2];
    const int t = threadIdx.x;
    double bv = 0.0, a = 0.0;
    if (t < n) {
        bv = (double)b[map[t]];
        a = act[map[t]] ? 1.0 : 0.0;
    }
    if (singular) {
        double s = block_sum(bv * a);
        __syncthreads();
        double cnt = block_sum(a);
        if (t == 0) { red[0] = s; red[1] = cnt; }
        __syncthreads();
        if (red[1] > 0.0) bv -= a * (red[0] / red[1]);
    }
    if (t < n) sb[t] = bv;
    __syncthreads();
    if (t < n) {
        double y = 0.0;
        for (int s = 0; s < n; ++s) y += ainv[(size_t)t * n + s] * sb[s];
        x[map[t]] = a != 0.0 ? (T)y : T(0);
    }
}

// ---------------------------------------------------------------------------
// hierarchy construction

template <typename T>
__global__ void __launch_bounds__(256) k_coarsen_cpl(MgLevel<T> F, MgLevel<T> C)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
    if (i > C.n0 || j > C.n1 || k > C.n2) return;
    const int cc = i + C.sy * j + C.sz * k;
    const int f0 = F.f0, f1 = F.f1, f2 = F.f2;
    const int i0 = (i - 1) * f0 + 1, j0 = (j - 1) * f1 + 1, k0 = (k - 1) * f2 + 1;
    const int i1 = min(i0 + f0 - 1, F.n0), j1 = min(j0 + f1 - 1, F.n1), k1 = min(k0 + f2 - 1, F.n2);
    unsigned char act = 0;
    T ex = T(0), se = T(0), sn = T(0), sT = T(0);
    for (int kk = k0; kk <= k1; ++kk)
        for (int jj = j0; jj <= j1; ++jj)
            for (int ii = i0; ii <= i1; ++ii) {
                const int fc = ii + F.sy * jj + F.sz * kk;
                act |= F.active[fc];
                ex += F.extra[fc];
                if (ii == i1) se += F.cE[fc];
                if (jj == j1) sn += F.cN[fc];
                if (kk == k1) sT += F.cT[fc];
            }
    C.active[cc] = act;
    C.extra[cc] = T(0.5) * ex;
    C.cE[cc] = i < C.n0 ? se / T(f0) : T(0);
    C.cN[cc] = j < C.n1 ? sn / T(f1) : T(0);
    C.cT[cc] = k < C.n2 ? sT / T(f2) : T(0);
}

template <typename T>
__global__ void __launch_bounds__(256) k_coarsen_diag(MgLevel<T> C)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
    if (i > C.n0 || j > C.n1 || k > C.n2) return;
    const int c = i + C.sy * j + C.sz * k;
    if (!C.active[c]) {
        C.diag[c] = T(-1);
        C.dinv[c] = T(0);
        return;
    }
    const T dg = C.cE[c] + C.cE[c - 1] + C.cN[c] + C.cN[c - C.sy] + C.cT[c] + C.cT[c - C.sz] + C.extra[c];
    C.diag[c] = dg;
    C.dinv[c] = dg > T(0) ? T(1) / dg : T(0);
}

template <typename T>
void mg_coarsen(const MgLevel<T> &F, MgLevel<T> &C, cudaStream_t st, int *launches)
{
    Launch3 l = launch_interior(C.n0, C.n1, C.n2);
    k_coarsen_cpl<T><<<l.grid, l.block, 0, st>>>(F, C);
    k_coarsen_diag<T><<<l.grid, l.block, 0, st>>>(C);
    *launches += 2;
}

// Dense inverse of the coarsest operator by in-place Gauss-Jordan (SPD, no
// pivoting); all-Neumann systems get the rank-one term s*1*1^T on the active
// cells so that the inverse maps zero-mean vectors to the zero-mean solution.
template <typename T>
__global__ void __launch_bounds__(256) k_coarse_inverse(MgLevel<T> L, double *__restrict__ Aout,
                                                        const int *__restrict__ map, int n, int singular)
{
    extern __shared__ double A[];      // n*n, in shared memory
    __shared__ double fcol[128];
    __shared__ double red[2];
    __shared__ int smap[128];
    const int t = threadIdx.x;
    const int nt = blockDim.x;
    for (int e = t; e < n * n; e += nt) A[e] = 0.0;
    for (int a = t; a < n; a += nt) smap[a] = map[a];
    __syncthreads();
    double dsum = 0.0, cnt = 0.0;
    for (int a = t; a < n; a += nt) {
        const int c = smap[a];
        A[a * n + a] = (double)L.diag[c];
        if (L.active[c]) { dsum += (double)L.diag[c]; cnt += 1.0; }
        const int nb[6] = {c + 1, c - 1, c + L.sy, c - L.sy, c + L.sz, c - L.sz};
        const T w[6] = {L.cE[c], L.cE[c - 1], L.cN[c], L.cN[c - L.sy], L.cT[c], L.cT[c - L.sz]};
        for (int q = 0; q < 6; ++q) {
            if (w[q] == T(0)) continue;
            for (int b = 0; b < n; ++b)
                if (smap[b] == nb[q]) { A[a * n + b] -= (double)w[q]; break; }
        }
    }
    dsum = block_sum(dsum);
    __syncthreads();
    cnt = block_sum(cnt);
    if (t == 0) { red[0] = dsum; red[1] = cnt; }
    __syncthreads();
    if (singular && red[1] > 0.0) {
        const double s = red[0] / red[1] / red[1];
        for (int e = t; e < n * n; e += nt) {
            const int a = e / n, b = e % n;
            if (L.active[smap[a]] && L.active[smap[b]]) A[e] += s;
        }
    }
    __syncthreads();
    for (int kk = 0; kk < n; ++kk) {
        const double piv = A[kk * n + kk];
        const double pinv = piv > 0.0 ? 1.0 / piv : 0.0;
        __syncthreads();
        for (int a = t; a < n; a += nt) fcol[a] = A[a * n + kk];
        __syncthreads();
        for (int b = t; b < n; b += nt) A[kk * n + b] = (b == kk) ? pinv : A[kk * n + b] * pinv;
        __syncthreads();
        for (int e = t; e < n * n; e += nt) {
            const int a = e / n, b = e % n;
            if (a == kk) continue;
            if (b == kk)
                A[e] = -fcol[a] * pinv;
            else
                A[e] -= fcol[a] * A[kk * n + b];
        }
        __syncthreads();
    }
    for (int e = t; e < n * n; e += nt) Aout[e] = A[e];
}

template <typename T>
void mg_coarse_inverse(const MgLevel<T> &L, double *ainv, int *map, int n, bool singular, cudaStream_t st,
                       int *launches)
{
    const size_t smem = (size_t)n * n * sizeof(double);
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_coarse_inverse<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 128 * 128 * 8);
        attr_set = true;
    }
    k_coarse_inverse<T><<<1, 256, smem, st>>>(L, ainv, map, n, singular ? 1 : 0);
    *launches += 1;
}

// Algorithmic bytes of one Chebyshev step on level F: b, x, diag, cE, cN,
// cT (+ the stored inverse diagonal on FP64 levels) and the previous update
// (absent in the first step, where it is x) read; x and, except in the last
// step, the update written.
template <typename T>
double smooth_bytes(const MgLevel<T> &F, bool first, bool writes_d)
{
    const double cells = (double)F.n0 * F.n1 * F.n2;
    const int arrays = 6 + (sizeof(T) == 8 ? 1 : 0) + (first ? 0 : 1) + 1 + (writes_d ? 1 : 0);
    return arrays * sizeof(T) * cells;
}

// Algorithmic bytes of the first (zero-guess) line step: b, diag, cT read,
// x written.
template <typename T>
double line_first_bytes(const MgLevel<T> &F)
{
    return 4.0 * sizeof(T) * (double)F.n0 * F.n1 * F.n2;
}

// Algorithmic bytes of the split prolongation + first post-smoothing step:
// x read and written, the active mask and the coarse correction read; then
// b, x, diag, cE, cN, cT (+ dinv on FP64 levels) read, x (+ the update)
// written.
template <typename T>
double prolong_bytes(const MgLevel<T> &F, bool writes_d)
{
    const double cells = (double)F.n0 * F.n1 * F.n2;
    const double s = sizeof(T);
    return cells * (2.0 * s + 1.0 + s / 8.0 + (6 + (sizeof(T) == 8 ? 1 : 0) + 1 + (writes_d ? 1 : 0)) * s);
}

// Algorithmic bytes of a fused pair of steps: b, diag, cE, cN, cT and x
// read (+ the previous update), x (+ the update) written; with the
// prolongation before it, x read and written once more, the active mask and
// the coarse correction read.
double pair_bytes(const MgLevel<float> &F, bool reads_d, bool writes_d, bool prolong)
{
    const double cells = (double)F.n0 * F.n1 * F.n2;
    return cells * (4.0 * (7 + (reads_d ? 1 : 0) + (writes_d ? 1 : 0)) + (prolong ? 8.0 + 1.0 + 4.0 / 8.0 : 0.0));
}

// Algorithmic bytes of the fused last step and restriction: b, x, the
// previous update, diag, cE, cN, cT read, x written, the coarse rhs written.
double restrict_fused_bytes(const MgLevel<float> &F)
{
    const double cells = (double)F.n0 * F.n1 * F.n2;
    return cells * (4.0 * 8 + 4.0 / 8.0);
}
template <typename T>
double restrict_fused_bytes(const MgLevel<T> &)
{
    return -1.0;
}

template <typename T>
T *mg_vcycle(MgLevel<T> *L, int nlev, const ChebCoef &cc, const double *ainv, const int *map, int ncoarse,
             bool singular, bool first_done, cudaStream_t st, int *launches, KTimer *kt, cudaEvent_t coarse_ready)
{
    T *cur[32];
    bool first_written[32] = {};    // level l's first step already written by the restriction into it
    const int last = nlev - 1;
    for (int l = 0; l < last; ++l) {
        MgLevel<T> &F = L[l];
        LevelView<T> v = F.view();
        Launch3 lf = launch_interior(F.n0, F.n1, F.n2);
        T *xa = F.x, *xb = F.xb;
        if (cc.lines) {
            const int id0 = l == 0 ? kt_begin(kt, KC_SMOOTH, st, line_first_bytes<T>(F)) : -1;
            launch_cheb_line<T>(F, nullptr, nullptr, xa, nullptr, 0.0, cc.first, true, st);
            kt_end(kt, id0, st);
            *launches += 1;
            for (int s = 1; s < cc.degree; ++s) {
                const T *dprev = (s == 1) ? xa : F.d;
                T *dout = (s == cc.degree - 1) ? nullptr : F.d;
                const int id = l == 0 ? kt_begin(kt, KC_SMOOTH, st, smooth_bytes<T>(F, s == 1, dout != nullptr)) : -1;
                launch_cheb_line<T>(F, xa, dprev, xb, dout, cc.c1[s], cc.c2[s], false, st);
                kt_end(kt, id, st);
                *launches += 1;
                T *tmp = xa; xa = xb; xb = tmp;
            }
            cur[l] = xa;
            MgLevel<T> &C = L[l + 1];
            dim3 rg((F.n0 + 31) / 32, (C.n1 + 3) / 4, C.n2), rb(32, 4, 1);
            const int id = l == 0 ? kt_begin(kt, KC_RESTRICT, st) : -1;
            k_restrict<T><<<rg, rb, 0, st>>>(v, F.b, xa, C.view(), C.b, F.f0, F.f1, F.f2, nullptr, T(0));
            kt_end(kt, id, st);
            *launches += 1;
            continue;
        }
        if (!(l == 0 ? first_done : first_written[l])) {
            k_cheb_first<T><<<lf.grid, lf.block, 0, st>>>(v, F.b, xa, (T)cc.first);
            *launches += 1;
        }
        int s = 1;
        if constexpr (sizeof(T) == 4) {
            // steps 1 and 2 in one pass (step 1's previous update is x
            // itself), and steps 3 and 4 too when they are the last two
            const int m = cc.degree - 1;
            if (use_pairs(F) && m >= 2) {
                T *dout = m > 2 ? F.d : nullptr;
                const int id = l == 0 ? kt_begin(kt, KC_SMOOTH2, st, pair_bytes(F, false, dout != nullptr, false)) : -1;
                cheb_pair(F, xa, nullptr, xb, dout, cc.c1[1], cc.c2[1], cc.c1[2], cc.c2[2], st);
                kt_end(kt, id, st);
                *launches += 1;
                { T *tmp = xa; xa = xb; xb = tmp; }
                s = 3;
                if (m == 4) {
                    const int id2 = l == 0 ? kt_begin(kt, KC_SMOOTH2, st, pair_bytes(F, true, false, false)) : -1;
                    cheb_pair(F, xa, F.d, xb, nullptr, cc.c1[3], cc.c2[3], cc.c1[4], cc.c2[4], st);
                    kt_end(kt, id2, st);
                    *launches += 1;
                    { T *tmp = xa; xa = xb; xb = tmp; }
                    s = 5;
                }
            }
        }
        if constexpr (sizeof(T) == 4) {
            // a single last step before the restriction: both in one pass
            if (s == cc.degree - 1 && s >= 3 && F.f0 == 2 && F.f1 == 2 && F.f2 == 2 && use_pairs(F)) {
                const int id = l == 0 ? kt_begin(kt, KC_RESTRICT, st, restrict_fused_bytes(F)) : -1;
                const bool wx = l + 1 < last;
                const bool fused = cheb_restrict(F, L[l + 1], xa, xb, cc.c1[s], cc.c2[s], wx ? L[l + 1].x : nullptr,
                                                 cc.first, st);
                kt_end(kt, id, st);
                if (fused) {
                    *launches += 1;
                    cur[l] = xb;
                    first_written[l + 1] = wx;
                    continue;
                }
            }
        }
        for (; s < cc.degree; ++s) {
            // the first step's previous update is x itself (zero guess); the
            // last step's update is not needed by anything that follows
            const T *dprev = (s == 1) ? xa : F.d;
            T *dout = (s == cc.degree - 1) ? nullptr : F.d;
            const int id = l == 0 ? kt_begin(kt, KC_SMOOTH, st, smooth_bytes<T>(F, s == 1, dout != nullptr)) : -1;
            k_cheb_step<T><<<lf.grid, lf.block, 0, st>>>(v, F.b, xa, dprev, xb, dout, (T)cc.c1[s], (T)cc.c2[s]);
            kt_end(kt, id, st);
            *launches += 1;
            T *tmp = xa; xa = xb; xb = tmp;
        }
        cur[l] = xa;
        MgLevel<T> &C = L[l + 1];
        dim3 rg((F.n0 + 31) / 32, (C.n1 + 3) / 4, C.n2), rb(32, 4, 1);
        const int id = l == 0 ? kt_begin(kt, KC_RESTRICT, st) : -1;
        const bool wx = l + 1 < last;
        k_restrict<T><<<rg, rb, 0, st>>>(v, F.b, xa, C.view(), C.b, F.f0, F.f1, F.f2, wx ? C.x : nullptr,
                                         (T)cc.first);
        first_written[l + 1] = wx;
        kt_end(kt, id, st);
        *launches += 1;
    }
    {
        MgLevel<T> &Cst = L[last];
        if (coarse_ready) cudaStreamWaitEvent(st, coarse_ready, 0);
        k_coarse_solve<T><<<1, 128, 0, st>>>(Cst.b, Cst.x, Cst.active, ainv, map, ncoarse, singular ? 1 : 0);
        *launches += 1;
        cur[last] = Cst.x;
    }
    for (int l = last - 1; l >= 0; --l) {
        MgLevel<T> &F = L[l];
        MgLevel<T> &C = L[l + 1];
        LevelView<T> v = F.view();
        Launch3 lf = launch_interior(F.n0, F.n1, F.n2);
        T *xa = cur[l];
        T *xb = (xa == F.x) ? F.xb : F.x;
        const bool more = cc.degree > 1;
        if (cc.lines) {
            const int idp = l == 0 ? kt_begin(kt, KC_PROLONG, st, prolong_bytes<T>(F, more)) : -1;
            launch_prolong<T>(F, C, xa, cur[l + 1], st);
            launch_cheb_line<T>(F, xa, xa, xb, more ? F.d : nullptr, 0.0, cc.first, false, st);
            kt_end(kt, idp, st);
            *launches += 2;
            { T *tmp = xa; xa = xb; xb = tmp; }
            for (int s = 1; s < cc.degree; ++s) {
                const bool last_step = s == cc.degree - 1;
                const int id = l == 0 ? kt_begin(kt, KC_SMOOTH, st, smooth_bytes<T>(F, false, !last_step)) : -1;
                launch_cheb_line<T>(F, xa, F.d, xb, last_step ? nullptr : F.d, cc.c1[s], cc.c2[s], false, st);
                kt_end(kt, id, st);
                *launches += 1;
                T *tmp = xa; xa = xb; xb = tmp;
            }
            cur[l] = xa;
            continue;
        }
        int s = 1;
        bool paired = false;
        if constexpr (sizeof(T) == 4) {
            // prolongation (in place), then the first post-smoothing step
            // (its previous update term is 0) and step 1 in one pass; steps
            // 2 and 3 too when they are the last two
            const int m = cc.degree - 1;
            if (use_pairs(F) && m >= 1) {
                T *dout = m >= 2 ? F.d : nullptr;
                const int idp = l == 0 ? kt_begin(kt, KC_PROLONG, st, pair_bytes(F, false, dout != nullptr, true)) : -1;
                launch_prolong<T>(F, C, xa, cur[l + 1], st);
                cheb_pair(F, xa, nullptr, xb, dout, 0.0, cc.first, cc.c1[1], cc.c2[1], st);
                kt_end(kt, idp, st);
                *launches += 2;
                { T *tmp = xa; xa = xb; xb = tmp; }
                s = 2;
                if (m == 3) {
                    const int id2 = l == 0 ? kt_begin(kt, KC_SMOOTH2, st, pair_bytes(F, true, false, false)) : -1;
                    cheb_pair(F, xa, F.d, xb, nullptr, cc.c1[2], cc.c2[2], cc.c1[3], cc.c2[3], st);
                    kt_end(kt, id2, st);
                    *launches += 1;
                    { T *tmp = xa; xa = xb; xb = tmp; }
                    s = 4;
                }
                paired = true;
            }
        }
        if (paired) {
        } else if ((long long)F.n0 * F.n1 * F.n2 >= (1LL << 18)) {
            const int idp = l == 0 ? kt_begin(kt, KC_PROLONG, st, prolong_bytes<T>(F, more)) : -1;
            launch_prolong<T>(F, C, xa, cur[l + 1], st);
            // first post-smoothing step from x: the previous update term is 0
            k_cheb_step<T><<<lf.grid, lf.block, 0, st>>>(v, F.b, xa, xa, xb, more ? F.d : nullptr, T(0),
                                                         (T)cc.first);
            kt_end(kt, idp, st);
            *launches += 2;
        } else {
            const int idp = l == 0 ? kt_begin(kt, KC_PROLONG, st) : -1;
            k_post_first<T><<<lf.grid, lf.block, 0, st>>>(v, F.b, xa, C.view(), cur[l + 1], xb, more ? F.d : nullptr,
                                                          F.f0, F.f1, F.f2, (T)cc.first);
            kt_end(kt, idp, st);
            *launches += 1;
        }
        if (!paired) { T *tmp = xa; xa = xb; xb = tmp; }
        for (; s < cc.degree; ++s) {
            const bool last_step = s == cc.degree - 1;
            const int id = l == 0 ? kt_begin(kt, KC_SMOOTH, st, smooth_bytes<T>(F, false, !last_step)) : -1;
            k_cheb_step<T><<<lf.grid, lf.block, 0, st>>>(v, F.b, xa, F.d, xb, last_step ? nullptr : F.d,
                                                         (T)cc.c1[s], (T)cc.c2[s]);
            kt_end(kt, id, st);
            *launches += 1;
            T *tmp = xa; xa = xb; xb = tmp;
        }
        cur[l] = xa;
    }
    return cur[0];
}

// ---------------------------------------------------------------------------
// single launches for timing (scf_debug_time_kernel)
template <typename T>
void probe_smooth(MgLevel<T> &F, const ChebCoef &cc, cudaStream_t st)
{
    Launch3 lf = launch_interior(F.n0, F.n1, F.n2);
    const int s = cc.degree > 1 ? 1 : 0;
    k_cheb_step<T><<<lf.grid, lf.block, 0, st>>>(F.view(), F.b, F.x, F.d, F.xb, F.d, (T)cc.c1[s], (T)cc.c2[s]);
}

cudaError_t probe_smooth2(MgLevel<float> &F, const ChebCoef &cc, cudaStream_t st)
{
    return cheb_pair(F, F.x, F.d, F.xb, nullptr, cc.c1[1], cc.c2[1], cc.c1[2], cc.c2[2], st);
}

template <typename T>
void probe_restrict(MgLevel<T> &F, MgLevel<T> &C, cudaStream_t st)
{
    dim3 rg((F.n0 + 31) / 32, (C.n1 + 3) / 4, C.n2), rb(32, 4, 1);
    k_restrict<T><<<rg, rb, 0, st>>>(F.view(), F.b, F.x, C.view(), C.b, F.f0, F.f1, F.f2, nullptr, T(0));
}

template <typename T>
void probe_prolong(MgLevel<T> &F, MgLevel<T> &C, const ChebCoef &cc, cudaStream_t st)
{
    Launch3 lf = launch_interior(F.n0, F.n1, F.n2);
    k_post_first<T><<<lf.grid, lf.block, 0, st>>>(F.view(), F.b, F.x, C.view(), C.x, F.xb, F.d, F.f0, F.f1, F.f2,
                                                   (T)cc.first);
}

void probe_spmv(const LevelView<double> &A, const double *p, double *q, Reducer &R, cudaStream_t st)
{
    Launch3 l = launch_zchunk(A.n0, A.n1, A.n2);
    k_spmv_dot<<<l.grid, l.block, 0, st>>>(A, p, q, R.partials, R.max_blocks);
}

template void probe_smooth<float>(MgLevel<float> &, const ChebCoef &, cudaStream_t);
template void probe_smooth<double>(MgLevel<double> &, const ChebCoef &, cudaStream_t);
template void probe_restrict<float>(MgLevel<float> &, MgLevel<float> &, cudaStream_t);
template void probe_restrict<double>(MgLevel<double> &, MgLevel<double> &, cudaStream_t);
template void probe_prolong<float>(MgLevel<float> &, MgLevel<float> &, const ChebCoef &, cudaStream_t);
template void probe_prolong<double>(MgLevel<double> &, MgLevel<double> &, const ChebCoef &, cudaStream_t);

// explicit instantiations
template void mg_coarsen<float>(const MgLevel<float> &, MgLevel<float> &, cudaStream_t, int *);
template void mg_coarsen<double>(const MgLevel<double> &, MgLevel<double> &, cudaStream_t, int *);
template void mg_coarse_inverse<float>(const MgLevel<float> &, double *, int *, int, bool, cudaStream_t, int *);
template void mg_coarse_inverse<double>(const MgLevel<double> &, double *, int *, int, bool, cudaStream_t, int *);
template float *mg_vcycle<float>(MgLevel<float> *, int, const ChebCoef &, const double *, const int *, int, bool,
                                 bool, cudaStream_t, int *, KTimer *, cudaEvent_t);
template double *mg_vcycle<double>(MgLevel<double> *, int, const ChebCoef &, const double *, const int *, int, bool,
                                   bool, cudaStream_t, int *, KTimer *, cudaEvent_t);
template void cg_update<float>(const LevelView<double> &, double *, double *, const double *, const double *, float *,
                               const LevelView<float> &, float *, double, Reducer &, cudaStream_t, int *, KTimer *);
template void cg_update<double>(const LevelView<double> &, double *, double *, const double *, const double *,
                                double *, const LevelView<double> &, double *, double, Reducer &, cudaStream_t, int *,
                                KTimer *);
template void cg_dot_rz<float>(const LevelView<double> &, const double *, const float *, const float *, Reducer &,
                               cudaStream_t, int *);
template void cg_dot_rz<double>(const LevelView<double> &, const double *, const double *, const double *,
                                Reducer &, cudaStream_t, int *);
template void cg_pupdate<float>(const LevelView<double> &, const float *, double *, const double *, bool,
                                cudaStream_t, int *);
template void cg_pupdate<double>(const LevelView<double> &, const double *, double *, const double *, bool,
                                 cudaStream_t, int *);
