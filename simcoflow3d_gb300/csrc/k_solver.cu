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
#include <cuda_pipeline.h>

#include "scf_kernels.h"

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

template <typename T>
__device__ __forceinline__ T cheb_update(T b, T dg, T dinv, T x0, T xe, T xw, T xn, T xs, T xt, T xb, T ce, T cw,
                                         T cn, T cs, T ct, T cb, T dprev, T c1, T c2)
{
    T s = fx_mul(ce, xe);
    s = fx_fma(cw, xw, s);
    s = fx_fma(cn, xn, s);
    s = fx_fma(cs, xs, s);
    s = fx_fma(ct, xt, s);
    s = fx_fma(cb, xb, s);
    const T r = fx_sub(b, fx_fma(dg, x0, -s));
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
// Two Chebyshev steps in one pass over a large FP32 level (2.5-D temporal
// blocking).  A block owns a tile of 32 x 8 (i, j) columns and marches along
// k over `planes` planes.  For plane kk it
//   1. issues the asynchronous copies (cp.async) of plane kk + C2_AHEAD:
//      operator, right-hand side and previous update on the tile with a
//      one-cell halo, and x of the plane above it with a two-cell halo, into
//      rings in shared memory, so that C2_AHEAD planes are in flight while
//      plane kk is computed;
//   2. applies the first step on the 34 x 10 cells of plane kk (ghost cells
//      give 0, the value the one-step kernel leaves there) into a
//      three-plane ring in shared memory;
//   3. applies the second step on the 32 x 8 cells of plane kk - 1.
// Each array is read from DRAM about once per pass (halo columns come from
// L2), so two steps move about the bytes of one.  Both steps go through
// cheb_update: the result is that of two k_cheb_step launches, bit for bit.
// The output x must not be the input x, nor dout the previous update when
// both are given: neighbouring tiles read their halos from them.
constexpr int C2_TX = 32, C2_TY = 8, C2_THREADS = C2_TX * C2_TY;
// Tiles in shared memory, each starting on an even column (i0 - 1 or
// i0 - 3): with an even row length n0 + 2 every row starts 8-byte aligned,
// so each thread copies at most one pair of cells of each tile per plane.
constexpr int C2_EX = C2_TX + 2, C2_EY = C2_TY + 2, C2_NE = C2_EX * C2_EY;  // first-step cells, from (i0-1, j0-1)
constexpr int C2_WE = C2_TX + 4, C2_NCE = C2_WE * C2_EY;                 // cE from column i0 - 3
constexpr int C2_NCN = C2_EX * (C2_EY + 1);                              // cN from row j0 - 2
constexpr int C2_XX = C2_TX + 6, C2_XY = C2_TY + 4, C2_NX = C2_XX * C2_XY;  // x from (i0-3, j0-2)
constexpr int C2_NH = C2_NE - C2_THREADS;                                // halo cells of step 1
constexpr int C2_AHEAD = 1;                                              // planes copied ahead
// ring depths in planes: when plane kk + C2_AHEAD is issued, inputs of
// planes kk - 1 .. kk + C2_AHEAD - 1 and x of planes kk - 1 .. kk + C2_AHEAD
// are in use or on their way (the second step reads no inputs: the thread
// keeps its column's from the first step)
constexpr int C2_RD = C2_AHEAD + 2, C2_RX = C2_AHEAD + 3, C2_R1 = 3;
constexpr int C2_B = 0, C2_D = C2_NE, C2_P = 2 * C2_NE, C2_T = 3 * C2_NE, C2_E = 4 * C2_NE,
              C2_N = 4 * C2_NE + C2_NCE, C2_SLOT = 4 * C2_NE + C2_NCE + C2_NCN;
constexpr size_t C2_SMEM = sizeof(float) * (C2_RD * C2_SLOT + C2_RX * C2_NX + C2_R1 * C2_NE);
constexpr int C2_PLANES = 32;
static_assert(C2_NH <= C2_THREADS && C2_NE <= 2 * C2_THREADS && C2_NCE <= 2 * C2_THREADS &&
                  C2_NCN <= 2 * C2_THREADS && C2_NX <= 2 * C2_THREADS,
              "one pair of cells of each tile per thread");
static_assert(C2_EX % 2 == 0 && C2_WE % 2 == 0 && C2_XX % 2 == 0 && C2_SLOT % 2 == 0 && C2_NX % 2 == 0 &&
                  C2_D % 2 == 0 && C2_N % 2 == 0,
              "tile rows and ring slots of whole pairs");

struct PairArgs {
    LevelView<float> F;
    const float *b, *x;
    const float *dprev;          // nullptr: the first step's previous update is x itself
    float *xout, *dout;          // dout nullptr: the second step's update is not kept
    float c1a, c2a, c1b, c2b;
    int planes;
};

// In-plane offsets (i + sy j) of this thread's pair of cells of each tile
// and a bit per tile when the pair lies in the ghosted array: the same for
// every plane, so each copy is one add.
struct C2Offs {
    int e, ce, cn, x;
    unsigned ok;
};

// Pair p of a tile w cells wide starting at (i0 + di, j0 + dj) with n cells.
__device__ __forceinline__ void c2_off(const LevelView<float> &F, int p, int n, int w, int di, int dj, int i0,
                                       int j0, int *off, unsigned *ok, unsigned bit)
{
    const int wp = w / 2, qy = p / wp, qx = 2 * (p - qy * wp);
    const int i = i0 + di + qx, j = j0 + dj + qy;
    *off = i + F.sy * j;
    if (2 * p < n && i >= 0 && i + 1 <= F.n0 + 1 && (unsigned)j <= (unsigned)(F.n1 + 1)) *ok |= bit;
}

__device__ __forceinline__ C2Offs c2_offsets(const LevelView<float> &F, int i0, int j0, int tid)
{
    C2Offs o;
    o.ok = 0u;
    c2_off(F, tid, C2_NE, C2_EX, -1, -1, i0, j0, &o.e, &o.ok, 1u);
    c2_off(F, tid, C2_NCE, C2_WE, -3, -1, i0, j0, &o.ce, &o.ok, 2u);
    c2_off(F, tid, C2_NCN, C2_EX, -1, -2, i0, j0, &o.cn, &o.ok, 4u);
    c2_off(F, tid, C2_NX, C2_XX, -3, -2, i0, j0, &o.x, &o.ok, 8u);
    return o;
}

__device__ __forceinline__ void c2_cp(unsigned dst, const float *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst), "l"(src) : "memory");
}

// Copies of plane P's first-step inputs into the ring slot at shared
// address `slot` (planes 0..n2: plane 0 only for its cT) and of x of plane
// X into the x plane at shared address `xs` (planes 0..n2+1).  Pairs
// outside the ghosted array are not copied; no first step of an interior
// cell reads them.
template <bool DP>
__device__ __forceinline__ void c2_issue(const PairArgs &a, const C2Offs &o, unsigned slot, int P, unsigned xs, int X,
                                         int tid)
{
    const LevelView<float> &F = a.F;
    const unsigned q = 8u * tid;     // bytes
    if (P >= 0 && P <= F.n2) {
        const int base = F.sz * P;
        if (o.ok & 1u) {
            const int c = base + o.e;
            c2_cp(slot + 4u * C2_B + q, a.b + c);
            c2_cp(slot + 4u * C2_D + q, F.diag + c);
            if (DP) c2_cp(slot + 4u * C2_P + q, a.dprev + c);
            c2_cp(slot + 4u * C2_T + q, F.cT + c);
        }
        if (o.ok & 2u) c2_cp(slot + 4u * C2_E + q, F.cE + base + o.ce);
        if (o.ok & 4u) c2_cp(slot + 4u * C2_N + q, F.cN + base + o.cn);
    }
    if (X >= 0 && X <= F.n2 + 1 && (o.ok & 8u)) c2_cp(xs + q, a.x + F.sz * X + o.x);
}

struct C2Cell {
    float b, dg, dinv, ce, cw, cn, cs, ct, cb;
};

// First step at plane P on cell q = ex + 34 ey of the tile: the plane's
// inputs at offset dc (the plane below at dm) of the shared array S, x of
// planes P - 1, P, P + 1 at xm, x0, xp (qx: the cell in the x tile), x after
// the step written at o1; `in` whether the cell is interior.  Returns the
// update and the cell's inputs.
template <bool DP>
__device__ __forceinline__ float c2_first(const PairArgs &a, float *S, int dc, int dm, int xm, int x0, int xp, int o1,
                                          int q, int qe, int qn, int qx, bool in, C2Cell &k)
{
    if (!in) {
        S[o1 + q] = 0.f;
        return 0.f;
    }
    k.b = S[dc + C2_B + q];
    k.dg = S[dc + C2_D + q];
    k.dinv = jacobi_inv(k.dg);
    k.ce = S[dc + C2_E + qe + 2];
    k.cw = S[dc + C2_E + qe + 1];
    k.cn = S[dc + C2_N + qn + C2_EX];
    k.cs = S[dc + C2_N + qn];
    k.ct = S[dc + C2_T + q];
    k.cb = S[dm + C2_T + q];
    const float xc = S[x0 + qx];
    const float dn = cheb_update(k.b, k.dg, k.dinv, xc, S[x0 + qx + 1], S[x0 + qx - 1], S[x0 + qx + C2_XX],
                                 S[x0 + qx - C2_XX], S[xp + qx], S[xm + qx], k.ce, k.cw, k.cn, k.cs, k.ct, k.cb,
                                 DP ? S[dc + C2_P + q] : xc, a.c1a, a.c2a);
    S[o1 + q] = fx_add(xc, dn);
    return dn;
}

__device__ __forceinline__ int c2_wrap(int i, int r) { return i >= r ? i - r : i; }

template <bool DP, bool DO>
__global__ void __launch_bounds__(C2_THREADS, 4) k_cheb_pair(PairArgs a)
{
    extern __shared__ __align__(16) float c2_smem[];
    float *S = c2_smem;
    // offsets in S: C2_RD slots of first-step inputs, C2_RX planes of x,
    // C2_R1 planes of x after the first step
    constexpr int SD = 0, SX = C2_RD * C2_SLOT, S1 = SX + C2_RX * C2_NX;
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(c2_smem);
    const LevelView<float> &F = a.F;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + C2_TX * ty;
    const int i0 = blockIdx.x * C2_TX + 1, j0 = blockIdx.y * C2_TY + 1;
    const int k0 = blockIdx.z * a.planes + 1, k1 = min(k0 + a.planes - 1, F.n2);
    const C2Offs o = c2_offsets(F, i0, j0, tid);
    // this thread's column (tx + 1, ty + 1) of the 34 x 10 tile and its halo
    // cell (the ring around the 32 x 8 tile), as tile indices
    auto idx = [&](int ex, int ey, int &q, int &qe, int &qn, int &qx, bool &in) {
        const int i = i0 - 1 + ex, j = j0 - 1 + ey;
        q = ex + C2_EX * ey;
        qe = ex + C2_WE * ey;
        qn = ex + C2_EX * ey;
        qx = (ex + 2) + C2_XX * (ey + 1);
        in = i >= 1 && i <= F.n0 && j >= 1 && j <= F.n1;
    };
    int q0, qe0, qn0, qx0, qh = 0, qeh = 0, qnh = 0, qxh = 0;
    bool in0, inh = false;
    idx(tx + 1, ty + 1, q0, qe0, qn0, qx0, in0);
    int hx = -1, hy = 0;
    if (tid < C2_EX) { hx = tid; hy = 0; }
    else if (tid < 2 * C2_EX) { hx = tid - C2_EX; hy = C2_EY - 1; }
    else if (tid < 2 * C2_EX + C2_TY) { hx = 0; hy = tid - 2 * C2_EX + 1; }
    else if (tid < C2_NH) { hx = C2_EX - 1; hy = tid - 2 * C2_EX - C2_TY + 1; }
    const bool halo = hx >= 0;
    if (halo) idx(hx, hy, qh, qeh, qnh, qxh, inh);

    // group g: inputs of plane g and x of plane g + 1 (the first group also
    // x of plane k0 - 2); groups k0 - 2 .. k0 - 2 + C2_AHEAD before the loop.
    // Ring index of plane P: (P + 2) mod depth (P >= k0 - 2 >= -1).
    auto issue = [&](int rslot, int P, int rxs, int X) {
        c2_issue<DP>(a, o, sbase + 4u * (SD + rslot * C2_SLOT), P, sbase + 4u * (SX + rxs * C2_NX), X, tid);
    };
    issue(k0 % C2_RD, k0 - 2, k0 % C2_RX, k0 - 2);
    for (int g = k0 - 2; g <= k0 - 2 + C2_AHEAD; ++g) {
        issue((g + 2) % C2_RD, g == k0 - 2 ? -1 : g, (g + 3) % C2_RX, g + 1);
        __pipeline_commit();
    }
    // ring indices of plane kk (and the planes around it), advanced by one per plane
    int rd = (k0 + 1) % C2_RD, rx = (k0 + 1) % C2_RX, r1 = (k0 + 1) % C2_R1;
    float d1 = 0.f;     // first-step update of this thread's column, plane below
    C2Cell kc = {}, kp = {};
    const bool out_ok = tx + i0 <= F.n0 && ty + j0 <= F.n1;
    int c = (i0 + tx) + F.sy * (j0 + ty) + F.sz * (k0 - 2);   // output cell at plane kk - 1
    for (int kk = k0 - 1; kk <= k1 + 1; ++kk, c += F.sz) {
        const int g = kk + C2_AHEAD;
        if (g <= k1 + 1) issue(c2_wrap(rd + C2_AHEAD, C2_RD), g, c2_wrap(rx + C2_AHEAD + 1, C2_RX), g + 1);
        __pipeline_commit();
        __pipeline_wait_prior(C2_AHEAD);    // groups up to kk have landed
        __syncthreads();
        const int dc = SD + rd * C2_SLOT, dm = SD + (rd == 0 ? C2_RD - 1 : rd - 1) * C2_SLOT;
        const int x0 = SX + rx * C2_NX, xm = SX + (rx == 0 ? C2_RX - 1 : rx - 1) * C2_NX;
        const int xp = SX + c2_wrap(rx + 1, C2_RX) * C2_NX;
        const int o1 = S1 + r1 * C2_NE;
        const bool plane_in = kk >= 1 && kk <= F.n2;
        const float dn1 = c2_first<DP>(a, S, dc, dm, xm, x0, xp, o1, q0, qe0, qn0, qx0, in0 && plane_in, kc);
        if (halo) {
            C2Cell kh;
            c2_first<DP>(a, S, dc, dm, xm, x0, xp, o1, qh, qeh, qnh, qxh, inh && plane_in, kh);
        }
        __syncthreads();
        if (kk - 1 >= k0 && out_ok) {
            // second step at plane kk - 1 from the first-step planes kk - 2 .. kk
            const int r1m = r1 == 0 ? C2_R1 - 1 : r1 - 1;
            const int y0 = S1 + r1m * C2_NE, ym = S1 + (r1m == 0 ? C2_R1 - 1 : r1m - 1) * C2_NE, yp = o1;
            const int q = q0;
            const float xc = S[y0 + q];
            const float dn = cheb_update(kp.b, kp.dg, kp.dinv, xc, S[y0 + q + 1], S[y0 + q - 1], S[y0 + q + C2_EX],
                                         S[y0 + q - C2_EX], S[yp + q], S[ym + q], kp.ce, kp.cw, kp.cn, kp.cs, kp.ct,
                                         kp.cb, d1, a.c1b, a.c2b);
            a.xout[c] = fx_add(xc, dn);
            if (DO) a.dout[c] = dn;
        }
        d1 = dn1;
        kp = kc;
        rd = c2_wrap(rd + 1, C2_RD);
        rx = c2_wrap(rx + 1, C2_RX);
        r1 = c2_wrap(r1 + 1, C2_R1);
    }
    __pipeline_wait_prior(0);
}

// Smoother pairing: 1 (the default) on the levels where the pair kernel
// measured faster than two one-step launches -- at least 2^22 cells, with
// at least two waves of four blocks per SM -- 2 on every FP32 level of at
// least 2^18 cells, 0 off; k-planes per block of the pair kernel (fewer
// when that fills the grid).
static int g_pairs = 1, g_pair_planes = C2_PLANES;

void set_smoother_pairs(int on, int planes)
{
    g_pairs = on < 0 ? 0 : (on > 2 ? 2 : on);
    g_pair_planes = planes > 0 ? planes : C2_PLANES;
}

int smoother_pairs_state() { return g_pairs + 3 * g_pair_planes; }

// k-planes per block of the pair kernel on level F, 0: one-step kernels.
template <typename T>
int pair_planes(const MgLevel<T> &F)
{
    const long long cells = (long long)F.n0 * F.n1 * F.n2;
    if (sizeof(T) != 4 || g_pairs == 0 || cells < (1LL << 18) || (F.n0 & 1)) return 0;
    if (g_pairs == 2) return g_pair_planes;
    if (cells < (1LL << 22)) return 0;
    const long long tiles = (long long)((F.n0 + C2_TX - 1) / C2_TX) * ((F.n1 + C2_TY - 1) / C2_TY);
    for (int planes = g_pair_planes; planes >= 8; planes /= 2)
        if (tiles * ((F.n2 + planes - 1) / planes) >= 2LL * 4 * 152) return planes;
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
        const void *fns[4] = {(const void *)k_cheb_pair<false, false>, (const void *)k_cheb_pair<false, true>,
                              (const void *)k_cheb_pair<true, false>, (const void *)k_cheb_pair<true, true>};
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
// itself.  Needs an even n0 (rows 8-byte aligned); otherwise launches
// nothing and returns cudaErrorInvalidValue.
cudaError_t cheb_pair(const MgLevel<float> &F, const float *xin, const float *dprev, float *xout, float *dout,
                      double c1a, double c2a, double c1b, double c2b, cudaStream_t st)
{
    if (F.n0 & 1) return cudaErrorInvalidValue;
    PairArgs a;
    a.F = F.view();
    a.b = F.b; a.x = xin; a.dprev = dprev; a.xout = xout; a.dout = dout;
    a.c1a = (float)c1a; a.c2a = (float)c2a; a.c1b = (float)c1b; a.c2b = (float)c2b;
    a.planes = pair_planes(F) > 0 ? pair_planes(F) : g_pair_planes;
    pair_smem_attr();
    const dim3 blk(C2_TX, C2_TY, 1);
    const dim3 grd((F.n0 + C2_TX - 1) / C2_TX, (F.n1 + C2_TY - 1) / C2_TY, (F.n2 + a.planes - 1) / a.planes);
    if (dprev && dout) k_cheb_pair<true, true><<<grd, blk, C2_SMEM, st>>>(a);
    else if (dprev) k_cheb_pair<true, false><<<grd, blk, C2_SMEM, st>>>(a);
    else if (dout) k_cheb_pair<false, true><<<grd, blk, C2_SMEM, st>>>(a);
    else k_cheb_pair<false, false><<<grd, blk, C2_SMEM, st>>>(a);
    return cudaSuccess;
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

// Residual of the fine level summed over each coarse cell's children.  One
// thread per fine i and coarse (J,K): it sums the residuals of its (up to
// 2x2) fine cells in j and k, then lanes i and i^1 add their sums with a
// shuffle (always in the order even + odd), so the result is reproducible.
template <typename T>
__global__ void __launch_bounds__(128) k_restrict(LevelView<T> F, const T *__restrict__ b,
                                                  const T *__restrict__ x, LevelView<T> C, T *__restrict__ bc,
                                                  int f0, int f1, int f2)
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
                s += b[fc] - apply_row(F, x, fc);
            }
    }
    if (f0 == 2) {
        const T o = __shfl_xor_sync(0xffffffffu, s, 1);
        if ((threadIdx.x & 1) == 0) s = s + o;
        else return;
    }
    if (!in) return;
    const int I = f0 == 2 ? ((i - 1) >> 1) + 1 : i;
    bc[I + C.sy * J + C.sz * K] = s;
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
// prolongations cost more than one extra pass over x.
template <typename T>
__global__ void __launch_bounds__(256) k_prolong(LevelView<T> F, const unsigned char *__restrict__ act,
                                                 T *__restrict__ x, LevelView<T> C, const T *__restrict__ e, int s0,
                                                 int s1, int s2)
{
    INTERIOR_IJK(F);
    if (!in || !act[c]) return;
    x[c] += e[(((i - 1) >> s0) + 1) + C.sy * (((j - 1) >> s1) + 1) + C.sz * (((k - 1) >> s2) + 1)];
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

template <typename T>
T *mg_vcycle(MgLevel<T> *L, int nlev, const ChebCoef &cc, const double *ainv, const int *map, int ncoarse,
             bool singular, bool first_done, cudaStream_t st, int *launches, KTimer *kt)
{
    T *cur[32];
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
            k_restrict<T><<<rg, rb, 0, st>>>(v, F.b, xa, C.view(), C.b, F.f0, F.f1, F.f2);
            kt_end(kt, id, st);
            *launches += 1;
            continue;
        }
        if (!(l == 0 && first_done)) {
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
        k_restrict<T><<<rg, rb, 0, st>>>(v, F.b, xa, C.view(), C.b, F.f0, F.f1, F.f2);
        kt_end(kt, id, st);
        *launches += 1;
    }
    {
        MgLevel<T> &Cst = L[last];
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
            k_prolong<T><<<lf.grid, lf.block, 0, st>>>(v, F.active, xa, C.view(), cur[l + 1], F.f0 - 1, F.f1 - 1,
                                                       F.f2 - 1);
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
                k_prolong<T><<<lf.grid, lf.block, 0, st>>>(v, F.active, xa, C.view(), cur[l + 1], F.f0 - 1, F.f1 - 1,
                                                           F.f2 - 1);
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
            k_prolong<T><<<lf.grid, lf.block, 0, st>>>(v, F.active, xa, C.view(), cur[l + 1], F.f0 - 1, F.f1 - 1,
                                                       F.f2 - 1);
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
    k_restrict<T><<<rg, rb, 0, st>>>(F.view(), F.b, F.x, C.view(), C.b, F.f0, F.f1, F.f2);
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
                                 bool, cudaStream_t, int *, KTimer *);
template double *mg_vcycle<double>(MgLevel<double> *, int, const ChebCoef &, const double *, const int *, int, bool,
                                   bool, cudaStream_t, int *, KTimer *);
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
