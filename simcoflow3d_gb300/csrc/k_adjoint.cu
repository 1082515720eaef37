// k_adjoint.cu -- loss and adjoint gradient of the projection.
//
// Loss: J = sum_c g_c p_c + 1/2 sum_{active c} (D u)_c^2, with p the
// zero-mean pressure, u the corrected face velocity (ComputePUVW.f90:181-232,
// before the boundary routines; the west/south/bottom boundary faces keep
// u*) and D the discrete divergence of SetPoissonVectors
// (ProjectionP.f90:521-526).  Densities are a per-cell field; a face between
// an owner cell a and its E/N/T neighbour b has the GFM density
// rho_f = lam rho_a + (1-lam) rho_b, lam = |phiL_a|/(|phiL_a|+|phiL_b|+tol),
// and coefficient Dp/DGrid * rho_ref/rho_f -- the reference's coefficient
// (ProjectionP.f90:155-235) when rho is the density of each cell's phase.
//
// Adjoint (the operator A is symmetric):  A lam = P g + A_m r, r = D u,
// where A_m is the face Laplacian with the correction's masked weights and P
// removes the mean over active cells; then
//   dJ/du*_f  = m_f a_f (r_c - r_n) - a_f (lam_c - lam_n)
//   dJ/dcoef_f = -a_f (lam_c - lam_n)(p_c - p_n) - m_f a_f (r_c - r_n)(p_n - p_c)
//   dJ/drho   = sum over faces of dJ/dcoef_f * dcoef_f/drho.
// All-Neumann pressure boundaries.
#include "scf_kernels.h"

namespace {

__device__ __forceinline__ int face_stride(const Dims &d, int ax) { return ax == 0 ? 1 : ax == 1 ? d.gx : d.gx * d.gy; }
__device__ __forceinline__ int cell_stride(const Dims &d, int ax) { return ax == 0 ? 1 : ax == 1 ? d.I : d.I * d.J; }

}  // namespace

// Coefficients with per-cell densities (before the boundary-plane copy).
__global__ void __launch_bounds__(256) k_pocoef_rho(AsmArgs a, const double *__restrict__ rho, double rho_ref)
{
    const Dims &d = a.d;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
    if (i > d.I || j > d.J || k > d.K) return;
    const int gc = gidx(d, i, j, k), nc = nidx(d, i, j, k);
    const int pc = a.phase[gc];
    for (int f = 0; f < 6; ++f) {
        const int ax = f % 3, sgn = f < 3 ? -1 : 1;
        double coef = 0.0;
        if (pc != 0) {
            const int gn = gc + sgn * face_stride(d, ax);
            const int pn = a.phase[gn];
            const int im = i - (f == 0), jm = j - (f == 1), km = k - (f == 2);
            const double *dp = ax == 0 ? a.dpu : ax == 1 ? a.dpv : a.dpw;
            const double *dg = ax == 0 ? a.udx : ax == 1 ? a.vdy : a.wdz;
            const double ratio = dp[gidx(d, im, jm, km)] / dg[nidx(d, im < 1 ? 1 : im, jm < 1 ? 1 : jm, km < 1 ? 1 : km)];
            double lam = 1.0;
            if (pn != 0) {
                const double x = fabs(a.phil[gc]), y = fabs(a.phil[gn]);
                lam = x / ((x + y) + a.tol);
            }
            const double rf = lam * rho[gc] + (1.0 - lam) * rho[gn];
            coef = ratio * rho_ref / rf;
        }
        a.pocoef[nc + (long long)d.n * f] = coef;
    }
}

// u of the upper face of cell (i,j,k) along ax (corrected, or 0 if masked)
__device__ __forceinline__ double upper_u(const AdjArgs &A, int ax, int g, int n)
{
    const Dims &d = A.d;
    const int *mo = ax == 0 ? A.umoex : ax == 1 ? A.vmoex : A.wmoex;
    const int *ct = ax == 0 ? A.uct : ax == 1 ? A.vct : A.wct;
    const double *us = ax == 0 ? A.us : ax == 1 ? A.vs : A.ws;
    if (mo[n] == 1 || ct[n] == 2) return 0.0;
    return us[g] - (A.pp[g + face_stride(d, ax)] - A.pp[g]) * A.pocoef[n + (long long)d.n * (3 + ax)];
}

__device__ __forceinline__ double area(const AdjArgs &A, int ax, int g, int n)
{
    const double *ar = ax == 0 ? A.ee : ax == 1 ? A.ne : A.te;
    const double d1 = ax == 0 ? A.pdy[n] : A.pdx[n];
    const double d2 = ax == 2 ? A.pdy[n] : A.pdz[n];
    return d1 * d2 * ar[g];
}

// r = D u on active cells; partial sums of g.p and r.r/2
__global__ void __launch_bounds__(256) k_adj_divergence(AdjArgs A, double *__restrict__ part, int n0)
{
    const Dims &d = A.d;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
    double sp = 0.0, sr = 0.0;
    if (i <= d.I && j <= d.J && k <= d.K) {
        const int g = gidx(d, i, j, k), n = nidx(d, i, j, k);
        double r = 0.0;
        if (A.ct[n] != 2) {
            const int idx[3] = {i, j, k};
            for (int ax = 0; ax < 3; ++ax) {
                const double uu = upper_u(A, ax, g, n);
                const int gl = g - face_stride(d, ax);
                const double ul = idx[ax] > 1 ? upper_u(A, ax, gl, n - cell_stride(d, ax))
                                              : (ax == 0 ? A.us : ax == 1 ? A.vs : A.ws)[gl];
                const double *ar = ax == 0 ? A.ee : ax == 1 ? A.ne : A.te;
                const double d1 = ax == 0 ? A.pdy[n] : A.pdx[n];
                const double d2 = ax == 2 ? A.pdy[n] : A.pdz[n];
                r += d1 * d2 * (ar[g] * uu - ar[gl] * ul);
            }
            sp = A.gw[g] * A.pp[g];
            sr = 0.5 * r * r;
        }
        A.r[g] = r;
    }
    sp = block_sum(sp);
    __syncthreads();
    sr = block_sum(sr);
    if (thread_linear() == 0) {
        part[block_linear()] = sp;
        part[n0 + block_linear()] = sr;
    }
}

// adjoint right-hand side: (g - mean g) + A_m r, written to b
__global__ void __launch_bounds__(256) k_adj_rhs(AdjArgs A, const double *__restrict__ scal, double *__restrict__ b)
{
    const Dims &d = A.d;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
    if (i > d.I || j > d.J || k > d.K) return;
    const int g = gidx(d, i, j, k), n = nidx(d, i, j, k);
    if (A.ct[n] == 2) { b[g] = 0.0; return; }
    double s = A.gw[g] - scal[S_MEAN];
    const int idx[3] = {i, j, k};
    const int lim[3] = {d.I, d.J, d.K};
    for (int ax = 0; ax < 3; ++ax) {
        const int *mo = ax == 0 ? A.umoex : ax == 1 ? A.vmoex : A.wmoex;
        const int *ct = ax == 0 ? A.uct : ax == 1 ? A.vct : A.wct;
        const int fs = face_stride(d, ax), cs = cell_stride(d, ax);
        if (idx[ax] < lim[ax] && mo[n] != 1 && ct[n] != 2)
            s += A.pocoef[n + (long long)d.n * (3 + ax)] * area(A, ax, g, n) * (A.r[g] - A.r[g + fs]);
        if (idx[ax] > 1 && mo[n - cs] != 1 && ct[n - cs] != 2)
            s -= A.pocoef[n - cs + (long long)d.n * (3 + ax)] * area(A, ax, g - fs, n - cs) * (A.r[g - fs] - A.r[g]);
    }
    b[g] = s;
}

// gradients: u* faces (ghosted, face-indexed like u*) and cell densities
__global__ void __launch_bounds__(256) k_adj_grad(AdjArgs A, const double *__restrict__ lam, const double *__restrict__ rho,
                                                  double rho_ref, double *gu, double *gv, double *gw, double *grho)
{
    const Dims &d = A.d;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
    if (i > d.I || j > d.J || k > d.K) return;
    const int g = gidx(d, i, j, k), n = nidx(d, i, j, k);
    const int idx[3] = {i, j, k};
    const int lim[3] = {d.I, d.J, d.K};
    double *gout[3] = {gu, gv, gw};
    double gr = 0.0;
    const double *p = A.pfwd;
    for (int ax = 0; ax < 3; ++ax) {
        const int *mo = ax == 0 ? A.umoex : ax == 1 ? A.vmoex : A.wmoex;
        const int *ct = ax == 0 ? A.uct : ax == 1 ? A.vct : A.wct;
        const int fs = face_stride(d, ax), cs = cell_stride(d, ax);
        const double m = (mo[n] != 1 && ct[n] != 2) ? 1.0 : 0.0;
        const double a = area(A, ax, g, n);
        const bool inner = idx[ax] < lim[ax];
        const double rn = inner ? A.r[g + fs] : 0.0, ln = inner ? lam[g + fs] : 0.0;
        if (gout[ax]) {
            gout[ax][g] = m * a * (A.r[g] - rn) - a * (lam[g] - ln);
            if (idx[ax] == 1) {
                const double al = area(A, ax, g - fs, n);
                gout[ax][g - fs] = -al * A.r[g] + al * lam[g];
            }
        }
        if (!grho) continue;
        // own upper face (owner = this cell) and lower face (owner = lower cell)
        for (int side = 0; side < 2; ++side) {
            const int go = side == 0 ? g : g - fs;          // owner (ghosted)
            const int no = side == 0 ? n : n - cs;          // owner (interior)
            const bool ok = side == 0 ? inner : idx[ax] > 1;
            if (!ok) continue;
            const int gu_ = go + fs;                         // upper cell
            const double coef = A.pocoef[no + (long long)d.n * (3 + ax)];
            if (coef == 0.0) continue;
            const double mo_ = (mo[no] != 1 && ct[no] != 2) ? 1.0 : 0.0;
            const double ao = area(A, ax, go, no);
            const double gcoef = -ao * (lam[go] - lam[gu_]) * (p[go] - p[gu_]) -
                                 mo_ * ao * (A.r[go] - A.r[gu_]) * (p[gu_] - p[go]);
            double l = 1.0;
            if (A.phase[gu_] != 0) {
                const double x = fabs(A.phil[go]), y = fabs(A.phil[gu_]);
                l = x / ((x + y) + A.tol);
            }
            const double rf = l * rho[go] + (1.0 - l) * rho[gu_];
            const double dc = -coef / rf;
            gr += gcoef * dc * (side == 0 ? l : 1.0 - l);
        }
    }
    if (grho) grho[g] = A.ct[n] != 2 ? gr : 0.0;
}

__global__ void k_phase_density(const unsigned char *__restrict__ ph, double *__restrict__ rho, int ng, double rl,
                                double rg)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x)
        rho[g] = ph[g] == 2 ? rg : rl;
}

void fill_phase_density(const unsigned char *phase, double *rho, int ng, double rho_l, double rho_g, cudaStream_t st,
                        int *launches)
{
    k_phase_density<<<152 * 8, 256, 0, st>>>(phase, rho, ng, rho_l, rho_g);
    *launches += 1;
}

void launch_pocoef_rho(const AsmArgs &a, const double *rho, double rho_ref, cudaStream_t st, int *launches)
{
    Launch3 l = launch_interior(a.d.I, a.d.J, a.d.K);
    k_pocoef_rho<<<l.grid, l.block, 0, st>>>(a, rho, rho_ref);
    *launches += 1;
}

void launch_adj_divergence(const AdjArgs &A, Reducer &R, cudaStream_t st, int *launches)
{
    Launch3 l = launch_interior(A.d.I, A.d.J, A.d.K);
    k_adj_divergence<<<l.grid, l.block, 0, st>>>(A, R.partials, R.max_blocks);
    *launches += 1;
    reduce2_to(R, (int)nblocks(l), 2, st, launches);
}

void launch_adj_rhs(const AdjArgs &A, const double *scal, double *b, cudaStream_t st, int *launches)
{
    Launch3 l = launch_interior(A.d.I, A.d.J, A.d.K);
    k_adj_rhs<<<l.grid, l.block, 0, st>>>(A, scal, b);
    *launches += 1;
}

void launch_adj_grad(const AdjArgs &A, const double *lam, const double *rho, double rho_ref, double *gu, double *gv,
                     double *gw, double *grho, cudaStream_t st, int *launches)
{
    Launch3 l = launch_interior(A.d.I, A.d.J, A.d.K);
    k_adj_grad<<<l.grid, l.block, 0, st>>>(A, lam, rho, rho_ref, gu, gv, gw, grho);
    *launches += 1;
}
