// k_assemble.cu -- face coefficients, pressure operator and right-hand side.
//
// Compiled with -fmad=false: every product and sum is rounded on its own, in
// the reference's evaluation order, so PoCoef, the operator and b are
// bit-identical to a strict IEEE evaluation of the Fortran expressions.
#include "scf_kernels.h"

namespace {

// 1 = wet, 2 = dry, 0 = neither (ProjectionP.f90:170-174,212-221)
__device__ __forceinline__ int phase_of(double vofl, double vof, double phil, double epsi)
{
    const double hi = 1.0 - epsi;
    if ((vofl >= 0.5 && vof > hi) || (phil < 0.0 && vof <= hi && vof > epsi)) return 1;
    if ((vofl < 0.5 && vof > hi) || (phil >= 0.0 && vof <= hi && vof > epsi)) return 2;
    return 0;
}

// Direction table, faces W,S,B,E,N,T (PoCoef order).
__device__ __constant__ int c_di[6] = {-1, 0, 0, 1, 0, 0};
__device__ __constant__ int c_dj[6] = {0, -1, 0, 0, 1, 0};
__device__ __constant__ int c_dk[6] = {0, 0, -1, 0, 0, 1};

struct FaceGeo {
    const double *dp, *dg;
};

__device__ __forceinline__ FaceGeo face_geo(const AsmArgs &a, int f)
{
    FaceGeo g;
    const int axis = f % 3;
    g.dp = axis == 0 ? a.dpu : axis == 1 ? a.dpv : a.dpw;
    g.dg = axis == 0 ? a.udx : axis == 1 ? a.vdy : a.wdz;
    return g;
}

// Dp(im,jm,km)/DGrid with DGrid at (max(im,1),max(jm,1),max(km,1))
// (ProjectionP.f90:145-153).
__device__ __forceinline__ void face_terms(const AsmArgs &a, int f, int i, int j, int k, double &dp, double &dgrid)
{
    const Dims &d = a.d;
    const int minus = f < 3;
    const int im = i - (minus ? (c_di[f] != 0) : 0);
    const int jm = j - (minus ? (c_dj[f] != 0) : 0);
    const int km = k - (minus ? (c_dk[f] != 0) : 0);
    FaceGeo g = face_geo(a, f);
    dp = g.dp[gidx(d, im, jm, km)];
    dgrid = g.dg[nidx(d, im < 1 ? 1 : im, jm < 1 ? 1 : jm, km < 1 ? 1 : km)];
}

// The reference's coefficient expression Dp/DGrid*BetaP*BetaM/Beta.
__device__ __forceinline__ double coef_expr(double dp, double dgrid, double betap, double betam, double beta)
{
    double t = dp / dgrid;
    t = t * betap;
    t = t * betam;
    return t / beta;
}

__device__ __forceinline__ double lamda_of(const AsmArgs &a, int gc, int gn)
{
    const double pc = fabs(a.phil[gc]), pn = fabs(a.phil[gn]);
    return pc / ((pc + pn) + a.tol);
}

}  // namespace

// ---------------------------------------------------------------------------
// K1: Compute1DGFMCoefficient for the six faces (ProjectionP.f90:123-265).
//
// The reference's BetaW/BetaD are locals that keep their last assigned value:
// a wet (dry) cell whose neighbour is neither wet nor dry reuses the BetaW
// (BetaD) of the latest earlier cell, in its loop order (i outer, j, k
// innermost), that assigned it within the same face call.  Each thread
// marches one (i,j) column in k -- exactly a contiguous run of that loop
// order -- and carries the twelve (face, W/D) values in registers.  Cells
// with no earlier assignment inside their column ("head" cells) are listed
// and resolved from per-column and per-group summaries (k_pocoef_heads).
namespace {
__device__ __forceinline__ double beta_of(int pc, int pn, double lam, double betap, double betam)
{
    if (pc == 1) return pn == 2 ? lam * betam + (1.0 - lam) * betap : betam;
    return pn == 1 ? lam * betap + (1.0 - lam) * betam : betap;
}
}  // namespace

__global__ void __launch_bounds__(128) k_pocoef(AsmArgs a)
{
    const Dims &d = a.d;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > d.I || j > d.J) return;
    const int col = (i - 1) * d.J + (j - 1);   // column index in loop order
    double carry[12];
    unsigned mask = 0;
#pragma unroll
    for (int s = 0; s < 12; ++s) carry[s] = 0.0;
    for (int k = 1; k <= d.K; ++k) {
        const int gc = gidx(d, i, j, k), nc = nidx(d, i, j, k);
        const int pc = phase_of(a.vofl[gc], a.vof[gc], a.phil[gc], a.epsi);
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            double coef = 0.0;
            if (pc != 0) {
                const int gn = gidx(d, i + c_di[f], j + c_dj[f], k + c_dk[f]);
                const int pn = phase_of(a.vofl[gn], a.vof[gn], a.phil[gn], a.epsi);
                const int s = 2 * f + (pc == 2);
                double dp, dg;
                face_terms(a, f, i, j, k, dp, dg);
                if (pn != 0) {
                    const double lam = (pc != pn) ? lamda_of(a, gc, gn) : 0.0;
                    const double beta = beta_of(pc, pn, lam, a.betap, a.betam);
                    carry[s] = beta;
                    mask |= 1u << s;
                    coef = coef_expr(dp, dg, a.betap, a.betam, beta);
                } else if (mask & (1u << s)) {
                    coef = coef_expr(dp, dg, a.betap, a.betam, carry[s]);
                } else {
                    unsigned slot = atomicAdd(a.stale_count, 1u);
                    if (slot < a.stale_cap) {
                        const long long L = ((long long)col) * d.K + (k - 1);
                        a.stale_list[slot] = (L << 4) | ((long long)s);
                    } else {
                        atomicOr(a.flags, FLAG_STALE_OVERFLOW);
                    }
                }
            }
            a.pocoef[nc + (long long)d.n * f] = coef;
        }
    }
#pragma unroll
    for (int s = 0; s < 12; ++s) a.col_val[(long long)col * 12 + s] = carry[s];
    a.col_mask[col] = (unsigned short)mask;
}

// Group summaries: the last assignment of each (face, W/D) stream within
// 64 consecutive columns.
__global__ void k_pocoef_groups(AsmArgs a, int ncol, int ngrp)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngrp) return;
    double v[12];
    unsigned m = 0;
#pragma unroll
    for (int s = 0; s < 12; ++s) v[s] = 0.0;
    const int c1 = min(ncol, (g + 1) * 64);
    for (int c = g * 64; c < c1; ++c) {
        const unsigned cm = a.col_mask[c];
        if (!cm) continue;
#pragma unroll
        for (int s = 0; s < 12; ++s)
            if (cm & (1u << s)) v[s] = a.col_val[(long long)c * 12 + s];
        m |= cm;
    }
#pragma unroll
    for (int s = 0; s < 12; ++s) a.grp_val[(long long)g * 12 + s] = v[s];
    a.grp_mask[g] = (unsigned short)m;
}

// Head cells: the carried value comes from the latest earlier column (first
// within the cell's group, then whole groups) that assigned the stream.
__global__ void k_pocoef_heads(AsmArgs a, unsigned count)
{
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const Dims &d = a.d;
    const long long e = a.stale_list[t];
    const int s = (int)(e & 15);
    const int f = s >> 1;
    const long long L = e >> 4;
    const int col = (int)(L / d.K), k = (int)(L % d.K) + 1;
    const int i = col / d.J + 1, j = col % d.J + 1;
    const unsigned bit = 1u << s;
    double beta = a.stale_init;
    bool found = false;
    const int g = col / 64;
    for (int c = col - 1; c >= g * 64; --c)
        if (a.col_mask[c] & bit) { beta = a.col_val[(long long)c * 12 + s]; found = true; break; }
    if (!found)
        for (int q = g - 1; q >= 0; --q)
            if (a.grp_mask[q] & bit) { beta = a.grp_val[(long long)q * 12 + s]; break; }
    double dp, dg;
    face_terms(a, f, i, j, k, dp, dg);
    a.pocoef[nidx(d, i, j, k) + (long long)d.n * f] = coef_expr(dp, dg, a.betap, a.betam, beta);
}

// Boundary planes take the neighbouring plane (ProjectionP.f90:256-264).
__global__ void k_pocoef_boundary(AsmArgs a)
{
    const Dims &d = a.d;
    const int f = blockIdx.z;  // 0..5
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int axis = f % 3;
    const int na = axis == 0 ? d.J : d.I;
    const int nb = axis == 2 ? d.J : d.K;
    if (t >= na * nb) return;
    const int p = t % na + 1, q = t / na + 1;
    const bool minus = f < 3;
    double *pc = a.pocoef + (long long)d.n * f;
    if (axis == 0) {
        const int dst = minus ? 1 : d.I, src = minus ? 2 : d.I - 1;
        pc[nidx(d, dst, p, q)] = pc[nidx(d, src, p, q)];
    } else if (axis == 1) {
        const int dst = minus ? 1 : d.J, src = minus ? 2 : d.J - 1;
        pc[nidx(d, p, dst, q)] = pc[nidx(d, p, src, q)];
    } else {
        const int dst = minus ? 1 : d.K, src = minus ? 2 : d.K - 1;
        pc[nidx(d, p, q, dst)] = pc[nidx(d, p, q, src)];
    }
}

// ---------------------------------------------------------------------------
// K2: operator rows of SetPoissonMatrix (ProjectionP.f90:330-478) and the
// right-hand side of SetPoissonVectors (ProjectionP.f90:513-564).
// Per active cell: the exact diagonal, the couplings towards E/N/T from the
// cell's own row, the diagonal part without a coupling (Dirichlet faces and
// faces to solid cells, used to coarsen), and b.  Solid cells: identity.
template <bool MIXED>
__global__ void k_operator(AsmArgs a, OpArgs o)
{
    const Dims &d = a.d;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
    if (i > d.I || j > d.J || k > d.K) return;
    const int g = gidx(d, i, j, k), n = nidx(d, i, j, k);
    const int ct = a.ct[n], pos = a.pos[n];
    if ((pos == -1) != (ct == 2) || pos > a.ext_cell || pos < -1) atomicOr(a.flags, FLAG_BAD_POSNU);
    if (ct == 2) {
        o.diag[g] = 1.0; o.dinv[g] = 0.0; o.cE[g] = 0.0; o.cN[g] = 0.0; o.cT[g] = 0.0;
        o.extra[g] = 0.0; o.b[g] = 0.0; o.active[g] = 0;
        if (MIXED) {
            o.diag32[g] = 1.0f; o.dinv32[g] = 0.0f; o.cE32[g] = 0.0f; o.cN32[g] = 0.0f; o.cT32[g] = 0.0f;
            o.extra32[g] = 0.0f;
        }
        return;
    }
    const double dx = a.pdx[n], dy = a.pdy[n], dz = a.pdz[n];
    const long long N = d.n;
    const double p1 = a.pocoef[n], p2 = a.pocoef[n + N], p3 = a.pocoef[n + 2 * N];
    const double p4 = a.pocoef[n + 3 * N], p5 = a.pocoef[n + 4 * N], p6 = a.pocoef[n + 5 * N];
    const double eW = a.ee[g - 1], eE = a.ee[g];
    const double nS = a.ne[g - d.gx], nN = a.ne[g];
    const double tB = a.te[g - d.gx * d.gy], tT = a.te[g];
    const double t1 = p1 * eW * dy * dz, t2 = p2 * nS * dx * dz, t3 = p3 * tB * dx * dy;
    const double t4 = p4 * eE * dy * dz, t5 = p5 * nN * dx * dz, t6 = p6 * tT * dx * dy;
    double dg = t1 + t2 + t3 + t4 + t5 + t6;
    const int *fl = a.flag;
    if (fl[0] == 1 && i == 1) dg = dg - t1;
    if (fl[2] == 1 && j == 1) dg = dg - t2;
    if (fl[4] == 1 && k == 1) dg = dg - t3;
    if (fl[1] == 1 && i == d.I) dg = dg - t4;
    if (fl[3] == 1 && j == d.J) dg = dg - t5;
    if (fl[5] == 1 && k == d.K) dg = dg - t6;
    double cE = 0.0, cN = 0.0, cT = 0.0, ex = 0.0;
    if (i == 1) { if (fl[0] == 0) ex += t1; } else if (a.pos[n - 1] == -1) ex += t1;
    if (j == 1) { if (fl[2] == 0) ex += t2; } else if (a.pos[n - d.I] == -1) ex += t2;
    if (k == 1) { if (fl[4] == 0) ex += t3; } else if (a.pos[n - d.I * d.J] == -1) ex += t3;
    if (i == d.I) { if (fl[1] == 0) ex += t4; } else if (a.pos[n + 1] == -1) ex += t4; else cE = t4;
    if (j == d.J) { if (fl[3] == 0) ex += t5; } else if (a.pos[n + d.I] == -1) ex += t5; else cN = t5;
    if (k == d.K) { if (fl[5] == 0) ex += t6; } else if (a.pos[n + d.I * d.J] == -1) ex += t6; else cT = t6;

    // right-hand side (ProjectionP.f90:521-546)
    const double *u = a.us, *v = a.vs, *w = a.ws;
    const int sy = d.gx, sz = d.gx * d.gy;
    double r = -dy * dz * (eE * u[g] - eW * u[g - 1]) - dx * dz * (nN * v[g] - nS * v[g - sy]) -
               dx * dy * (tT * w[g] - tB * w[g - sz]);
    r = r + (a.vof[g] - a.vofo[g]) * dx * dy * dz / a.dt;
    if (fl[0] == 0 && i == 1) r = r + p1 * a.bvar[0][(j - 1) + d.J * (k - 1)];
    if (fl[1] == 0 && i == d.I) r = r + p4 * a.bvar[1][(j - 1) + d.J * (k - 1)];
    if (fl[2] == 0 && j == 1) r = r + p2 * a.bvar[2][(i - 1) + d.I * (k - 1)];
    if (fl[3] == 0 && j == d.J) r = r + p5 * a.bvar[3][(i - 1) + d.I * (k - 1)];
    if (fl[4] == 0 && k == 1) r = r + p3 * a.bvar[4][(i - 1) + d.I * (j - 1)];
    if (fl[5] == 0 && k == d.K) r = r + p6 * a.bvar[5][(i - 1) + d.I * (j - 1)];

    if (!(dg > 0.0) || !isfinite(dg)) atomicOr(a.flags, isfinite(dg) ? FLAG_BAD_DIAG : FLAG_NONFINITE);
    if (!isfinite(r) || !isfinite(cE) || !isfinite(cN) || !isfinite(cT) || !isfinite(ex))
        atomicOr(a.flags, FLAG_NONFINITE);
    const int phc = phase_of(a.vofl[g], a.vof[g], a.phil[g], a.epsi);
    if (phc == 0) atomicOr(a.flags, FLAG_NEITHER_ACTIVE);

    o.diag[g] = dg;
    o.dinv[g] = dg > 0.0 ? 1.0 / dg : 0.0;
    o.cE[g] = cE; o.cN[g] = cN; o.cT[g] = cT;
    o.extra[g] = ex;
    o.b[g] = r;
    o.active[g] = 1;
    if (MIXED) {
        const float d32 = (float)dg;
        o.diag32[g] = d32;
        o.dinv32[g] = d32 > 0.0f ? 1.0f / d32 : 0.0f;
        o.cE32[g] = (float)cE; o.cN32[g] = (float)cN; o.cT32[g] = (float)cT;
        o.extra32[g] = (float)ex;
    }
}

// ---------------------------------------------------------------------------
// host launchers
int launch_assemble(const AsmArgs &a, const OpArgs &o, bool mixed, cudaStream_t st, unsigned *stale_count_host,
                    int *launches)
{
    const Dims &d = a.d;
    cudaMemsetAsync(a.stale_count, 0, sizeof(unsigned), st);
    {
        dim3 b(32, 4), g((d.I + 31) / 32, (d.J + 3) / 4);
        k_pocoef<<<g, b, 0, st>>>(a);
        *launches += 1;
    }
    cudaMemcpyAsync(stale_count_host, a.stale_count, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    unsigned cnt = *stale_count_host;
    if (cnt > a.stale_cap) cnt = a.stale_cap;
    if (cnt) {
        const int ncol = d.I * d.J, ngrp = (ncol + 63) / 64;
        k_pocoef_groups<<<(ngrp + 127) / 128, 128, 0, st>>>(a, ncol, ngrp);
        k_pocoef_heads<<<(cnt + 127) / 128, 128, 0, st>>>(a, cnt);
        *launches += 2;
    }
    {
        int m = d.J * d.K;
        if (d.I * d.K > m) m = d.I * d.K;
        if (d.I * d.J > m) m = d.I * d.J;
        dim3 g((m + 255) / 256, 1, 6);
        k_pocoef_boundary<<<g, 256, 0, st>>>(a);
        *launches += 1;
    }
    Launch3 l = launch_interior(d.I, d.J, d.K);
    if (mixed)
        k_operator<true><<<l.grid, l.block, 0, st>>>(a, o);
    else
        k_operator<false><<<l.grid, l.block, 0, st>>>(a, o);
    *launches += 1;
    return (int)cudaGetLastError();
}
