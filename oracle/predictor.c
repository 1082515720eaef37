/*
 * predictor.c -- CPU restatement of the implicit solves of SIMCOFlow's
 * momentum predictor (src/PredictUVW.f90).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the CUDA predictor kernels and
 * the timed CPU baseline of their benchmark; nothing in the product links or
 * calls it.  Parity status: the reference (Fortran + HYPRE) cannot be built
 * on this machine and its tests hold no golden values for these routines, so
 * the restatement is pinned by known-answer tests in tests/ (a diagonal
 * system solved in closed form, a 1-D diffusion row checked by hand, the
 * numbering and boundary rules), not by reference outputs.  The reference
 * solves with HYPRE PCG + BoomerAMG to its own tolerance; here the system is
 * solved with Jacobi-preconditioned BiCGStab to a much tighter one, so parity
 * is "same system, same solution".
 *
 * Loops and expressions keep the reference's order; built with
 * -ffp-contract=off.  Fortran Fr**2.d0 is written Fr*Fr (exact).
 *
 * Indexing (column-major, i fastest): ghosted (0:I+1,0:J+1,0:K+1), interior
 * (1:I,1:J,1:K); face arrays DFEW (0:I+1,1:J,1:K), DFNS (1:I,0:J+1,1:K),
 * DFTB (1:I,1:J,0:K+1); PosNu (1:I-iu,1:J-iv,1:K-iw).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "../include/scf_predictor.h"

static int I, J, K;
#define G(i, j, k) ((size_t)(i) + (size_t)(I + 2) * ((size_t)(j) + (size_t)(J + 2) * (size_t)(k)))
#define N(i, j, k) ((size_t)((i) - 1) + (size_t)I * ((size_t)((j) - 1) + (size_t)J * (size_t)((k) - 1)))
#define FEW(i, j, k) ((size_t)(i) + (size_t)(I + 2) * ((size_t)((j) - 1) + (size_t)J * (size_t)((k) - 1)))
#define FNS(i, j, k) ((size_t)((i) - 1) + (size_t)I * ((size_t)(j) + (size_t)(J + 2) * (size_t)((k) - 1)))
#define FTB(i, j, k) ((size_t)((i) - 1) + (size_t)I * ((size_t)((j) - 1) + (size_t)J * (size_t)(k)))

/* One cell's row: the seven coefficients in HYPRE's order W,S,B,P,E,N,T
 * (PredictUVW.f90:1044-1097), the right-hand side, Dp, and which
 * off-diagonals exist.                                                    */
typedef struct {
    double aw, as, ab, ap, ae, an, at;
    double rhs, dp;
} MomRow;

/* SetMatrix (PredictUVW.f90:904-1040) and SetVectors (1211-1260) for the
 * active cell (i, j, k) of component comp (1 = u, 2 = v, 3 = w).           */
static MomRow mom_row(const scf_mom_in *in, const scf_mom_opts *o, int comp, int i, int j, int k)
{
    const int iu = comp == 1, iv = comp == 2, iw = comp == 3;
    const int ie = I - iu, je = J - iv, ke = K - iw;
    const double CoefEW = (double)iu + (double)iv / 2.0 + (double)iw / 2.0;
    const double CoefNS = (double)iu / 2.0 + (double)iv + (double)iw / 2.0;
    const double CoefTB = (double)iu / 2.0 + (double)iv / 2.0 + (double)iw;
    const double omb = 1.0 - o->beta_vis;
    const size_t g = G(i, j, k), n = N(i, j, k);
    const double vof = in->vof[g], vofl = in->vofl[g];
    const double RhoCell = vofl * o->rho_w_ref + (vof - vofl) * o->rho_a_ref;
    double Dfe = omb * in->df_ew[FEW(i + 1, j, k)] / RhoCell;
    double Dfw = omb * in->df_ew[FEW(i, j, k)] / RhoCell;
    double Dfn = omb * in->df_ns[FNS(i, j + 1, k)] / RhoCell;
    double Dfs = omb * in->df_ns[FNS(i, j, k)] / RhoCell;
    double Dft = omb * in->df_tb[FTB(i, j, k + 1)] / RhoCell;
    double Dfb = omb * in->df_tb[FTB(i, j, k)] / RhoCell;
    const double ee = in->edf_ew[FEW(i + 1, j, k)], ew = in->edf_ew[FEW(i, j, k)];
    const double en = in->edf_ns[FNS(i, j + 1, k)], es = in->edf_ns[FNS(i, j, k)];
    const double et = in->edf_tb[FTB(i, j, k + 1)], eb = in->edf_tb[FTB(i, j, k)];
    const double etaE = in->eta_e[g], etaW = in->eta_e[G(i - 1, j, k)];
    const double etaN = in->eta_n[g], etaS = in->eta_n[G(i, j - 1, k)];
    const double etaT = in->eta_t[g], etaB = in->eta_t[G(i, j, k - 1)];
    double Fep = ee * (1.0 - etaE) / RhoCell, Fem = ee * etaE / RhoCell;
    double Fwp = ew * etaW / RhoCell, Fwm = ew * (1.0 - etaW) / RhoCell;
    double Fnp = en * (1.0 - etaN) / RhoCell, Fnm = en * etaN / RhoCell;
    double Fsp = es * etaS / RhoCell, Fsm = es * (1.0 - etaS) / RhoCell;
    double Ftp = et * (1.0 - etaT) / RhoCell, Ftm = et * etaT / RhoCell;
    double Fbp = eb * etaB / RhoCell, Fbm = eb * (1.0 - etaB) / RhoCell;
    /* boundary faces (PredictUVW.f90:939-1009): Neumann drops the face,
     * Dirichlet scales it by the half-cell factor of the component */
    if (i == 1) {
        if (in->bc_flag[0] == 1) { Dfw = 0.0; Fwp = 0.0; Fwm = 0.0; }
        else { Dfw = Dfw * CoefEW; Fwp = Fwp * CoefEW; Fwm = Fwm * CoefEW; }
    }
    if (i == ie) {
        if (in->bc_flag[1] == 1) { Dfe = 0.0; Fep = 0.0; Fem = 0.0; }
        else { Dfe = Dfe * CoefEW; Fep = Fep * CoefEW; Fem = Fem * CoefEW; }
    }
    if (j == 1) {
        if (in->bc_flag[2] == 1) { Dfs = 0.0; Fsp = 0.0; Fsm = 0.0; }
        else { Dfs = Dfs * CoefNS; Fsp = Fsp * CoefNS; Fsm = Fsm * CoefNS; }
    }
    if (j == je) {
        if (in->bc_flag[3] == 1) { Dfn = 0.0; Fnp = 0.0; Fnm = 0.0; }
        else { Dfn = Dfn * CoefNS; Fnp = Fnp * CoefNS; Fnm = Fnm * CoefNS; }
    }
    if (k == 1) {
        if (in->bc_flag[4] == 1) { Dfb = 0.0; Fbp = 0.0; Fbm = 0.0; }
        else { Dfb = Dfb * CoefTB; Fbp = Fbp * CoefTB; Fbm = Fbm * CoefTB; }
    }
    if (k == ke) {
        if (in->bc_flag[5] == 1) { Dft = 0.0; Ftp = 0.0; Ftm = 0.0; }
        else { Dft = Dft * CoefTB; Ftp = Ftp * CoefTB; Ftm = Ftm * CoefTB; }
    }
    MomRow r;
    double aE = Dfe, aW = Dfw, aN = Dfn, aS = Dfs, aT = Dft, aB = Dfb;
    /* CWE/CSN/CBT (1011-1016): the boundary coefficients before the
     * cut-cell terms, used by SetVectors */
    const double cw = aW, ce = aE, cs = aS, cn = aN, cb = aB, ct = aT;
    const double dx = in->grid_dx[n], dy = in->grid_dy[n], dz = in->grid_dz[n];
    double aP = vof * dx * dy * dz / o->dt + aE + aW + aN + aS + aT + aB + in->fric[n];
    aP = aP + Fep - Fwp + Fnp - Fsp + Ftp - Fbp;
    aE = aE - Fem;
    aW = aW + Fwm;
    aN = aN - Fnm;
    aS = aS + Fsm;
    aT = aT - Ftm;
    aB = aB + Fbm;
    const double dp0 = 1.0 / (aP - aE - aW - aN - aS - aT - aB);
    r.aw = aW; r.as = aS; r.ab = aB; r.ap = aP; r.ae = aE; r.an = aN; r.at = aT;
    /* SetVectors (1211-1251); the component's own velocity is iu*u+iv*v+iw*w
     * (+0.0 turns a -0 into +0 as the reference's sum with the 0*v terms
     * does for finite v, w) */
    const double U = in->tvar[g] + 0.0;
    const double vo = in->vof_old[g];
    const double G3 = o->gx * (double)iu + o->gy * (double)iv + o->gz * (double)iw;
    double rhs = U * vof * dx * dy * dz / o->dt - U * (vof - vo) * dx * dy * dz / o->dt +
                 1.0 / (o->fr * o->fr) * vof * dx * dy * dz * G3 / o->g;
    r.dp = vof * dx * dy * dz * dp0;
    rhs = rhs - in->flux_div[n];
    if (i == 1) rhs = rhs + cw * in->bc_var[0][(size_t)(j - 1) + (size_t)J * (k - 1)];
    if (i == ie) rhs = rhs + ce * in->bc_var[1][(size_t)(j - 1) + (size_t)J * (k - 1)];
    if (j == 1) rhs = rhs + cs * in->bc_var[2][(size_t)(i - 1) + (size_t)I * (k - 1)];
    if (j == je) rhs = rhs + cn * in->bc_var[3][(size_t)(i - 1) + (size_t)I * (k - 1)];
    if (k == 1) rhs = rhs + cb * in->bc_var[4][(size_t)(i - 1) + (size_t)I * (j - 1)];
    if (k == ke) rhs = rhs + ct * in->bc_var[5][(size_t)(i - 1) + (size_t)I * (j - 1)];
    r.rhs = rhs;
    return r;
}

static int32_t posnu_at(const scf_mom_in *in, int comp, int i, int j, int k)
{
    const int ie = I - (comp == 1), je = J - (comp == 2);
    return in->posnu[(size_t)(i - 1) + (size_t)ie * ((size_t)(j - 1) + (size_t)je * (size_t)(k - 1))];
}

/* The system of one component as HYPRE receives it: CSR rows in PosNu
 * order (row ExtCell+1 rows), entries in the order W,S,B,P,E,N,T of the
 * existing ones (PredictUVW.f90:1044-1097), the rhs (SetVectors), and
 * PUVW%Dp on the loop range (zeroed first, 913).  rowptr has ExtCell+2
 * entries, cols/vals room for 7 per row.  Returns the number of entries, or
 * -1 when a row index is out of range or a row is set twice or not at all. */
long oracle_mom_system(int imax, int jmax, int kmax, int comp, const scf_mom_in *in, const scf_mom_opts *o,
                       int64_t *rowptr, int32_t *cols, double *vals, double *rhs, double *dp)
{
    I = imax; J = jmax; K = kmax;
    const int ie = I - (comp == 1), je = J - (comp == 2), ke = K - (comp == 3);
    const long nrow = (long)in->extcell + 1;
    int32_t *cnt = calloc((size_t)nrow, sizeof(int32_t));
    int32_t *c7 = malloc(sizeof(int32_t) * 7 * (size_t)nrow);
    double *v7 = malloc(sizeof(double) * 7 * (size_t)nrow);
    char *seen = calloc((size_t)nrow, 1);
    long bad = 0;
    for (int i = 1; i <= ie; ++i)
        for (int j = 1; j <= je; ++j)
            for (int k = 1; k <= ke; ++k) {
                dp[G(i, j, k)] = 0.0;
                if (in->cell_type[N(i, j, k)] == 2) continue;
                const MomRow r = mom_row(in, o, comp, i, j, k);
                const int32_t row = posnu_at(in, comp, i, j, k);
                if (row < 0 || row >= nrow || seen[row]) { bad = 1; continue; }
                seen[row] = 1;
                dp[G(i, j, k)] = r.dp;
                rhs[row] = r.rhs;
                int m = 0;
                int32_t *cc = c7 + 7 * (size_t)row;
                double *vv = v7 + 7 * (size_t)row;
#define NB(cond, ii, jj, kk, val)                                            \
    if (cond) {                                                              \
        const int32_t q = posnu_at(in, comp, ii, jj, kk);                    \
        if (q != -1) { cc[m] = q; vv[m] = -(val); ++m; }                     \
    }
                NB(i > 1, i - 1, j, k, r.aw)
                NB(j > 1, i, j - 1, k, r.as)
                NB(k > 1, i, j, k - 1, r.ab)
                cc[m] = row; vv[m] = r.ap; ++m;
                NB(i < ie, i + 1, j, k, r.ae)
                NB(j < je, i, j + 1, k, r.an)
                NB(k < ke, i, j, k + 1, r.at)
#undef NB
                cnt[row] = m;
            }
    for (long r = 0; r < nrow; ++r)
        if (!seen[r]) bad = 1;
    long nnz = 0;
    rowptr[0] = 0;
    for (long r = 0; r < nrow; ++r) {
        for (int m = 0; m < cnt[r]; ++m) {
            cols[nnz] = c7[7 * r + m];
            vals[nnz] = v7[7 * r + m];
            ++nnz;
        }
        rowptr[r + 1] = nnz;
    }
    free(cnt); free(c7); free(v7); free(seen);
    return bad ? -1 : nnz;
}

static double dot(long n, const double *a, const double *b)
{
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

static void csr_mv(long n, const int64_t *rp, const int32_t *ci, const double *va, const double *x, double *y)
{
#pragma omp parallel for schedule(static)
    for (long r = 0; r < n; ++r) {
        double s = 0.0;
        for (int64_t q = rp[r]; q < rp[r + 1]; ++q) s += va[q] * x[ci[q]];
        y[r] = s;
    }
}

/* Jacobi-preconditioned BiCGStab (van der Vorst 1992) on a CSR system from
 * x = 0, to ||b - A x|| <= tol ||b|| (true residual, checked on
 * convergence of the recursive one).  Returns the iterations, or -1. */
int oracle_csr_bicgstab(long n, const int64_t *rp, const int32_t *ci, const double *va, const double *b, double *x,
                        double tol, int maxit, double *relres)
{
    double *dinv = malloc(sizeof(double) * n), *r = malloc(sizeof(double) * n), *r0 = malloc(sizeof(double) * n);
    double *p = malloc(sizeof(double) * n), *v = malloc(sizeof(double) * n), *s = malloc(sizeof(double) * n);
    double *t = malloc(sizeof(double) * n), *ph = malloc(sizeof(double) * n), *sh = malloc(sizeof(double) * n);
    for (long i = 0; i < n; ++i) {
        double d = 0.0;
        for (int64_t q = rp[i]; q < rp[i + 1]; ++q)
            if (ci[q] == i) d = va[q];
        dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
        x[i] = 0.0;
        r[i] = b[i]; r0[i] = b[i]; p[i] = 0.0; v[i] = 0.0;
    }
    const double bn = sqrt(dot(n, b, b));
    int it = 0, done = bn == 0.0;
    double rho = 1.0, alpha = 1.0, omega = 1.0, res = 0.0;
    while (!done && it < maxit) {
        const double rho1 = dot(n, r0, r);
        if (rho1 == 0.0) break;
        const double beta = (rho1 / rho) * (alpha / omega);
        rho = rho1;
        for (long i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
        for (long i = 0; i < n; ++i) ph[i] = dinv[i] * p[i];
        csr_mv(n, rp, ci, va, ph, v);
        alpha = rho / dot(n, r0, v);
        for (long i = 0; i < n; ++i) s[i] = r[i] - alpha * v[i];
        for (long i = 0; i < n; ++i) sh[i] = dinv[i] * s[i];
        csr_mv(n, rp, ci, va, sh, t);
        const double tt = dot(n, t, t);
        omega = tt > 0.0 ? dot(n, t, s) / tt : 0.0;
        for (long i = 0; i < n; ++i) {
            x[i] += alpha * ph[i] + omega * sh[i];
            r[i] = s[i] - omega * t[i];
        }
        ++it;
        if (sqrt(dot(n, r, r)) <= tol * bn || omega == 0.0) {
            csr_mv(n, rp, ci, va, x, t);
            for (long i = 0; i < n; ++i) t[i] = b[i] - t[i];
            res = sqrt(dot(n, t, t)) / bn;
            if (res <= tol) done = 1;
            else {   /* restart from the true residual */
                for (long i = 0; i < n; ++i) { r[i] = t[i]; r0[i] = t[i]; p[i] = 0.0; v[i] = 0.0; }
                rho = alpha = omega = 1.0;
            }
        }
    }
    if (relres) *relres = bn == 0.0 ? 0.0 : res;
    free(dinv); free(r); free(r0); free(p); free(v); free(s); free(t); free(ph); free(sh);
    return done ? it : -1;
}

/* DeltaGetValues (PredictUVW.f90:1294-1336): walks the loop range with a
 * running row counter; a cell whose PosNu equals the counter takes x and
 * advances it, every other cell gets 0.                                    */
void oracle_mom_get_values(int imax, int jmax, int kmax, int comp, const scf_mom_in *in, const double *x, double *var)
{
    I = imax; J = jmax; K = kmax;
    const int ie = I - (comp == 1), je = J - (comp == 2), ke = K - (comp == 3);
    int32_t ctr = 0;
    for (int i = 1; i <= ie; ++i)
        for (int j = 1; j <= je; ++j)
            for (int k = 1; k <= ke; ++k) {
                if (posnu_at(in, comp, i, j, k) == ctr) {
                    var[G(i, j, k)] = x[ctr];
                    ++ctr;
                } else {
                    var[G(i, j, k)] = 0.0;
                }
            }
}

/* The tail of PredictingUVW (PredictUVW.f90:766-802): Dp ghost planes of
 * PU, PV, PW copied plane by plane in the reference's order, then
 * PredictorVelocityBoundaryCondition (3796-3894) and
 * PredictorVelocityInternalCellCondition (3896-3914).                       */
void oracle_predict_tail(int imax, int jmax, int kmax, const scf_mom_in in[3], double *pu, double *pv, double *pw,
                         double *dpu, double *dpv, double *dpw)
{
    I = imax; J = jmax; K = kmax;
#define PLANE_I(a, dst, src) \
    for (int k = 0; k <= K + 1; ++k) for (int j = 0; j <= J + 1; ++j) a[G(dst, j, k)] = a[G(src, j, k)];
#define PLANE_J(a, dst, src) \
    for (int k = 0; k <= K + 1; ++k) for (int i = 0; i <= I + 1; ++i) a[G(i, dst, k)] = a[G(i, src, k)];
#define PLANE_K(a, dst, src) \
    for (int j = 0; j <= J + 1; ++j) for (int i = 0; i <= I + 1; ++i) a[G(i, j, dst)] = a[G(i, j, src)];
    PLANE_I(dpu, 0, 1) PLANE_I(dpu, I, I - 1) PLANE_I(dpu, I + 1, I)
    PLANE_J(dpu, 0, 1) PLANE_J(dpu, J + 1, J) PLANE_K(dpu, 0, 1) PLANE_K(dpu, K + 1, K)
    PLANE_I(dpv, 0, 1) PLANE_I(dpv, I + 1, I) PLANE_J(dpv, 0, 1) PLANE_J(dpv, J, J - 1)
    PLANE_J(dpv, J + 1, J) PLANE_K(dpv, 0, 1) PLANE_K(dpv, K + 1, K)
    PLANE_I(dpw, 0, 1) PLANE_I(dpw, I + 1, I) PLANE_J(dpw, 0, 1) PLANE_J(dpw, J + 1, J)
    PLANE_K(dpw, 0, 1) PLANE_K(dpw, K, K - 1) PLANE_K(dpw, K + 1, K)
#undef PLANE_I
#undef PLANE_J
#undef PLANE_K
    for (int j = 1; j <= J; ++j)
        for (int k = 1; k <= K; ++k) {
            pu[G(0, j, k)] = in[0].bc_flag[0] == 1 ? pu[G(1, j, k)] : in[0].bc_var[0][(size_t)(j - 1) + (size_t)J * (k - 1)];
            const double ve = in[0].bc_var[1][(size_t)(j - 1) + (size_t)J * (k - 1)];
            pu[G(I, j, k)] = in[0].bc_flag[1] == 1 ? pu[G(I - 1, j, k)] : ve;
            pu[G(I + 1, j, k)] = 2.0 * ve - pu[G(I - 1, j, k)];
        }
    for (int i = 1; i <= I; ++i)
        for (int k = 1; k <= K; ++k) {
            pv[G(i, 0, k)] = in[1].bc_flag[2] == 1 ? pv[G(i, 1, k)] : in[1].bc_var[2][(size_t)(i - 1) + (size_t)I * (k - 1)];
            const double vn = in[1].bc_var[3][(size_t)(i - 1) + (size_t)I * (k - 1)];
            pv[G(i, J, k)] = in[1].bc_flag[3] == 1 ? pv[G(i, J - 1, k)] : vn;
            pv[G(i, J + 1, k)] = 2.0 * vn - pv[G(i, J - 1, k)];
        }
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j) {
            pw[G(i, j, 0)] = in[2].bc_flag[4] == 1 ? pw[G(i, j, 1)] : in[2].bc_var[4][(size_t)(i - 1) + (size_t)I * (j - 1)];
            const double vt = in[2].bc_var[5][(size_t)(i - 1) + (size_t)I * (j - 1)];
            pw[G(i, j, K)] = in[2].bc_flag[5] == 1 ? pw[G(i, j, K - 1)] : vt;
            pw[G(i, j, K + 1)] = 2.0 * vt - pw[G(i, j, K - 1)];
        }
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                if (in[0].cell_type[N(i, j, k)] == 2) pu[G(i, j, k)] = 0.0;
                if (in[1].cell_type[N(i, j, k)] == 2) pv[G(i, j, k)] = 0.0;
                if (in[2].cell_type[N(i, j, k)] == 2) pw[G(i, j, k)] = 0.0;
            }
}
