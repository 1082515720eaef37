/*
 * oracle.c -- CPU restatement of SIMCOFlow's pressure-projection path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA library
 * and the timed CPU baseline of the benchmark; nothing in the product links
 * or calls it.  Parity status: the reference (Fortran + MPI + HYPRE) cannot
 * be built on this machine (no Fortran compiler, no MPI, no HYPRE), and its
 * own tests hold no golden values for this path, so this restatement is
 * pinned by the known-answer tests in tests/ (exact discrete eigenmodes,
 * a stratified column with a closed-form GFM solution, symmetry and
 * conservation invariants), not by reference outputs.
 *
 * Each function names the reference lines it restates.  Loops keep the
 * reference's order (i outer, k innermost) wherever the order changes the
 * result (the stale BetaW/BetaD of Compute1DGFMCoefficient, the sequential
 * boundary conditions).  Build with -ffp-contract=off so that results do not
 * depend on the host's fused multiply-add.
 *
 * Indexing: ghosted arrays (0:I+1,0:J+1,0:K+1) column-major; interior arrays
 * (1:I,1:J,1:K).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/scf_projection.h"

#define GI(i, j, k) ((size_t)(i) + (size_t)(I + 2) * ((size_t)(j) + (size_t)(J + 2) * (size_t)(k)))
#define NI(i, j, k) ((size_t)((i) - 1) + (size_t)I * ((size_t)((j) - 1) + (size_t)J * (size_t)((k) - 1)))
#define PCF(i, j, k, f) (NI(i, j, k) + (size_t)I * J * K * (size_t)((f) - 1))

typedef struct {
    int I, J, K;
} dims_t;

/* ------------------------------------------------------------------------ */
/* Compute1DGFMCoefficient (ProjectionP.f90:123-265), all six calls of
 * PoissonEquationSolver (ProjectionP.f90:53-64).                            */
static int is_wet(double vofl, double vof, double phil, double epsi)
{
    return (vofl >= 0.5 && vof > 1.0 - epsi) || (phil < 0.0 && vof <= 1.0 - epsi && vof > epsi);
}
static int is_dry(double vofl, double vof, double phil, double epsi)
{
    return (vofl < 0.5 && vof > 1.0 - epsi) || (phil >= 0.0 && vof <= 1.0 - epsi && vof > epsi);
}

int oracle_pocoef(int I, int J, int K, const scf_poisson_in *in, double rho_l, double rho_g,
                  double rho_ref, double epsi, double tol, double stale_init, double *pocoef)
{
    const double betap = 1.0 / (rho_l / rho_ref);
    const double betam = 1.0 / (rho_g / rho_ref);
    for (int f = 1; f <= 6; ++f) {
        int ium = f == 1, jvm = f == 2, kwm = f == 3, iup = f == 4, jvp = f == 5, kwp = f == 6;
        const double *dp = (f == 1 || f == 4) ? in->pu_dp : (f == 2 || f == 5) ? in->pv_dp : in->pw_dp;
        const double *dg = (f == 1 || f == 4) ? in->ugrid_dx : (f == 2 || f == 5) ? in->vgrid_dy : in->wgrid_dz;
        double betaw = stale_init, betad = stale_init;
        for (int k = 1; k <= K; ++k)
            for (int j = 1; j <= J; ++j)
                for (int i = 1; i <= I; ++i) pocoef[PCF(i, j, k, f)] = 0.0;
        for (int i = 1; i <= I; ++i)
            for (int j = 1; j <= J; ++j)
                for (int k = 1; k <= K; ++k) {
                    int ii = i - ium + iup, jj = j - jvm + jvp, kk = k - kwm + kwp;
                    int im = i - ium, jm = j - jvm, km = k - kwm;
                    int a = im < 1 ? 1 : im, b = jm < 1 ? 1 : jm, c = km < 1 ? 1 : km;
                    double dgrid = dg[NI(a, b, c)];
                    size_t gc = GI(i, j, k), gn = GI(ii, jj, kk);
                    double pc = fabs(in->pcell_phil[gc]), pn = fabs(in->pcell_phil[gn]);
                    double lamda = pc / (pc + pn + tol);
                    double vlc = in->pcell_vofl[gc], vc = in->pcell_vof[gc], phc = in->pcell_phil[gc];
                    double vln = in->pcell_vofl[gn], vn = in->pcell_vof[gn], phn = in->pcell_phil[gn];
                    double dpv = dp[GI(im, jm, km)];
                    if (is_wet(vlc, vc, phc, epsi)) {
                        if (is_dry(vln, vn, phn, epsi))
                            betaw = lamda * betam + (1.0 - lamda) * betap;
                        else if (is_wet(vln, vn, phn, epsi))
                            betaw = betam;
                        pocoef[PCF(i, j, k, f)] = dpv / dgrid * betap * betam / betaw;
                    } else if (is_dry(vlc, vc, phc, epsi)) {
                        if (is_wet(vln, vn, phn, epsi))
                            betad = lamda * betap + (1.0 - lamda) * betam;
                        else if (is_dry(vln, vn, phn, epsi))
                            betad = betap;
                        pocoef[PCF(i, j, k, f)] = dpv / dgrid * betap * betam / betad;
                    }
                }
        /* boundary planes copy their neighbour plane (ProjectionP.f90:256-264) */
        if (ium || iup) {
            int dst = ium ? 1 : I, src = ium ? 2 : I - 1;
            for (int k = 1; k <= K; ++k)
                for (int j = 1; j <= J; ++j) pocoef[PCF(dst, j, k, f)] = pocoef[PCF(src, j, k, f)];
        }
        if (jvm || jvp) {
            int dst = jvm ? 1 : J, src = jvm ? 2 : J - 1;
            for (int k = 1; k <= K; ++k)
                for (int i = 1; i <= I; ++i) pocoef[PCF(i, dst, k, f)] = pocoef[PCF(i, src, k, f)];
        }
        if (kwm || kwp) {
            int dst = kwm ? 1 : K, src = kwm ? 2 : K - 1;
            for (int j = 1; j <= J; ++j)
                for (int i = 1; i <= I; ++i) pocoef[PCF(i, j, dst, f)] = pocoef[PCF(i, j, src, f)];
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* SetPoissonMatrix (ProjectionP.f90:301-482) as CSR in PosNu row order.
 * Entries of a row are stored in the reference's order W,S,B,diag,E,N,T.
 * Returns the number of rows that fail the reference's diagonal-dominance
 * check (the rows on which the reference halts with `pause`, 463-474).      */
int64_t oracle_matrix_csr(int I, int J, int K, const scf_poisson_in *in, const double *pocoef,
                          int64_t *rowptr, int32_t *cols, double *vals)
{
    const int WB = in->bcp_flag[0], EB = in->bcp_flag[1], SB = in->bcp_flag[2];
    const int NB = in->bcp_flag[3], BB = in->bcp_flag[4], TB = in->bcp_flag[5];
    const int32_t *pos = in->pcell_posnu, *ct = in->pcell_cell_type;
    const double *EE = in->pcell_eearea, *NE = in->pcell_nearea, *TE = in->pcell_tearea;
    int64_t nnz_total = 0, bad = 0;
    int32_t nrow = in->pcell_extcell + 1;
    /* rows are filled in loop order; PosNu numbers them in the same order */
    int64_t *rowlen = (int64_t *)calloc((size_t)nrow, sizeof(int64_t));
    int32_t *tcols = (int32_t *)malloc((size_t)nrow * 7 * sizeof(int32_t));
    double *tvals = (double *)malloc((size_t)nrow * 7 * sizeof(double));
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                if (ct[NI(i, j, k)] == 2) continue;
                double dx = in->pgrid_dx[NI(i, j, k)], dy = in->pgrid_dy[NI(i, j, k)], dz = in->pgrid_dz[NI(i, j, k)];
                int32_t ictr = pos[NI(i, j, k)];
                int nnz = 0;
                int32_t c[7];
                double v[7];
                double mp1 = 0, mp2 = 0, mp3 = 0, mp4 = 0, mp5 = 0, mp6 = 0, mp;
                const double p1 = pocoef[PCF(i, j, k, 1)], p2 = pocoef[PCF(i, j, k, 2)], p3 = pocoef[PCF(i, j, k, 3)];
                const double p4 = pocoef[PCF(i, j, k, 4)], p5 = pocoef[PCF(i, j, k, 5)], p6 = pocoef[PCF(i, j, k, 6)];
                if (i > 1 && pos[NI(i - 1, j, k)] != -1) {
                    c[nnz] = pos[NI(i - 1, j, k)];
                    v[nnz] = -p1 * EE[GI(i - 1, j, k)] * dy * dz;
                    mp1 = fabs(v[nnz]);
                    nnz++;
                }
                if (j > 1 && pos[NI(i, j - 1, k)] != -1) {
                    c[nnz] = pos[NI(i, j - 1, k)];
                    v[nnz] = -p2 * NE[GI(i, j - 1, k)] * dx * dz;
                    mp2 = fabs(v[nnz]);
                    nnz++;
                }
                if (k > 1 && pos[NI(i, j, k - 1)] != -1) {
                    c[nnz] = pos[NI(i, j, k - 1)];
                    v[nnz] = -p3 * TE[GI(i, j, k - 1)] * dx * dy;
                    mp3 = fabs(v[nnz]);
                    nnz++;
                }
                c[nnz] = ictr;
                v[nnz] = p1 * EE[GI(i - 1, j, k)] * dy * dz + p2 * NE[GI(i, j - 1, k)] * dx * dz +
                         p3 * TE[GI(i, j, k - 1)] * dx * dy + p4 * EE[GI(i, j, k)] * dy * dz +
                         p5 * NE[GI(i, j, k)] * dx * dz + p6 * TE[GI(i, j, k)] * dx * dy;
                mp = fabs(v[nnz]);
                if (WB == 1 && i == 1) v[nnz] = v[nnz] - p1 * EE[GI(i - 1, j, k)] * dy * dz;
                if (SB == 1 && j == 1) v[nnz] = v[nnz] - p2 * NE[GI(i, j - 1, k)] * dx * dz;
                if (BB == 1 && k == 1) v[nnz] = v[nnz] - p3 * TE[GI(i, j, k - 1)] * dx * dy;
                if (EB == 1 && i == I) v[nnz] = v[nnz] - p4 * EE[GI(i, j, k)] * dy * dz;
                if (NB == 1 && j == J) v[nnz] = v[nnz] - p5 * NE[GI(i, j, k)] * dx * dz;
                if (TB == 1 && k == K) v[nnz] = v[nnz] - p6 * TE[GI(i, j, k)] * dx * dy;
                nnz++;
                if (i < I && pos[NI(i + 1, j, k)] != -1) {
                    c[nnz] = pos[NI(i + 1, j, k)];
                    v[nnz] = -p4 * EE[GI(i, j, k)] * dy * dz;
                    mp4 = fabs(v[nnz]);
                    nnz++;
                }
                if (j < J && pos[NI(i, j + 1, k)] != -1) {
                    c[nnz] = pos[NI(i, j + 1, k)];
                    v[nnz] = -p5 * NE[GI(i, j, k)] * dx * dz;
                    mp5 = fabs(v[nnz]);
                    nnz++;
                }
                if (k < K && pos[NI(i, j, k + 1)] != -1) {
                    c[nnz] = pos[NI(i, j, k + 1)];
                    v[nnz] = -p6 * TE[GI(i, j, k)] * dx * dy;
                    mp6 = fabs(v[nnz]);
                    nnz++;
                }
                if (ictr < 0 || ictr >= nrow) { free(rowlen); free(tcols); free(tvals); return -1; }
                rowlen[ictr] = nnz;
                memcpy(tcols + (size_t)ictr * 7, c, sizeof(int32_t) * nnz);
                memcpy(tvals + (size_t)ictr * 7, v, sizeof(double) * nnz);
                if (mp < mp1 + mp2 + mp3 + mp4 + mp5 + mp6 && i > 1 && j > 1 && k > 1) bad++;
            }
    rowptr[0] = 0;
    for (int32_t r = 0; r < nrow; ++r) {
        for (int64_t e = 0; e < rowlen[r]; ++e) {
            cols[nnz_total] = tcols[(size_t)r * 7 + e];
            vals[nnz_total] = tvals[(size_t)r * 7 + e];
            nnz_total++;
        }
        rowptr[r + 1] = nnz_total;
    }
    free(rowlen);
    free(tcols);
    free(tvals);
    return bad;
}

/* SetPoissonVectors (ProjectionP.f90:484-576): b in PosNu order. */
int oracle_rhs(int I, int J, int K, const scf_poisson_in *in, const double *pocoef, double *rhs)
{
    const double *u = in->pred_u, *v = in->pred_v, *w = in->pred_w;
    const double *EE = in->pcell_eearea, *NE = in->pcell_nearea, *TE = in->pcell_tearea;
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                if (in->pcell_cell_type[NI(i, j, k)] == 2) continue;
                double dx = in->pgrid_dx[NI(i, j, k)], dy = in->pgrid_dy[NI(i, j, k)], dz = in->pgrid_dz[NI(i, j, k)];
                int32_t ictr = in->pcell_posnu[NI(i, j, k)];
                double r = -dy * dz * (EE[GI(i, j, k)] * u[GI(i, j, k)] - EE[GI(i - 1, j, k)] * u[GI(i - 1, j, k)])
                           - dx * dz * (NE[GI(i, j, k)] * v[GI(i, j, k)] - NE[GI(i, j - 1, k)] * v[GI(i, j - 1, k)])
                           - dx * dy * (TE[GI(i, j, k)] * w[GI(i, j, k)] - TE[GI(i, j, k - 1)] * w[GI(i, j, k - 1)]);
                r = r + (in->pcell_vof[GI(i, j, k)] - in->vof_old[GI(i, j, k)]) * dx * dy * dz / in->dt;
                if (in->bcp_flag[0] == 0 && i == 1) r = r + pocoef[PCF(i, j, k, 1)] * in->bcp_var[0][(j - 1) + (size_t)J * (k - 1)];
                if (in->bcp_flag[1] == 0 && i == I) r = r + pocoef[PCF(i, j, k, 4)] * in->bcp_var[1][(j - 1) + (size_t)J * (k - 1)];
                if (in->bcp_flag[2] == 0 && j == 1) r = r + pocoef[PCF(i, j, k, 2)] * in->bcp_var[2][(i - 1) + (size_t)I * (k - 1)];
                if (in->bcp_flag[3] == 0 && j == J) r = r + pocoef[PCF(i, j, k, 5)] * in->bcp_var[3][(i - 1) + (size_t)I * (k - 1)];
                if (in->bcp_flag[4] == 0 && k == 1) r = r + pocoef[PCF(i, j, k, 3)] * in->bcp_var[4][(i - 1) + (size_t)I * (j - 1)];
                if (in->bcp_flag[5] == 0 && k == K) r = r + pocoef[PCF(i, j, k, 6)] * in->bcp_var[5][(i - 1) + (size_t)I * (j - 1)];
                rhs[ictr] = r;
            }
    return 0;
}

/* DeltaPressureGetValues + DeltaPressureBoundaryCondition
 * (ProjectionP.f90:578-643).  pp: ghosted, entries the reference does not
 * write are left as given.                                                 */
int oracle_scatter(int I, int J, int K, const scf_poisson_in *in, const double *x, double *pp)
{
    int32_t ctr = 0;
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                if (in->pcell_posnu[NI(i, j, k)] == ctr) {
                    pp[GI(i, j, k)] = x[ctr];
                    ctr++;
                } else {
                    pp[GI(i, j, k)] = 0.0;
                }
            }
    const int *f = in->bcp_flag;
    for (int j = 1; j <= J; ++j)
        for (int k = 1; k <= K; ++k) {
            pp[GI(0, j, k)] = (double)f[0] * pp[GI(1, j, k)];
            pp[GI(I + 1, j, k)] = (double)f[1] * pp[GI(I, j, k)];
        }
    for (int i = 1; i <= I; ++i)
        for (int k = 1; k <= K; ++k) {
            pp[GI(i, 0, k)] = (double)f[2] * pp[GI(i, 1, k)];
            pp[GI(i, J + 1, k)] = (double)f[3] * pp[GI(i, J, k)];
        }
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j) {
            pp[GI(i, j, 0)] = (double)f[4] * pp[GI(i, j, 1)];
            pp[GI(i, j, K + 1)] = (double)f[5] * pp[GI(i, j, K)];
        }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Velocity correction, BoundaryConditionVarNew and the Dirichlet-face mass
 * correction (ComputePUVW.f90:179-384,418-708; TypicalBC from
 * BoundaryFunction.f90:760-781).                                           */

/* Field plane accessors mirroring the Fortran sections passed as uin etc.:
 * a ghosted plane section X(ip,:,:) has lower bound 1 inside TypicalBC, so
 * Varin(a,b) = X(ip, a-1, b-1).                                             */
typedef struct {
    int I, J, K;
} shp_t;

static double *plane_ptr_x(double *F, int I, int J, int K, int ip, int a, int b) { return &F[GI(ip, a, b)]; }

/* TypicalBC with the reference's argument conventions.
 * face: 0..5 (W,E,S,N,B,T).  src: index of the plane section passed as the
 * field argument (e.g. 1 for u(1,:,:), Imax-1 for u(Imax-1,:,:)).
 * dscale: factor on the spacing (dxin, -dxin*2, ...).  d: PGrid%dx/dy/dz.   */
static void typical_bc(int I, int J, int K, int face, const double *F, int src, double dscale, int flag,
                       double cst, const double *d, double *var)
{
    if (face <= 1) { /* x-face: Var(J,K), d = dx(plane,:,:) */
        int pl = face == 0 ? 1 : I;
        for (int k = 1; k <= K; ++k)
            for (int j = 1; j <= J; ++j) {
                double val;
                if (flag == 0) val = cst;
                else val = F[GI(src, j - 1, k - 1)] - cst * (dscale * d[NI(pl, j, k)]) / 2.0;
                var[(j - 1) + (size_t)J * (k - 1)] = val;
            }
    } else if (face <= 3) { /* y-face: Var(I,K) */
        int pl = face == 2 ? 1 : J;
        for (int k = 1; k <= K; ++k)
            for (int i = 1; i <= I; ++i) {
                double val;
                if (flag == 0) val = cst;
                else val = F[GI(i - 1, src, k - 1)] - cst * (dscale * d[NI(i, pl, k)]) / 2.0;
                var[(i - 1) + (size_t)I * (k - 1)] = val;
            }
    } else { /* z-face: Var(I,J) */
        int pl = face == 4 ? 1 : K;
        for (int j = 1; j <= J; ++j)
            for (int i = 1; i <= I; ++i) {
                double val;
                if (flag == 0) val = cst;
                else val = F[GI(i - 1, j - 1, src)] - cst * (dscale * d[NI(i, j, pl)]) / 2.0;
                var[(i - 1) + (size_t)I * (j - 1)] = val;
            }
    }
}

/* X(plane) = Var on the face's plane (interior in-plane range). */
static void set_plane(int I, int J, int K, int face, double *F, int pl, const double *var)
{
    if (face <= 1) {
        for (int k = 1; k <= K; ++k)
            for (int j = 1; j <= J; ++j) F[GI(pl, j, k)] = var[(j - 1) + (size_t)J * (k - 1)];
    } else if (face <= 3) {
        for (int k = 1; k <= K; ++k)
            for (int i = 1; i <= I; ++i) F[GI(i, pl, k)] = var[(i - 1) + (size_t)I * (k - 1)];
    } else {
        for (int j = 1; j <= J; ++j)
            for (int i = 1; i <= I; ++i) F[GI(i, j, pl)] = var[(i - 1) + (size_t)I * (j - 1)];
    }
}

/* ComputeGhostVarBoundary (ComputePUVW.f90:696-708): X(out) from X(in). */
static void ghost_plane(int I, int J, int K, int face, double *F, int pin, int pout, int flag, const double *var)
{
    if (face <= 1) {
        for (int k = 1; k <= K; ++k)
            for (int j = 1; j <= J; ++j) {
                double b = var[(j - 1) + (size_t)J * (k - 1)], x = F[GI(pin, j, k)];
                F[GI(pout, j, k)] = flag == 1 ? b - x : 2.0 * b - x;
            }
    } else if (face <= 3) {
        for (int k = 1; k <= K; ++k)
            for (int i = 1; i <= I; ++i) {
                double b = var[(i - 1) + (size_t)I * (k - 1)], x = F[GI(i, pin, k)];
                F[GI(i, pout, k)] = flag == 1 ? b - x : 2.0 * b - x;
            }
    } else {
        for (int j = 1; j <= J; ++j)
            for (int i = 1; i <= I; ++i) {
                double b = var[(i - 1) + (size_t)I * (j - 1)], x = F[GI(i, j, pin)];
                F[GI(i, j, pout)] = flag == 1 ? b - x : 2.0 * b - x;
            }
    }
}

/* BC step table of BoundaryConditionVarNew for one field.
 * For each face: source plane of the field argument, spacing factor,
 * whether Var is copied into the boundary plane (and which), and the ghost
 * plane written (if any).  Values from ComputePUVW.f90:431-692 and the
 * TypicalBC calls of BoundaryFunction.f90:83-511.                          */
typedef struct {
    int src;      /* plane index of the field section passed to the BC     */
    double dsc;   /* factor on dxin/dyin/dzin                              */
    int setpl;    /* plane set to Var, or -999                             */
    int gin, gout;/* ghost: from plane gin to gout, or gout = -999          */
} bcstep_t;

static void bc_table(int I, int J, int K, int field, bcstep_t t[6])
{
    const int NO = -999;
    /* defaults: sources at the boundary planes, ghost from the boundary plane */
    bcstep_t d[6] = {
        {1, 1.0, NO, 1, 0},     {I, -1.0, NO, I, I + 1}, {1, 1.0, NO, 1, 0},
        {J, -1.0, NO, J, J + 1}, {1, 1.0, NO, 1, 0},     {K, -1.0, NO, K, K + 1}};
    memcpy(t, d, sizeof(d));
    if (field == 0) { /* u */
        t[0].setpl = 0; t[0].gout = NO;            /* u(0,:,:) = VarW, no ghost  */
        t[1].src = I - 1; t[1].dsc = -2.0; t[1].setpl = I; /* u(I)=VarE; ghost I+1 */
        t[3].dsc = -1.0;
    } else if (field == 1) { /* v */
        t[1].dsc = -1.0;
        t[2].setpl = 0; t[2].gout = NO;            /* v(:,0,:) = VarS */
        t[3].src = J - 1; t[3].dsc = -2.0; t[3].setpl = J;
    } else if (field == 2) { /* w */
        t[4].setpl = 0; t[4].gout = NO;            /* w(:,:,0) = VarB */
        t[5].src = K - 1; t[5].dsc = -2.0; t[5].setpl = K;
    } else { /* p */
        t[5].setpl = K;                            /* p(:,:,K) = VarT, then ghost */
    }
}

int oracle_correct(int I, int J, int K, const scf_poisson_in *in, const scf_correct_in *cr,
                   const double *pocoef, const double *pp, double *u, double *v, double *w, double *p,
                   double *bcvar /* 4*6 planes, packed, may be NULL */, int north_mass_fix)
{
    /* correction loop (ComputePUVW.f90:181-232) */
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                size_t n = NI(i, j, k), g = GI(i, j, k);
                if (cr->ucell_moexcell[n] != 1 && cr->ucell_cell_type[n] != 2)
                    u[g] = in->pred_u[g] - (pp[GI(i + 1, j, k)] - pp[g]) * pocoef[PCF(i, j, k, 4)];
                else
                    u[g] = 0.0;
                if (cr->vcell_moexcell[n] != 1 && cr->vcell_cell_type[n] != 2)
                    v[g] = in->pred_v[g] - (pp[GI(i, j + 1, k)] - pp[g]) * pocoef[PCF(i, j, k, 5)];
                else
                    v[g] = 0.0;
                if (cr->wcell_moexcell[n] != 1 && cr->wcell_cell_type[n] != 2)
                    w[g] = in->pred_w[g] - (pp[GI(i, j, k + 1)] - pp[g]) * pocoef[PCF(i, j, k, 6)];
                else
                    w[g] = 0.0;
                p[g] = pp[g];
            }
    /* BoundaryConditionVarNew (ComputePUVW.f90:418-694) */
    double *fields[4] = {u, v, w, p};
    const int32_t *flags[4] = {cr->bcu_flag, cr->bcv_flag, cr->bcw_flag, in->bcp_flag};
    const double *consts[4] = {cr->bcu_const, cr->bcv_const, cr->bcw_const, cr->bcp_const};
    const double *dd[6] = {in->pgrid_dx, in->pgrid_dx, in->pgrid_dy, in->pgrid_dy, in->pgrid_dz, in->pgrid_dz};
    size_t planesz[6] = {(size_t)J * K, (size_t)J * K, (size_t)I * K, (size_t)I * K, (size_t)I * J, (size_t)I * J};
    size_t maxp = planesz[0];
    if (planesz[2] > maxp) maxp = planesz[2];
    if (planesz[4] > maxp) maxp = planesz[4];
    double *var = (double *)malloc(maxp * sizeof(double));
    size_t off = 0;
    for (int fld = 0; fld < 4; ++fld) {
        bcstep_t t[6];
        bc_table(I, J, K, fld, t);
        for (int face = 0; face < 6; ++face) {
            typical_bc(I, J, K, face, fields[fld], t[face].src, t[face].dsc, flags[fld][face],
                       consts[fld][face], dd[face], var);
            if (t[face].setpl != -999) set_plane(I, J, K, face, fields[fld], t[face].setpl, var);
            if (t[face].gout != -999)
                ghost_plane(I, J, K, face, fields[fld], t[face].gin, t[face].gout, flags[fld][face], var);
            if (bcvar) memcpy(bcvar + off, var, planesz[face] * sizeof(double));
            off += planesz[face];
        }
    }
    free(var);
    /* Dirichlet-face mass correction, first Dirichlet p face only
     * (ComputePUVW.f90:260-384).  Quirks kept: NEArea(i,j,k) on both y faces
     * of the west/east branches, TEArea(i,j,k) on both z faces, etc.        */
    const double *EE = in->pcell_eearea, *NE = in->pcell_nearea, *TE = in->pcell_tearea;
    const double *DX = in->pgrid_dx, *DY = in->pgrid_dy, *DZ = in->pgrid_dz;
    const int *f = in->bcp_flag;
    if (f[0] == 0) {
        int i = 1;
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                size_t n = NI(i, j, k), g = GI(i, j, k);
                u[GI(i - 1, j, k)] = (DX[n] * DZ[n] * (NE[g] * v[g] - NE[g] * v[GI(i, j - 1, k)]) +
                                      DX[n] * DY[n] * (TE[g] * w[g] - TE[g] * w[GI(i, j, k - 1)]) +
                                      DY[n] * DZ[n] * EE[g] * u[g]) / EE[g] / DY[n] / DZ[n];
            }
    } else if (f[1] == 0) {
        int i = I;
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                size_t n = NI(i, j, k), g = GI(i, j, k);
                u[g] = (DX[n] * DZ[n] * (-NE[g] * v[g] + NE[g] * v[GI(i, j - 1, k)]) +
                        DX[n] * DY[n] * (-TE[g] * w[g] + TE[g] * w[GI(i, j, k - 1)]) +
                        DY[n] * DZ[n] * EE[g] * u[GI(i - 1, j, k)]) / EE[g] / DY[n] / DZ[n];
            }
    } else if (f[2] == 0) {
        int j = 1;
        for (int i = 1; i <= I; ++i)
            for (int k = 1; k <= K; ++k) {
                size_t n = NI(i, j, k), g = GI(i, j, k);
                v[GI(i, j - 1, k)] = (DY[n] * DZ[n] * (EE[g] * u[g] - EE[g] * u[GI(i - 1, j, k)]) +
                                      DX[n] * DY[n] * (TE[g] * w[g] - TE[g] * w[GI(i, j, k - 1)]) +
                                      DX[n] * DZ[n] * NE[g] * v[g]) / NE[g] / DX[n] / DZ[n];
            }
    } else if (f[3] == 0) {
        if (!north_mass_fix) return SCF_ERR_UNDEFINED_IN_REFERENCE;
        int j = J;
        for (int i = 1; i <= I; ++i)
            for (int k = 1; k <= K; ++k) {
                size_t n = NI(i, j, k), g = GI(i, j, k);
                v[g] = (-DY[n] * DZ[n] * (EE[g] * u[g] - EE[g] * u[GI(i - 1, j, k)])
                        - DX[n] * DY[n] * (TE[g] * w[g] - TE[g] * w[GI(i, j, k - 1)]) +
                        DX[n] * DZ[n] * NE[g] * v[GI(i, j - 1, k)]) / NE[g] / DX[n] / DZ[n];
            }
    } else if (f[4] == 0) {
        int k = 1;
        for (int i = 1; i <= I; ++i)
            for (int j = 1; j <= J; ++j) {
                size_t n = NI(i, j, k), g = GI(i, j, k);
                w[GI(i, j, k - 1)] = (DY[n] * DZ[n] * (EE[g] * u[g] - EE[g] * u[GI(i - 1, j, k)]) +
                                      DX[n] * DZ[n] * (NE[g] * v[g] - NE[g] * v[GI(i, j - 1, k)]) +
                                      DX[n] * DY[n] * TE[g] * w[g]) / TE[g] / DX[n] / DY[n];
            }
    } else if (f[5] == 0) {
        int k = K;
        for (int i = 1; i <= I; ++i)
            for (int j = 1; j <= J; ++j) {
                size_t n = NI(i, j, k), g = GI(i, j, k);
                w[g] = (-DY[n] * DZ[n] * (EE[g] * u[g] - EE[g] * u[GI(i - 1, j, k)])
                        - DX[n] * DZ[n] * (NE[g] * v[g] - NE[g] * v[GI(i, j - 1, k)]) +
                        DX[n] * DY[n] * TE[g] * w[GI(i, j, k - 1)]) / TE[g] / DX[n] / DY[n];
            }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* CSR helpers: y = A x, and a Jacobi-preconditioned CG (the reference's
 * PCG with a simpler preconditioner; HYPRE is not available to restate
 * BoomerAMG).  Singular (all-Neumann) systems: b and every residual are
 * projected to zero mean and the zero-mean x is returned.                   */
void oracle_csr_apply(int32_t n, const int64_t *rp, const int32_t *ci, const double *va, const double *x, double *y)
{
#pragma omp parallel for schedule(static)
    for (int32_t r = 0; r < n; ++r) {
        double s = 0.0;
        for (int64_t e = rp[r]; e < rp[r + 1]; ++e) s += va[e] * x[ci[e]];
        y[r] = s;
    }
}

static double dotn(int32_t n, const double *a, const double *b)
{
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int32_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

static void remove_mean(int32_t n, double *a)
{
    double s = 0.0;
    for (int32_t i = 0; i < n; ++i) s += a[i];
    s /= (double)n;
    for (int32_t i = 0; i < n; ++i) a[i] -= s;
}

/* returns iterations (negative if not converged); *relres = true residual */
int oracle_csr_pcg(int32_t n, const int64_t *rp, const int32_t *ci, const double *va, const double *b_in,
                   double *x, double tol, int maxit, int singular, double *relres)
{
    double *b = (double *)malloc(sizeof(double) * n), *r = (double *)malloc(sizeof(double) * n);
    double *z = (double *)malloc(sizeof(double) * n), *p = (double *)malloc(sizeof(double) * n);
    double *q = (double *)malloc(sizeof(double) * n), *dinv = (double *)malloc(sizeof(double) * n);
    memcpy(b, b_in, sizeof(double) * n);
    if (singular) remove_mean(n, b);
    for (int32_t i = 0; i < n; ++i) {
        double d = 0.0;
        for (int64_t e = rp[i]; e < rp[i + 1]; ++e)
            if (ci[e] == i) d = va[e];
        dinv[i] = d != 0.0 ? 1.0 / d : 0.0;
        x[i] = 0.0;
    }
    double bn = sqrt(dotn(n, b, b));
    if (bn == 0.0) {
        *relres = 0.0;
        free(b); free(r); free(z); free(p); free(q); free(dinv);
        return 0;
    }
    memcpy(r, b, sizeof(double) * n);
    for (int32_t i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
    memcpy(p, z, sizeof(double) * n);
    double rz = dotn(n, r, z);
    int it;
    for (it = 1; it <= maxit; ++it) {
        oracle_csr_apply(n, rp, ci, va, p, q);
        double alpha = rz / dotn(n, p, q);
        for (int32_t i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        if (singular) remove_mean(n, r);
        double rn = sqrt(dotn(n, r, r));
        if (rn <= tol * bn) break;
        for (int32_t i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
        double rz2 = dotn(n, r, z);
        double beta = rz2 / rz;
        rz = rz2;
        for (int32_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
    if (singular) remove_mean(n, x);
    oracle_csr_apply(n, rp, ci, va, x, q);
    double s = 0.0;
    for (int32_t i = 0; i < n; ++i) s += (b[i] - q[i]) * (b[i] - q[i]);
    *relres = sqrt(s) / bn;
    free(b); free(r); free(z); free(p); free(q); free(dinv);
    return it <= maxit ? it : -maxit;
}

/* ||b - A x|| / ||b|| with the literal CSR matrix; singular: b projected. */
double oracle_csr_relres(int32_t n, const int64_t *rp, const int32_t *ci, const double *va, const double *b_in,
                         const double *x, int singular)
{
    double *b = (double *)malloc(sizeof(double) * n), *q = (double *)malloc(sizeof(double) * n);
    memcpy(b, b_in, sizeof(double) * n);
    if (singular) remove_mean(n, b);
    oracle_csr_apply(n, rp, ci, va, x, q);
    double s = 0.0, t = 0.0;
    for (int32_t i = 0; i < n; ++i) {
        s += (b[i] - q[i]) * (b[i] - q[i]);
        t += b[i] * b[i];
    }
    free(b);
    free(q);
    return t > 0 ? sqrt(s / t) : sqrt(s);
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
