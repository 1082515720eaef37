/*
 * clsvof.c -- CPU restatement of the first pieces of SIMCOFlow's CLSVOF
 * module (src/Clsvof.f90): ComputeUVWLiquidField, which derives the liquid
 * fraction and level set of the U, V, W cells from the pressure cells after
 * each interface advection (called from src/Solver.f90:209);
 * Interface_Reconstruct, the normals and plane distances every sweep of
 * Clsvof_Scheme starts from; and the directional sweeps X_Sweep, Y_Sweep,
 * Z_Sweep with their geometric face fluxes, which advance the liquid
 * fraction and the level set along one axis.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for a future GPU restatement;
 * nothing in the product links or calls it.  Parity status: the reference
 * (Fortran) cannot be built on this machine and its tests hold no golden
 * values for these routines, so the restatement is pinned by known-answer
 * tests in tests/ (a horizontal interface seen by the U cells, the direction
 * averages written through the reference's index shift, a planar interface
 * reconstructed exactly, Find_Distance inverting Volume_Fraction_Calc, a
 * plane carried exactly by each sweep, the liquid of every line conserved
 * up to its wall fluxes, closed forms of the sweeps' boundary faces) and
 * by an independent vectorised restatement of Volume_Fraction_Calc
 * (simcoflow3d_gb300/workloads.py volume_fraction_calc), not by reference
 * outputs.  Newton_Raphson is capped at 200 steps (the reference loops
 * without a cap).
 *
 * Loops and expressions keep the reference's order; built with
 * -ffp-contract=off.  Fortran x**2.d0 is x*x (gfortran folds it exactly) and
 * x**3.d0 is pow(x, 3.0) (gfortran calls pow for it).
 *
 * Quirks of the reference kept as they are:
 *  - DirectionAverageArray (Clsvof.f90:328-353) writes through an
 *    assumed-shape dummy, which Fortran numbers from 1, while the velocity
 *    cells' phiL/nxL/nyL/nzL are allocated (0:I+1,0:J+1,0:K+1): the average
 *    of P cells (i, i+iu) lands in VelCell(i-1, j-1, k-1).
 *  - The V cells' left half uses the whole dy and phiL itself (not the
 *    shifted level set) for the corner distance (Clsvof.f90:231-236); their
 *    right half starts from phiL(i,j,k) with the normal of (i,j+1,k) and a
 *    plus sign (242-244).
 *  - The W cells' right half shifts the level set by +dz/2 (268-269) where
 *    the U cells' shifts by -dx/2 (208-209).
 *  - ComputeVelocityCellLiquidField's clamp of vof + vofL <= 1 (314-322)
 *    acts on the previous vofL, which the loops then overwrite.
 *
 * Indexing (column-major, i fastest): ghosted (0:I+1,0:J+1,0:K+1), interior
 * (1:I,1:J,1:K).
 */
#include <math.h>
#include <stddef.h>

static int I, J, K;
#define G(i, j, k) ((size_t)(i) + (size_t)(I + 2) * ((size_t)(j) + (size_t)(J + 2) * (size_t)(k)))
#define N(i, j, k) ((size_t)((i) - 1) + (size_t)I * ((size_t)((j) - 1) + (size_t)J * (size_t)((k) - 1)))

static double max3(double a, double b, double c)
{
    double m = a > b ? a : b;
    return m > c ? m : c;
}
static double min3(double a, double b, double c)
{
    double m = a < b ? a : b;
    return m < c ? m : c;
}

/* Volume_Fraction_Calc (Clsvof.f90:1475-1550): the volume of the dx*dy*dz
 * box on the positive side of the plane at distance s from the corner along
 * the normal (nxx, nyy, nzz) -- the Griebel-Klitz formula.                 */
double oracle_volume_fraction_calc(double dx, double dy, double dz, double nxx, double nyy, double nzz, double s)
{
    const double nx1 = fabs(nxx), ny1 = fabs(nyy), nz1 = fabs(nzz);
    const double dx1 = max3(nx1 * dx, ny1 * dy, nz1 * dz);
    const double dz1 = min3(nx1 * dx, ny1 * dy, nz1 * dz);
    const double dy1 = nx1 * dx + ny1 * dy + nz1 * dz - dx1 - dz1;
    const double sm = dx1 + dy1 + dz1;
    const double sc = s < sm - s ? s : sm - s;
    double fc;
    if (s <= 0.0) return 0.0;
    if (s >= sm) return 1.0 * dx * dy * dz;
    if (sc <= dz1) {
        fc = pow(sc, 3.0) / (6.0 * dx1 * dy1 * dz1);
    } else if (sc <= dy1) {
        fc = (sc * sc - dz1 * sc + dz1 * dz1 / 3.0) / (2.0 * dx1 * dy1);
    } else if (dx1 >= dy1 + dz1) {
        if (sc >= dy1 + dz1) {
            fc = (2.0 * sc - dy1 - dz1) / (2.0 * dx1);
        } else {
            fc = pow(sc, 3.0) - pow(sc - dz1, 3.0) - pow(sc - dy1, 3.0);
            fc = fc / (6.0 * dx1 * dy1 * dz1);
        }
    } else {
        if (sc > dx1)
            fc = pow(sc, 3.0) - pow(sc - dz1, 3.0) - pow(sc - dy1, 3.0) - pow(sc - dx1, 3.0);
        else
            fc = pow(sc, 3.0) - pow(sc - dz1, 3.0) - pow(sc - dy1, 3.0);
        fc = fc / (6.0 * dx1 * dy1 * dz1);
    }
    if (s <= 0.5 * sm) return fc * dx * dy * dz;
    return (1.0 - fc) * dx * dy * dz;
}

/* ConvertTheCoordinateSystem (Clsvof.f90:2458-2465): the level set measured
 * from the box's corner instead of its centre.                             */
double oracle_convert_coord(double dx, double dy, double dz, double nx, double ny, double nz, double phi)
{
    return phi + 0.5 * (fabs(nx) * dx + fabs(ny) * dy + fabs(nz) * dz);
}

/* DirectionAverageArray (Clsvof.f90:328-353) with the reference's index
 * shift of the output (see the header).  d: the P grid's spacing along the
 * averaged axis (interior), in: the P cell field (ghosted), out: the
 * velocity cell field (ghosted).                                            */
static void direction_average(const double *d, const double *in, double *out, int iu, int iv, int iw)
{
    for (int i = 1; i <= I - iu; ++i)
        for (int j = 1; j <= J - iv; ++j)
            for (int k = 1; k <= K - iw; ++k) {
                const double lamda = d[N(i + iu, j + iv, k + iw)] / (d[N(i, j, k)] + d[N(i + iu, j + iv, k + iw)]);
                out[G(i - 1, j - 1, k - 1)] = lamda * in[G(i, j, k)] + (1.0 - lamda) * in[G(i + iu, j + iv, k + iw)];
            }
    if (iu == 1)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) out[G(I - 1, j - 1, k - 1)] = out[G(I - 2, j - 1, k - 1)];
    if (iv == 1)
        for (int i = 1; i <= I; ++i)
            for (int k = 1; k <= K; ++k) out[G(i - 1, J - 1, k - 1)] = out[G(i - 1, J - 2, k - 1)];
    if (iw == 1)
        for (int i = 1; i <= I; ++i)
            for (int j = 1; j <= J; ++j) out[G(i - 1, j - 1, K - 1)] = out[G(i - 1, j - 1, K - 2)];
}

/* One velocity family's liquid fields: the four direction averages, then
 * the clamp of ComputeVelocityCellLiquidField (Clsvof.f90:300-326).        */
static void velocity_cell_liquid_field(const double *d, const double *pphil, const double *pnxl, const double *pnyl,
                                       const double *pnzl, double *vphil, double *vnxl, double *vnyl, double *vnzl,
                                       double *vvofl, const double *vvof, int iu, int iv, int iw)
{
    direction_average(d, pphil, vphil, iu, iv, iw);
    direction_average(d, pnxl, vnxl, iu, iv, iw);
    direction_average(d, pnyl, vnyl, iu, iv, iw);
    direction_average(d, pnzl, vnzl, iu, iv, iw);
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k)
                if (vvof[G(i, j, k)] + vvofl[G(i, j, k)] > 1.0) vvofl[G(i, j, k)] = 1.0 - vvof[G(i, j, k)];
}

/* ComputeUVWLiquidField (Clsvof.f90:174-298).  P grid spacings and the U,
 * V, W grid spacings are interior arrays; the P cell's phiL, nxL, nyL, nzL,
 * vofL and the velocity cells' arrays are ghosted.  vel_* point to the
 * three families u, v, w in that order ([3] arrays of pointers); vel_phil,
 * vel_nxl, vel_nyl, vel_nzl and vel_vofl are updated in place.             */
void oracle_uvw_liquid_field(int imax, int jmax, int kmax, const double *pdx, const double *pdy, const double *pdz,
                             const double *phil, const double *nxl, const double *nyl, const double *nzl,
                             const double *vofl, const double *const vdx[3], const double *const vdy[3],
                             const double *const vdz[3], double *const vel_phil[3], double *const vel_nxl[3],
                             double *const vel_nyl[3], double *const vel_nzl[3], double *const vel_vofl[3],
                             const double *const vel_vof[3])
{
    I = imax; J = jmax; K = kmax;
    double dcell, phinew, dist, left, right;
    /* U cells */
    velocity_cell_liquid_field(pdx, phil, nxl, nyl, nzl, vel_phil[0], vel_nxl[0], vel_nyl[0], vel_nzl[0],
                               vel_vofl[0], vel_vof[0], 1, 0, 0);
    for (int j = 1; j <= J; ++j)
        for (int k = 1; k <= K; ++k) {
            for (int i = 1; i <= I - 1; ++i) {
                const size_t a = G(i, j, k), b = G(i + 1, j, k), na = N(i, j, k), nb = N(i + 1, j, k);
                dcell = pdx[na] / 2.0;
                phinew = phil[a] + dcell * nxl[a];
                dist = oracle_convert_coord(dcell, pdy[na], pdz[na], nxl[a], nyl[a], nzl[a], phinew);
                left = oracle_volume_fraction_calc(dcell, pdy[na], pdz[na], nxl[a], nyl[a], nzl[a], dist);
                left = dcell * pdy[na] * pdz[na] - left;
                dcell = pdx[nb] / 2.0;
                phinew = phil[b] - dcell * nxl[b];
                dist = oracle_convert_coord(dcell, pdy[nb], pdz[nb], nxl[b], nyl[b], nzl[b], phinew);
                right = oracle_volume_fraction_calc(dcell, pdy[nb], pdz[nb], nxl[b], nyl[b], nzl[b], dist);
                right = dcell * pdy[nb] * pdz[nb] - right;
                vel_vofl[0][a] = (left + right) / vdx[0][na] / vdy[0][na] / vdz[0][na];
            }
            vel_vofl[0][G(I, j, k)] = vofl[G(I, j, k)];
        }
    /* V cells */
    velocity_cell_liquid_field(pdy, phil, nxl, nyl, nzl, vel_phil[1], vel_nxl[1], vel_nyl[1], vel_nzl[1],
                               vel_vofl[1], vel_vof[1], 0, 1, 0);
    for (int i = 1; i <= I; ++i)
        for (int k = 1; k <= K; ++k) {
            for (int j = 1; j <= J - 1; ++j) {
                const size_t a = G(i, j, k), b = G(i, j + 1, k), na = N(i, j, k), nb = N(i, j + 1, k);
                dcell = pdy[na] / 2.0;
                phinew = phil[a] + dcell * nyl[a];   /* computed and not used, as in the reference */
                (void)phinew;
                dist = oracle_convert_coord(pdx[na], pdy[na], pdz[na], nxl[a], nyl[a], nzl[a], phil[a]);
                left = oracle_volume_fraction_calc(pdx[na], dcell, pdz[na], nxl[a], nyl[a], nzl[a], dist);
                left = pdx[na] * dcell * pdz[na] - left;
                dcell = pdy[nb] / 2.0;
                phinew = phil[a] + dcell * nyl[b];
                dist = oracle_convert_coord(pdx[nb], dcell, pdz[nb], nxl[b], nyl[b], nzl[b], phinew);
                right = oracle_volume_fraction_calc(pdx[nb], dcell, pdz[nb], nxl[b], nyl[b], nzl[b], dist);
                right = pdx[nb] * dcell * pdz[nb] - right;
                vel_vofl[1][a] = (left + right) / vdx[1][na] / vdy[1][na] / vdz[1][na];
            }
            vel_vofl[1][G(i, J, k)] = vofl[G(i, J, k)];
        }
    /* W cells */
    velocity_cell_liquid_field(pdz, phil, nxl, nyl, nzl, vel_phil[2], vel_nxl[2], vel_nyl[2], vel_nzl[2],
                               vel_vofl[2], vel_vof[2], 0, 0, 1);
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j) {
            for (int k = 1; k <= K - 1; ++k) {
                const size_t a = G(i, j, k), b = G(i, j, k + 1), na = N(i, j, k), nb = N(i, j, k + 1);
                dcell = pdz[na] / 2.0;
                phinew = phil[a] + dcell * nzl[a];
                dist = oracle_convert_coord(pdx[na], pdy[na], dcell, nxl[a], nyl[a], nzl[a], phinew);
                left = oracle_volume_fraction_calc(pdx[na], pdy[na], dcell, nxl[a], nyl[a], nzl[a], dist);
                left = pdx[na] * pdy[na] * dcell - left;
                dcell = pdz[nb] / 2.0;
                phinew = phil[b] + dcell * nzl[b];
                dist = oracle_convert_coord(pdx[nb], pdy[nb], dcell, nxl[b], nyl[b], nzl[b], phinew);
                right = oracle_volume_fraction_calc(pdx[nb], pdy[nb], dcell, nxl[b], nyl[b], nzl[b], dist);
                right = pdx[nb] * pdy[nb] * dcell - right;
                vel_vofl[2][a] = (left + right) / vdx[2][na] / vdy[2][na] / vdz[2][na];
            }
            vel_vofl[2][G(i, j, K)] = vofl[G(i, j, K)];
        }
}

/* ---- interface reconstruction (Clsvof.f90:801-815, 1216-1473, 2361-2456) -- */

static const double VOFEPS = 1.0e-14;   /* Clsvof.f90:32 */
static const double ETA = 0.075;        /* Clsvof.f90:32 */
static const double TOLPAR = 1.0e-14;   /* Clsvof.f90:35 */

/* Newton_Raphson (Clsvof.f90:1462-1473) on a3 s^3 + a2 s^2 + a1 s + a0.  The
 * reference loops until the step is below 1e-6 |s|; here at most 200 steps
 * (the reference has no cap).                                              */
static double newton_raphson(double a3, double a2, double a1, double a0, double sc)
{
    const double tol = 1.0e-6;
    double delvar = 1.0e6;
    for (int it = 0; it < 200 && fabs(delvar) > tol * fabs(sc); ++it) {
        delvar = (a3 * pow(sc, 3.0) + a2 * (sc * sc) + a1 * sc + a0) / (3.0 * a3 * (sc * sc) + 2.0 * a2 * sc + a1);
        sc = sc - delvar;
    }
    return sc;
}

/* Cubic_Equation_Solve (1380-1398); case2 selects the first form.          */
static double cubic_solve(double fc, double dx1, double dy1, double dz1, double sc, int case2)
{
    if (case2)
        return newton_raphson(1.0, -3.0 * (dy1 + dz1), 3.0 * (dy1 * dy1 + dz1 * dz1),
                              6.0 * fc * dx1 * dy1 * dz1 - (pow(dy1, 3.0) + pow(dz1, 3.0)), sc);
    return newton_raphson(2.0, -3.0 * (dx1 + dy1 + dz1), 3.0 * (dx1 * dx1 + dy1 * dy1 + dz1 * dz1),
                          6.0 * fc * dx1 * dy1 * dz1 - (pow(dx1, 3.0) + pow(dy1, 3.0) + pow(dz1, 3.0)), sc);
}

static double final_distance(double f, double sc, double sm) { return f <= 0.5 ? sc : sm - sc; }

/* Find_Distance (1311-1378): the distance s from the box's corner along
 * the normal at which the plane cuts the liquid fraction f off the box.    */
double oracle_find_distance(double dx, double dy, double dz, double nxx, double nyy, double nzz, double f)
{
    const double nx1 = fabs(nxx), ny1 = fabs(nyy), nz1 = fabs(nzz);
    const double dx1 = max3(nx1 * dx, ny1 * dy, nz1 * dz);
    double dz1 = min3(nx1 * dx, ny1 * dy, nz1 * dz);
    if (fabs(dz1) < TOLPAR) dz1 = 0.0;
    double dy1 = nx1 * dx + ny1 * dy + nz1 * dz - dx1 - dz1;
    if (fabs(dy1) < TOLPAR) dy1 = 0.0;
    const double fc = f < 1.0 - f ? f : 1.0 - f;
    const double sm = dx1 + dy1 + dz1;
    double sc = 6.0 * fc * dx1 * dy1 * dz1;
    sc = copysign(1.0, sc) * pow(fabs(sc), 1.0 / 3.0);
    if (sc < dz1) return final_distance(f, sc, sm);
    sc = 0.5 * dz1 + sqrt(2.0 * fc * dx1 * dy1 - dz1 * dz1 / 12.0);
    if (sc < dy1) return final_distance(f, sc, sm);
    if (dx1 >= dy1 + dz1) {
        sc = fc * dx1 + (dy1 + dz1) / 2.0;
        if (sc >= dy1 + dz1) return final_distance(f, sc, sm);
        sc = cubic_solve(fc, dx1, dy1, dz1, sc, 1);
        return final_distance(f, sc, sm);
    }
    sc = fc * dx1 + (dy1 + dz1) / 2.0;
    if (sc >= dx1) {
        sc = cubic_solve(fc, dx1, dy1, dz1, sc, 0);
        if (sc < dx1) sc = cubic_solve(fc, dx1, dy1, dz1, sc, 1);
        return final_distance(f, sc, sm);
    }
    sc = cubic_solve(fc, dx1, dy1, dz1, sc, 1);
    return final_distance(f, sc, sm);
}

/* Isinterface (801-815): a partly filled cell, or a full/empty cell next to
 * its opposite.  vfl ghosted.                                              */
static int is_interface(const double *vfl, int i, int j, int k)
{
    const double v = vfl[G(i, j, k)];
    const double jump = 1.0 - 2.1 * VOFEPS;
    int flag = v > VOFEPS && v < 1.0 - VOFEPS;
    if (fabs(vfl[G(i - 1, j, k)] - v) >= jump) flag = 1;
    if (fabs(vfl[G(i + 1, j, k)] - v) >= jump) flag = 1;
    if (fabs(vfl[G(i, j - 1, k)] - v) >= jump) flag = 1;
    if (fabs(vfl[G(i, j + 1, k)] - v) >= jump) flag = 1;
    if (fabs(vfl[G(i, j, k - 1)] - v) >= jump) flag = 1;
    if (fabs(vfl[G(i, j, k + 1)] - v) >= jump) flag = 1;
    return flag;
}

/* Normal_Vector_Irre (2361-2456): per direction, a one-sided difference of
 * phi towards the side whose neighbour has |grad phi| within ETA of 1 when
 * the other side's does not, else the central difference.  x, y, z: cell
 * centres (interior arrays); phi ghosted; only called with 1 < i < I etc. */
static void normal_vector_irre(const double *x, const double *y, const double *z, const double *phi, int i, int j,
                               int k, double *nxx, double *nyy, double *nzz)
{
#define P(a, b, c) phi[G(a, b, c)]
#define X(a, b, c) x[N(a, b, c)]
#define Y(a, b, c) y[N(a, b, c)]
#define Z(a, b, c) z[N(a, b, c)]
    double vx, vy, vz, qm, qp;
    int dx, dy, dz;
    if (i >= 3) vx = (P(i, j, k) - P(i - 2, j, k)) / (X(i, j, k) - X(i - 2, j, k));
    else vx = (P(i, j, k) - P(i - 1, j, k)) / (X(i, j, k) - X(i - 1, j, k));
    vy = (P(i - 1, j + 1, k) - P(i - 1, j - 1, k)) / (Y(i - 1, j + 1, k) - Y(i - 1, j - 1, k));
    vz = (P(i - 1, j, k + 1) - P(i - 1, j, k - 1)) / (Z(i - 1, j, k + 1) - Z(i - 1, j, k - 1));
    qm = fabs(1.0 - sqrt(vx * vx + vy * vy + vz * vz));
    if (i <= I - 2) vx = (P(i + 2, j, k) - P(i, j, k)) / (X(i + 2, j, k) - X(i, j, k));
    else vx = (P(i + 1, j, k) - P(i, j, k)) / (X(i + 1, j, k) - X(i, j, k));
    vy = (P(i + 1, j + 1, k) - P(i + 1, j - 1, k)) / (Y(i + 1, j + 1, k) - Y(i + 1, j - 1, k));
    vz = (P(i + 1, j, k + 1) - P(i + 1, j, k - 1)) / (Z(i + 1, j, k + 1) - Z(i + 1, j, k - 1));
    qp = fabs(1.0 - sqrt(vx * vx + vy * vy + vz * vz));
    dx = (qm < ETA && qp >= ETA) ? -1 : (qm >= ETA && qp < ETA) ? 1 : 0;
    if (j >= 3) vy = (P(i, j, k) - P(i, j - 2, k)) / (Y(i, j, k) - Y(i, j - 2, k));
    else vy = (P(i, j, k) - P(i, j - 1, k)) / (Y(i, j, k) - Y(i, j - 1, k));
    vx = (P(i + 1, j - 1, k) - P(i - 1, j - 1, k)) / (X(i + 1, j - 1, k) - X(i - 1, j - 1, k));
    vz = (P(i, j - 1, k + 1) - P(i, j - 1, k - 1)) / (Z(i, j - 1, k + 1) - Z(i, j - 1, k - 1));
    qm = fabs(1.0 - sqrt(vx * vx + vy * vy + vz * vz));
    vx = (P(i + 1, j + 1, k) - P(i - 1, j + 1, k)) / (X(i + 1, j + 1, k) - X(i - 1, j + 1, k));
    if (j <= J - 2) vy = (P(i, j + 2, k) - P(i, j, k)) / (Y(i, j + 2, k) - Y(i, j, k));
    else vy = (P(i, j + 1, k) - P(i, j, k)) / (Y(i, j + 1, k) - Y(i, j, k));
    vz = (P(i, j + 1, k + 1) - P(i, j + 1, k - 1)) / (Z(i, j + 1, k + 1) - Z(i, j + 1, k - 1));
    qp = fabs(1.0 - sqrt(vx * vx + vy * vy + vz * vz));
    dy = (qm < ETA && qp >= ETA) ? -1 : (qm >= ETA && qp < ETA) ? 1 : 0;
    vx = (P(i + 1, j, k - 1) - P(i - 1, j, k - 1)) / (X(i + 1, j, k - 1) - X(i - 1, j, k - 1));
    vy = (P(i, j + 1, k - 1) - P(i, j - 1, k - 1)) / (Y(i, j + 1, k - 1) - Y(i, j - 1, k - 1));
    if (k >= 3) vz = (P(i, j, k) - P(i, j, k - 2)) / (Z(i, j, k) - Z(i, j, k - 2));
    else vz = (P(i, j, k) - P(i, j, k - 1)) / (Z(i, j, k) - Z(i, j, k - 1));
    qm = fabs(1.0 - sqrt(vx * vx + vy * vy + vz * vz));
    vx = (P(i + 1, j, k + 1) - P(i - 1, j, k + 1)) / (X(i + 1, j, k + 1) - X(i - 1, j, k + 1));
    vy = (P(i, j + 1, k + 1) - P(i, j - 1, k + 1)) / (Y(i, j + 1, k + 1) - Y(i, j - 1, k + 1));
    if (k <= K - 2) vz = (P(i, j, k + 2) - P(i, j, k)) / (Z(i, j, k + 2) - Z(i, j, k));
    else vz = (P(i, j, k + 1) - P(i, j, k)) / (Z(i, j, k + 1) - Z(i, j, k));
    qp = fabs(1.0 - sqrt(vx * vx + vy * vy + vz * vz));
    dz = (qm < ETA && qp >= ETA) ? -1 : (qm >= ETA && qp < ETA) ? 1 : 0;
    if (dx == -1) *nxx = (P(i, j, k) - P(i - 1, j, k)) / (X(i, j, k) - X(i - 1, j, k));
    if (dx == 1) *nxx = (P(i + 1, j, k) - P(i, j, k)) / (X(i + 1, j, k) - X(i, j, k));
    if (dx == 0) *nxx = (P(i + 1, j, k) - P(i - 1, j, k)) / (X(i + 1, j, k) - X(i - 1, j, k));
    if (dy == -1) *nyy = (P(i, j, k) - P(i, j - 1, k)) / (Y(i, j, k) - Y(i, j - 1, k));
    if (dy == 1) *nyy = (P(i, j + 1, k) - P(i, j, k)) / (Y(i, j + 1, k) - Y(i, j, k));
    if (dy == 0) *nyy = (P(i, j + 1, k) - P(i, j - 1, k)) / (Y(i, j + 1, k) - Y(i, j - 1, k));
    if (dz == -1) *nzz = (P(i, j, k) - P(i, j, k - 1)) / (Z(i, j, k) - Z(i, j, k - 1));
    if (dz == 1) *nzz = (P(i, j, k + 1) - P(i, j, k)) / (Z(i, j, k + 1) - Z(i, j, k));
    if (dz == 0) *nzz = (P(i, j, k + 1) - P(i, j, k - 1)) / (Z(i, j, k + 1) - Z(i, j, k - 1));
#undef P
#undef X
#undef Y
#undef Z
}

/* Interface_Reconstruct (1216-1309): for every interface cell the unit
 * normal of phi (Normal_Vector_Irre inside, clamped central differences
 * near the walls, +z when the gradient vanishes) and Find_Distance of its
 * liquid fraction; every other cell gets 0.  x, y, z, dx, dy, dz interior;
 * vfl, phi, nxx, nyy, nzz, diss ghosted (nxx, nyy, nzz zeroed whole first,
 * diss written on the interior only).                                      */
void oracle_interface_reconstruct(int imax, int jmax, int kmax, const double *x, const double *y, const double *z,
                                  const double *dx, const double *dy, const double *dz, const double *vfl,
                                  const double *phi, double *nxx, double *nyy, double *nzz, double *diss)
{
    I = imax; J = jmax; K = kmax;
    const size_t ng = (size_t)(I + 2) * (J + 2) * (K + 2);
    for (size_t q = 0; q < ng; ++q) nxx[q] = nyy[q] = nzz[q] = 0.0;
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                double n1 = 0.0, n2 = 0.0, n3 = 0.0, d1 = 0.0;
                if (is_interface(vfl, i, j, k)) {
                    if (i > 1 && i < I && j > 1 && j < J && k > 1 && k < K) {
                        normal_vector_irre(x, y, z, phi, i, j, k, &n1, &n2, &n3);
                    } else {
                        const int ip = i + 1 < I ? i + 1 : I, im = i - 1 > 1 ? i - 1 : 1;
                        const int jp = j + 1 < J ? j + 1 : J, jm = j - 1 > 1 ? j - 1 : 1;
                        const int kp = k + 1 < K ? k + 1 : K, km = k - 1 > 1 ? k - 1 : 1;
                        n1 = (phi[G(ip, j, k)] - phi[G(im, j, k)]) / (x[N(ip, j, k)] - x[N(im, j, k)]);
                        n2 = (phi[G(i, jp, k)] - phi[G(i, jm, k)]) / (y[N(i, jp, k)] - y[N(i, jm, k)]);
                        n3 = (phi[G(i, j, kp)] - phi[G(i, j, km)]) / (z[N(i, j, kp)] - z[N(i, j, km)]);
                    }
                    const double temp = sqrt(n1 * n1 + n2 * n2 + n3 * n3);
                    if (temp < 1.0e-14) {
                        n1 = 0.0; n2 = 0.0; n3 = 1.0;
                    } else {
                        n1 = n1 / temp; n2 = n2 / temp; n3 = n3 / temp;
                    }
                    d1 = oracle_find_distance(dx[N(i, j, k)], dy[N(i, j, k)], dz[N(i, j, k)], n1, n2, n3,
                                              vfl[G(i, j, k)]);
                }
                nxx[G(i, j, k)] = n1;
                nyy[G(i, j, k)] = n2;
                nzz[G(i, j, k)] = n3;
                diss[G(i, j, k)] = d1;
            }
}

/* ---- the directional sweeps (Clsvof.f90:817-1214, fluxes 1553-1688) ------ */

/* East_Flux / West_Flux / North_Flux / South_Flux / Top_Flux / Bottom_Flux
 * (1553-1688) in one: the liquid volume per unit face area that crosses the
 * face in one step, from the cell upstream.  axis 0/1/2 = x/y/z; side +1
 * the east/north/top face (the plane's normal component <= 0 takes the
 * slab next to the face), -1 the west/south/bottom face (>= 0 does).      */
static double face_flux(int axis, int side, double nxx, double nyy, double nzz, double diss, double volf, double dx,
                        double dy, double dz, double wdt)
{
    if (wdt == 0.0) return 0.0;
    const double nn = axis == 0 ? nxx : axis == 1 ? nyy : nzz;
    const int thin = side > 0 ? nn <= 0.0 : nn >= 0.0;
    double flux;
    if (axis == 0) {
        if (thin) flux = oracle_volume_fraction_calc(wdt, dy, dz, nxx, nyy, nzz, diss) / (wdt * dy * dz);
        else flux = (volf * dx * dy * dz - oracle_volume_fraction_calc(dx - wdt, dy, dz, nxx, nyy, nzz, diss)) /
                    (wdt * dy * dz);
    } else if (axis == 1) {
        if (thin) flux = oracle_volume_fraction_calc(dx, wdt, dz, nxx, nyy, nzz, diss) / (dx * wdt * dz);
        else flux = (volf * dx * dy * dz - oracle_volume_fraction_calc(dx, dy - wdt, dz, nxx, nyy, nzz, diss)) /
                    (dx * wdt * dz);
    } else {
        if (thin) flux = oracle_volume_fraction_calc(dx, dy, wdt, nxx, nyy, nzz, diss) / (dx * dy * wdt);
        else flux = (volf * dx * dy * dz - oracle_volume_fraction_calc(dx, dy, dz - wdt, nxx, nyy, nzz, diss)) /
                    (dx * dy * wdt);
    }
    return flux * wdt;
}

/* X_Sweep, Y_Sweep, Z_Sweep along `axis`, after Interface_Reconstruct:
 *   temvf -= the divergence of the geometric VOF fluxes (a full or empty
 *   upstream cell sends vfl*u*dt), temls -= the divergence of the level-set
 *   fluxes u*phi_face*dt, phi_face extrapolated half a step upstream.
 * Arrays ghosted except the spacings d* and the centres c* (interior).
 * vel: the velocity of the axis (ghosted; vel(i) at the + face of cell i,
 * vel(0) at the wall).  bc_vel, bc_lvs: the wall values at the - face
 * (BCu%VarW and BCLvs%VarW for x, the S and B planes for y and z).  Each
 * line along the axis is independent; within it the updates run in the
 * reference's order.  Quirks kept: the VOF branch tests vel > 0 for x and
 * y but vel >= 0 for z; at the first face, x's backward level-set
 * difference is (phi(3)-phi(1))/2*dx(2) and z's adds where x and y
 * subtract; at the last face z scales by dy where x and y use their own
 * spacing.  (The operand orders of the reference's flux products, ue*lse
 * against lsn*ve, are single commutative products and round the same.)    */
static void sweep(int axis, const double *dx, const double *dy, const double *dz, const double *cx, const double *cy,
                  const double *cz, const double *vfl, const double *phi, const double *nxx, const double *nyy,
                  const double *nzz, const double *diss, const double *vel, const double *bc_vel, const double *bc_lvs,
                  double dtv, double *temvf, double *temls)
{
    const int n = axis == 0 ? I : axis == 1 ? J : K;
    const int na = axis == 0 ? J : I, nb = axis == 2 ? J : K;
    const double *d = axis == 0 ? dx : axis == 1 ? dy : dz;
    const double *cc = axis == 0 ? cx : axis == 1 ? cy : cz;
    for (int a = 1; a <= na; ++a)
        for (int b = 1; b <= nb; ++b) {
            /* cell m of the line (a, b): x lines are (j, k), y lines (i, k),
             * z lines (i, j) */
#define CI(m) (axis == 0 ? (m) : a)
#define CJ(m) (axis == 1 ? (m) : (axis == 0 ? a : b))
#define CK(m) (axis == 2 ? (m) : b)
#define GP(m) G(CI(m), CJ(m), CK(m))
#define NP(m) N(CI(m), CJ(m), CK(m))
            /* VOF */
            for (int m = 1; m <= n - 1; ++m) {
                const size_t g0 = GP(m), g1 = GP(m + 1), n0 = NP(m), n1 = NP(m + 1);
                const double w = vel[g0];
                const int down = axis == 2 ? w >= 0.0 : w > 0.0;
                double flux;
                if (down) {
                    if (vfl[g0] >= 1.0 - VOFEPS || vfl[g0] <= VOFEPS) flux = vfl[g0] * w * dtv;
                    else flux = face_flux(axis, +1, nxx[g0], nyy[g0], nzz[g0], diss[g0], vfl[g0], dx[n0], dy[n0],
                                          dz[n0], w * dtv);
                } else {
                    if (vfl[g1] >= 1.0 - VOFEPS || vfl[g1] <= VOFEPS) flux = vfl[g1] * w * dtv;
                    else flux = -face_flux(axis, -1, nxx[g1], nyy[g1], nzz[g1], diss[g1], vfl[g1], dx[n1], dy[n1],
                                           dz[n1], -w * dtv);
                }
                temvf[g0] = temvf[g0] - flux / d[n0];
                temvf[g1] = temvf[g1] + flux / d[n1];
            }
            {
                const size_t g1 = GP(1), gn = GP(n);
                const size_t gw = G(axis == 0 ? 0 : CI(1), axis == 1 ? 0 : CJ(1), axis == 2 ? 0 : CK(1));
                double flux = vfl[g1] * vel[gw] * dtv;
                temvf[g1] = temvf[g1] + flux / d[NP(1)];
                flux = vfl[gn] * vel[gn] * dtv;
                temvf[gn] = temvf[gn] - flux / d[NP(n)];
            }
            /* level set, the faces between cells 2..n */
            for (int m = 2; m <= n - 1; ++m) {
                const double w = vel[GP(m)], dm = d[NP(m)];
                double ls;
                if (w >= 0.0)
                    ls = phi[GP(m)] + dm / 2.0 * (1.0 - w * dtv / dm) * (phi[GP(m + 1)] - phi[GP(m - 1)]) / (2.0 * dm);
                else if (m <= n - 2)
                    ls = phi[GP(m + 1)] - dm / 2.0 * (1.0 + w * dtv / dm) * (phi[GP(m + 2)] - phi[GP(m)]) / (2.0 * dm);
                else
                    ls = phi[GP(m + 1)] - dm / 2.0 * (1.0 + w * dtv / dm) * (phi[GP(m + 1)] - phi[GP(m)]) / dm;
                const double flux = w * ls * dtv;
                temls[GP(m)] = temls[GP(m)] - flux / d[NP(m)];
                temls[GP(m + 1)] = temls[GP(m + 1)] + flux / d[NP(m + 1)];
            }
            /* the face between cells 1 and 2, and the wall flux */
            {
                const double w = vel[GP(1)];
                double ls;
                if (w >= 0.0) {
                    const double den = axis == 0 ? d[NP(1)] : cc[NP(2)] - cc[NP(1)];
                    ls = phi[GP(1)] + d[NP(1)] / 2.0 * (1.0 - w * dtv / d[NP(1)]) * (phi[GP(2)] - phi[GP(1)]) / den;
                } else if (axis == 0) {
                    ls = phi[GP(2)] - d[NP(2)] / 2.0 * (1.0 + w * dtv / d[NP(2)]) * (phi[GP(3)] - phi[GP(1)]) / 2.0 *
                                          d[NP(2)];
                } else if (axis == 1) {
                    ls = phi[GP(2)] - d[NP(2)] / 2.0 * (1.0 + w * dtv / d[NP(2)]) * (phi[GP(3)] - phi[GP(1)]) /
                                          (cc[NP(3)] - cc[NP(1)]);
                } else {
                    ls = phi[GP(2)] + d[NP(2)] / 2.0 * (1.0 + w * dtv / d[NP(2)]) * (phi[GP(3)] - phi[GP(1)]) /
                                          (cc[NP(3)] - cc[NP(1)]);
                }
                double flux = ls * w * dtv;
                temls[GP(1)] = temls[GP(1)] - flux / d[NP(1)];
                temls[GP(2)] = temls[GP(2)] + flux / d[NP(2)];
                const size_t bw = (size_t)(a - 1) + (size_t)(axis == 0 ? J : I) * (size_t)(b - 1);
                flux = bc_vel[bw] * bc_lvs[bw] * dtv;
                temls[GP(1)] = temls[GP(1)] + flux / d[NP(1)];
            }
            /* the last face */
            {
                const double w = vel[GP(n)];
                double ls;
                if (w > 0.0) {
                    ls = phi[GP(n)] + d[NP(n)] / 2.0 * (1.0 - w * dtv / d[NP(n)]) * (phi[GP(n)] - phi[GP(n - 1)]) /
                                          (cc[NP(n)] - cc[NP(n - 1)]);
                } else {
                    const double scale = axis == 2 ? dy[NP(n - 1)] : d[NP(n - 1)];
                    ls = phi[GP(n)] - d[NP(n - 1)] / 2.0 * (1.0 + w * dtv / scale) * (phi[GP(n)] - phi[GP(n - 1)]) /
                                          (cc[NP(n)] - cc[NP(n - 1)]);
                }
                const double flux = ls * w * dtv;
                temls[GP(n)] = temls[GP(n)] - flux / d[NP(n)];
            }
#undef CI
#undef CJ
#undef CK
#undef GP
#undef NP
        }
}

/* One sweep as Clsvof_Scheme calls it: Interface_Reconstruct of vfl, phi
 * into the normals and distances, then the sweep of `axis` into temvf,
 * temls (which hold the copies of vfl, phi on entry).                      */
void oracle_clsvof_sweep(int imax, int jmax, int kmax, int axis, const double *x, const double *y, const double *z,
                         const double *dx, const double *dy, const double *dz, const double *vfl, const double *phi,
                         const double *vel, const double *bc_vel, const double *bc_lvs, double dtv, double *nxx,
                         double *nyy, double *nzz, double *diss, double *temvf, double *temls)
{
    oracle_interface_reconstruct(imax, jmax, kmax, x, y, z, dx, dy, dz, vfl, phi, nxx, nyy, nzz, diss);
    I = imax; J = jmax; K = kmax;
    sweep(axis, dx, dy, dz, x, y, z, vfl, phi, nxx, nyy, nzz, diss, vel, bc_vel, bc_lvs, dtv, temvf, temls);
}
