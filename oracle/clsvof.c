/*
 * clsvof.c -- CPU restatement of ComputeUVWLiquidField, the step of
 * SIMCOFlow's CLSVOF module (src/Clsvof.f90) that derives the liquid
 * fraction and level set of the U, V, W cells from the pressure cells after
 * each interface advection (called from src/Solver.f90:209).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for a future GPU restatement;
 * nothing in the product links or calls it.  Parity status: the reference
 * (Fortran) cannot be built on this machine and its tests hold no golden
 * values for this routine, so the restatement is pinned by known-answer
 * tests in tests/ (a horizontal interface seen by the U cells, the direction
 * averages written through the reference's index shift) and by an
 * independent vectorised restatement of Volume_Fraction_Calc
 * (simcoflow3d_gb300/workloads.py volume_fraction_calc), not by reference
 * outputs.
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
