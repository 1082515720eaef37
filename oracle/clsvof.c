/*
 * clsvof.c -- CPU restatement of the first pieces of SIMCOFlow's CLSVOF
 * module (src/Clsvof.f90): ComputeUVWLiquidField, which derives the liquid
 * fraction and level set of the U, V, W cells from the pressure cells after
 * each interface advection (called from src/Solver.f90:209);
 * Interface_Reconstruct, the normals and plane distances every sweep of
 * Clsvof_Scheme starts from; the directional sweeps X_Sweep, Y_Sweep,
 * Z_Sweep with their geometric face fluxes, which advance the liquid
 * fraction and the level set along one axis; BoundaryConditionLvsVof;
 * Redistance_Levelset; and Clsvof_Scheme itself, the six split sub-steps
 * of one time step.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for a future GPU restatement;
 * nothing in the product links or calls it.  Parity status: the reference
 * (Fortran) cannot be built on this machine and its tests hold no golden
 * values for these routines, so the restatement is pinned by known-answer
 * tests in tests/ (a horizontal interface seen by the U cells, the direction
 * averages written through the reference's index shift, a planar interface
 * reconstructed exactly, Find_Distance inverting Volume_Fraction_Calc, a
 * plane carried exactly by each sweep, the liquid of every line conserved
 * up to its wall fluxes, closed forms of the sweeps' boundary faces, a
 * plane carried through a whole step, a drop's volume kept in a shear) and
 * by independent restatements: a vectorised Volume_Fraction_Calc
 * (simcoflow3d_gb300/workloads.py volume_fraction_calc), a gather form of
 * Redistance_Levelset and a numpy BoundaryConditionLvsVof (tests/), which
 * the oracle matches bit for bit where the arithmetic is alike.  Not by
 * reference outputs.  Newton_Raphson is capped at 200 steps (the reference
 * loops without a cap).
 *
 * Loops and expressions keep the reference's order; built with
 * -ffp-contract=off.  Fortran x**2.d0 is x*x (gfortran folds it exactly).
 * x**3.d0 and x**(1.d0/3.d0) are the exact powers rounded once to nearest
 * (cube_rn, pow_third below).  gfortran calls the math library's pow for
 * both, which comes within a hair of that but, in glibc, falls on the wrong
 * side of a near-tie for about 0.08% of arguments (0.501 against 0.499 ulp,
 * checked with 300-bit arithmetic); the correctly rounded value is the one
 * every platform's reference build approximates, and the GPU reproduces it
 * bit for bit.
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
 *  - The sweeps' own quirks are listed above sweep(); Shortest_Point_2d's
 *    y-face case divides by |nzz| where it solves for x (2026), which can
 *    put band cells under their true distance; BoundaryConditionLvsVof
 *    builds the ghost level set from the fluid normals (PCell%nx, not
 *    nxL), the north ghost subtracting like the south (2142-2143).
 *
 * Indexing (column-major, i fastest): ghosted (0:I+1,0:J+1,0:K+1), interior
 * (1:I,1:J,1:K).
 */
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

static int I, J, K;

/* x**3 rounded once: x*x split exactly by an FMA, times x split again, one
 * rounding of the sum (Dekker's product; correct but for ties finer than
 * 2^-100 of the result).                                                   */
static double cube_rn(double x)
{
    const double p = x * x, e1 = fma(x, x, -p), c = p * x, e2 = fma(p, x, -c);
    return c + fma(e1, x, e2);
}

/* x**(1.d0/3.d0) = x**a with a = fl(1/3) = 1/3 - 2^-54/3, rounded once:
 * the cube root c refined by one Newton step on the residual x - c^3
 * (exact products by FMA), times x**(-2^-54/3) = 1 - (2^-54/3) ln x (the
 * next term is below 2^-90).  x > 0 finite; 0 and the rest go to pow.    */
static double pow_third(double x)
{
    if (!(x > 0.0) || isinf(x)) return pow(x, 1.0 / 3.0);
    const double c = cbrt(x);
    const double c2h = c * c, c2l = fma(c, c, -c2h);
    const double c3h = c2h * c, c3l = fma(c2h, c, -c3h) + c2l * c;
    const double d = ((x - c3h) - c3l) / (3.0 * c2h);
    const double g = -(0x1p-54 / 3.0) * log(x);
    return c + (d + c * g);
}
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

/* The two powers, exported for their tests. */
double oracle_cube_rn(double x) { return cube_rn(x); }
double oracle_pow_third(double x) { return pow_third(x); }

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
        fc = cube_rn(sc) / (6.0 * dx1 * dy1 * dz1);
    } else if (sc <= dy1) {
        fc = (sc * sc - dz1 * sc + dz1 * dz1 / 3.0) / (2.0 * dx1 * dy1);
    } else if (dx1 >= dy1 + dz1) {
        if (sc >= dy1 + dz1) {
            fc = (2.0 * sc - dy1 - dz1) / (2.0 * dx1);
        } else {
            fc = cube_rn(sc) - cube_rn(sc - dz1) - cube_rn(sc - dy1);
            fc = fc / (6.0 * dx1 * dy1 * dz1);
        }
    } else {
        if (sc > dx1)
            fc = cube_rn(sc) - cube_rn(sc - dz1) - cube_rn(sc - dy1) - cube_rn(sc - dx1);
        else
            fc = cube_rn(sc) - cube_rn(sc - dz1) - cube_rn(sc - dy1);
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
        delvar = (a3 * cube_rn(sc) + a2 * (sc * sc) + a1 * sc + a0) / (3.0 * a3 * (sc * sc) + 2.0 * a2 * sc + a1);
        sc = sc - delvar;
    }
    return sc;
}

/* Cubic_Equation_Solve (1380-1398); case2 selects the first form.          */
static double cubic_solve(double fc, double dx1, double dy1, double dz1, double sc, int case2)
{
    if (case2)
        return newton_raphson(1.0, -3.0 * (dy1 + dz1), 3.0 * (dy1 * dy1 + dz1 * dz1),
                              6.0 * fc * dx1 * dy1 * dz1 - (cube_rn(dy1) + cube_rn(dz1)), sc);
    return newton_raphson(2.0, -3.0 * (dx1 + dy1 + dz1), 3.0 * (dx1 * dx1 + dy1 * dy1 + dz1 * dz1),
                          6.0 * fc * dx1 * dy1 * dz1 - (cube_rn(dx1) + cube_rn(dy1) + cube_rn(dz1)), sc);
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
    sc = copysign(1.0, sc) * pow_third(fabs(sc));
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

/* ---- redistancing (Clsvof.f90:1689-1889, helpers 1904-1959, 1961-2060) --- */

static const int BAND_WIDTH = 4;   /* Clsvof.f90:31 */
static const int NV = 6;           /* Clsvof.f90:31 */

static double sgn(double a) { return copysign(1.0, a); }   /* dsign(1.d0, a) */

/* Isinsidecell (1904-1916) and Isinsiderect (1918-1927). */
static int inside_cell(double xp, double yp, double zp, double dx, double dy, double dz)
{
    return -0.5 * dx <= xp && xp <= 0.5 * dx && -0.5 * dy <= yp && yp <= 0.5 * dy && -0.5 * dz <= zp &&
           zp <= 0.5 * dz;
}
static int inside_rect(double d1, double d2, double r10, double r11, double r20, double r21)
{
    return r10 <= d1 && d1 <= r11 && r20 <= d2 && d2 <= r21;
}

/* Iscutface (1929-1959): does the plane cross the face at `fp` normal to
 * axis `cas` (its four corners not all on one side). */
static int cut_face(double fp, double nxx, double nyy, double nzz, double diss, double dx, double dy, double dz,
                    int cas)
{
    double p1, p2, p3, p4;
    if (cas == 1) {
        p1 = fp * nxx - 0.5 * dy * nyy - 0.5 * dz * nzz + diss;
        p2 = fp * nxx - 0.5 * dy * nyy + 0.5 * dz * nzz + diss;
        p3 = fp * nxx + 0.5 * dy * nyy + 0.5 * dz * nzz + diss;
        p4 = fp * nxx + 0.5 * dy * nyy - 0.5 * dz * nzz + diss;
    } else if (cas == 2) {
        p1 = -0.5 * dx * nxx + fp * nyy - 0.5 * dz * nzz + diss;
        p2 = -0.5 * dx * nxx + fp * nyy + 0.5 * dz * nzz + diss;
        p3 = 0.5 * dx * nxx + fp * nyy + 0.5 * dz * nzz + diss;
        p4 = 0.5 * dx * nxx + fp * nyy - 0.5 * dz * nzz + diss;
    } else {
        p1 = -0.5 * dx * nxx - 0.5 * dy * nyy + fp * nzz + diss;
        p2 = -0.5 * dx * nxx + 0.5 * dy * nyy + fp * nzz + diss;
        p3 = 0.5 * dx * nxx + 0.5 * dy * nyy + fp * nzz + diss;
        p4 = 0.5 * dx * nxx - 0.5 * dy * nyy + fp * nzz + diss;
    }
    return !(p1 * p2 >= 0.0 && p2 * p3 >= 0.0 && p3 * p4 >= 0.0 && p4 * p1 >= 0.0);
}

/* Shortest_Point_2d (1961-2060): the point of the plane's trace on the face
 * normal to axis `cas` (whose coordinate the caller has set) nearest the
 * centre of the cell (ii, jj, kk) away; the other two coordinates are
 * written.  Kept: the y-face case divides by |nzz| where it solves for x. */
static void shortest_point_2d(double nx1, double ny1, double nz1, double dis1, int ii, int jj, int kk, int cas,
                              double dx, double dy, double dz, double *xs, double *ys, double *zs)
{
    const double epsi = 1.0e-30;
    if (cas == 1) {
        const double temp = sqrt(ny1 * ny1 + nz1 * nz1 + epsi * epsi);
        const double nyy = ny1 / temp, nzz = nz1 / temp, diss = dis1 / temp;
        const double dij1 = nyy * dy * (double)jj + nzz * dz * (double)kk + diss;
        const double yp = dy * (double)jj - dij1 * nyy, zp = dz * (double)kk - dij1 * nzz;
        if (inside_rect(yp, zp, -0.5 * dy, 0.5 * dy, -0.5 * dz, 0.5 * dz)) {
            *ys = yp;
            *zs = zp;
            return;
        }
        const double yoff = fmax(fabs(yp) - 0.5 * dy, 0.0), zoff = fmax(fabs(zp) - 0.5 * dz, 0.0);
        const double yfc = sgn(yp) * 0.5 * dy, zfc = sgn(zp) * 0.5 * dz;
        if (yoff * fabs(nyy) > zoff * fabs(nzz)) {
            *ys = yfc;
            *zs = (diss + nyy * *ys) / (sgn(-nzz) * fmax(fabs(nzz), TOLPAR));
        } else {
            *zs = zfc;
            *ys = (diss + nzz * *zs) / (sgn(-nyy) * fmax(fabs(nyy), TOLPAR));
        }
    } else if (cas == 2) {
        const double temp = sqrt(nx1 * nx1 + nz1 * nz1 + epsi * epsi);
        const double nxx = nx1 / temp, nzz = nz1 / temp, diss = dis1 / temp;
        const double dij1 = nxx * dx * (double)ii + nzz * dz * (double)kk + diss;
        const double xp = dx * (double)ii - dij1 * nxx, zp = dz * (double)kk - dij1 * nzz;
        if (inside_rect(xp, zp, -0.5 * dx, 0.5 * dx, -0.5 * dz, 0.5 * dz)) {
            *xs = xp;
            *zs = zp;
            return;
        }
        const double xoff = fmax(fabs(xp) - 0.5 * dx, 0.0), zoff = fmax(fabs(zp) - 0.5 * dz, 0.0);
        const double xfc = sgn(xp) * 0.5 * dx, zfc = sgn(zp) * 0.5 * dz;
        if (xoff * fabs(nxx) > zoff * fabs(nzz)) {
            *xs = xfc;
            *zs = (diss + nxx * *xs) / (sgn(-nzz) * fmax(fabs(nzz), TOLPAR));
        } else {
            *zs = zfc;
            *xs = (diss + nzz * *zs) / (sgn(-nxx) * fmax(fabs(nzz), TOLPAR));
        }
    } else {
        const double temp = sqrt(nx1 * nx1 + ny1 * ny1 + epsi * epsi);
        const double nxx = nx1 / temp, nyy = ny1 / temp, diss = dis1 / temp;
        const double dij1 = nxx * dx * (double)ii + nyy * dy * (double)jj + diss;
        const double xp = dx * (double)ii - dij1 * nxx, yp = dy * (double)jj - dij1 * nyy;
        if (inside_rect(xp, yp, -0.5 * dx, 0.5 * dx, -0.5 * dy, 0.5 * dy)) {
            *xs = xp;
            *ys = yp;
            return;
        }
        const double xoff = fmax(fabs(xp) - 0.5 * dx, 0.0), yoff = fmax(fabs(yp) - 0.5 * dy, 0.0);
        const double xfc = sgn(xp) * 0.5 * dx, yfc = sgn(yp) * 0.5 * dy;
        if (xoff * fabs(nxx) > yoff * fabs(nyy)) {
            *xs = xfc;
            *ys = (diss + nxx * *xs) / (sgn(-nyy) * fmax(fabs(nyy), TOLPAR));
        } else {
            *ys = yfc;
            *xs = (diss + nyy * *ys) / (sgn(-nxx) * fmax(fabs(nxx), TOLPAR));
        }
    }
}

/* The distance from the centre of the cell (ii, jj, kk) away to the plane
 * piece n.x + diss = 0 of an interface cell, as the band loop of
 * Redistance_Levelset measures it (1740-1861): the facing boundary point
 * when it lies across the plane from that centre, else the foot of the
 * perpendicular when it falls inside the cell, else the nearest point of
 * the plane's trace on the face it leaves through.  `side` is phi at the
 * target centre. */
static double band_distance(double nxx, double nyy, double nzz, double diss, int ii, int jj, int kk, double dx,
                            double dy, double dz, double side)
{
    const int l = ii < -1 ? -1 : ii > 1 ? 1 : ii;
    const int m = jj < -1 ? -1 : jj > 1 ? 1 : jj;
    const int n = kk < -1 ? -1 : kk > 1 ? 1 : kk;
    const double xv = dx * (double)l / 2.0, yv = dy * (double)m / 2.0, zv = dz * (double)n / 2.0;
    const double dv = nxx * xv + nyy * yv + nzz * zv + diss;
    const double X = dx * (double)ii, Y = dy * (double)jj, Z = dz * (double)kk;
    if (dv * sgn(side) <= 0.0) return sqrt((X - xv) * (X - xv) + (Y - yv) * (Y - yv) + (Z - zv) * (Z - zv));
    const double dij1 = nxx * dx * (double)ii + nyy * dy * (double)jj + nzz * dz * (double)kk + diss;
    const double xp = X - dij1 * nxx, yp = Y - dij1 * nyy, zp = Z - dij1 * nzz;
    if (inside_cell(xp, yp, zp, dx, dy, dz))
        return sqrt((X - xp) * (X - xp) + (Y - yp) * (Y - yp) + (Z - zp) * (Z - zp));
    const double xoff = fmax(fabs(xp) - 0.5 * dx, 0.0);
    const double yoff = fmax(fabs(yp) - 0.5 * dy, 0.0);
    const double zoff = fmax(fabs(zp) - 0.5 * dz, 0.0);
    const double xfc = sgn(xp) * 0.5 * dx, yfc = sgn(yp) * 0.5 * dy, zfc = sgn(zp) * 0.5 * dz;
    const double ax = xoff * fabs(nxx), ay = yoff * fabs(nyy), az = zoff * fabs(nzz);
    double xs = 0.0, ys = 0.0, zs = 0.0, diss1;
    int cas;
    if (ax >= ay && ax >= az) {
        if (cut_face(xfc, nxx, nyy, nzz, diss, dx, dy, dz, 1)) {
            xs = xfc; diss1 = nxx * xs + diss; cas = 1;
        } else if (ay > az) {
            ys = yfc; diss1 = nyy * ys + diss; cas = 2;
        } else {
            zs = zfc; diss1 = nzz * zs + diss; cas = 3;
        }
        shortest_point_2d(nxx, nyy, nzz, diss1, ii, jj, kk, cas, dx, dy, dz, &xs, &ys, &zs);
    }
    if (ay >= ax && ay >= az) {
        if (cut_face(yfc, nxx, nyy, nzz, diss, dx, dy, dz, 2)) {
            ys = yfc; diss1 = nyy * ys + diss; cas = 2;
        } else if (ax > az) {
            xs = xfc; diss1 = nxx * xs + diss; cas = 1;
        } else {
            zs = zfc; diss1 = nzz * zs + diss; cas = 3;
        }
        shortest_point_2d(nxx, nyy, nzz, diss1, ii, jj, kk, cas, dx, dy, dz, &xs, &ys, &zs);
    }
    if (az >= ax && az >= ay) {
        if (cut_face(zfc, nxx, nyy, nzz, diss, dx, dy, dz, 3)) {
            zs = zfc; diss1 = nzz * zs + diss; cas = 3;
        } else if (ax > ay) {
            xs = xfc; diss1 = nxx * xs + diss; cas = 1;
        } else {
            ys = yfc; diss1 = nyy * ys + diss; cas = 2;
        }
        shortest_point_2d(nxx, nyy, nzz, diss1, ii, jj, kk, cas, dx, dy, dz, &xs, &ys, &zs);
    }
    return sqrt((X - xs) * (X - xs) + (Y - ys) * (Y - ys) + (Z - zs) * (Z - zs));
}

/* Redistance_Levelset (1689-1889).  Each interface cell (1e-15 < vfl <
 * 1-1e-15) takes sign(0.5-vfl)|dis| (dis from its centre); each full or
 * empty cell within BAND_WIDTH cells of an interface cell (in every index)
 * takes sign(0.5-vfl) times the least band_distance over those interface
 * cells; every other cell sign(0.5-vfl)(BAND_WIDTH+1) dx sqrt(3).  A full or
 * empty cell is never an interface cell and only its running minimum is
 * written, so the result does not depend on the loop order (the reference
 * loops i, j, k over the interface cells and ii, jj, kk over the band).
 * The distances use the interface cell's spacings.  phi is read (its sign
 * at the target) before any of it is written.                               */
static void redistance(const double *dx, const double *dy, const double *dz, const double *vfl, double *phi,
                       const double *nxx, const double *nyy, const double *nzz, const double *dis, double *aux,
                       int *fix)
{
    const double epsi = 1.0e-15;
    const size_t nin = (size_t)I * J * K;
    for (size_t q = 0; q < nin; ++q) { aux[q] = 1.0e4; fix[q] = 0; }
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                const size_t g = G(i, j, k), c = N(i, j, k);
                if (!(0.0 + epsi < vfl[g] && vfl[g] < 1.0 - epsi)) continue;
                aux[c] = sgn(0.5 - vfl[g]) * fabs(dis[g]);
                fix[c] = 1;
                for (int ii = -BAND_WIDTH; ii <= BAND_WIDTH; ++ii)
                    for (int jj = -BAND_WIDTH; jj <= BAND_WIDTH; ++jj)
                        for (int kk = -BAND_WIDTH; kk <= BAND_WIDTH; ++kk) {
                            const int ti = i + ii, tj = j + jj, tk = k + kk;
                            if (!(1 <= ti && ti <= I && 1 <= tj && tj <= J && 1 <= tk && tk <= K)) continue;
                            const size_t tg = G(ti, tj, tk), tc = N(ti, tj, tk);
                            if (!(vfl[tg] < 0.0 + epsi || vfl[tg] > 1.0 - epsi)) continue;
                            fix[tc] = 1;
                            const double deuc = band_distance(nxx[g], nyy[g], nzz[g], dis[g], ii, jj, kk, dx[c],
                                                              dy[c], dz[c], phi[tg]);
                            const double cur = fabs(aux[tc]);
                            aux[tc] = sgn(0.5 - vfl[tg]) * (deuc < cur ? deuc : cur);
                        }
            }
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                const size_t g = G(i, j, k), c = N(i, j, k);
                if (fix[c] == 1) phi[g] = aux[c];
                else phi[g] = (double)(BAND_WIDTH + 1) * dx[c] * sqrt(3.0) * sgn(0.5 - vfl[g]);
            }
}

/* ---- the boundary planes and the scheme (Clsvof.f90:355-798, 2087-2221) -- */

/* One CLSVOF time step, Clsvof_Scheme's arguments flattened.  Arrays:
 * x..dz interior; vofl, phil, nxl, nyl, nzl, nx, ny, nz, u, v, w ghosted;
 * the wall planes face by face W, E, S, N, B, T, (J,K) for W/E, (I,K) for
 * S/N, (I,J) for B/T, numbered like the sweeps' bc planes.                  */
struct oracle_clsvof_args {
    int imax, jmax, kmax;
    const double *x, *y, *z, *dx, *dy, *dz;
    double *vofl, *phil;                 /* in/out */
    double *nxl, *nyl, *nzl;             /* in/out: the liquid normals */
    const double *nx, *ny, *nz;          /* the fluid normals (the ghost level set uses them) */
    const double *u, *v, *w;             /* face velocities */
    const double *bc_vel[3];             /* BCu%VarW, BCv%VarS, BCw%VarB */
    double *lvs_bc[6];                   /* BCLvs%Var*: in (W, S, B feed the sweeps) and out */
    double *vof_bc[6];                   /* BCVof%Var*: out */
    int lvs_flag[6], vof_flag[6];        /* 0 Dirichlet, else Neumann */
    double lvs_const[6], vof_const[6];
    double dt;
};

/* TypicalBC (BoundaryFunction.f90) over one face: Dirichlet const, else the
 * inner value less const*d/2 (d negative on the E, N, T faces). */
static double typical_bc(int flag, double cst, double var, double d)
{
    return flag == 0 ? cst : var - cst * d / 2.0;
}

/* BoundaryConditionLvsVof (2087-2221).  The level-set planes: W and E take
 * LvSBoundaryCondition, phiL - nxL*d/2 with d = +dx, -dx (BCLvsW/E are
 * passed the liquid normals), S, N, B, T take TypicalBC; the level-set
 * ghosts are phiL -/+ the FLUID normal times the spacing, and the N ghost
 * subtracts like S (kept).  Then the VOF planes (TypicalBC) and the VOF
 * ghosts (copies).  Ghost edges and corners are not touched.               */
static void boundary_lvs_vof(const struct oracle_clsvof_args *a)
{
    double *phil = a->phil, *vofl = a->vofl;
    for (int pass = 0; pass < 2; ++pass) {
        double *f = pass == 0 ? phil : vofl;
        double *const *bc = pass == 0 ? a->lvs_bc : a->vof_bc;
        const int *flag = pass == 0 ? a->lvs_flag : a->vof_flag;
        const double *cst = pass == 0 ? a->lvs_const : a->vof_const;
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                const size_t b = (size_t)(j - 1) + (size_t)J * (k - 1);
                const size_t g1 = G(1, j, k), gI = G(I, j, k);
                const double d1 = a->dx[N(1, j, k)], dI = a->dx[N(I, j, k)];
                bc[0][b] = typical_bc(flag[0], cst[0], f[g1], d1);
                if (pass == 0) bc[0][b] = f[g1] - a->nxl[g1] * d1 / 2.0;
                f[G(0, j, k)] = pass == 0 ? f[g1] - a->nx[g1] * d1 : f[g1];
                bc[1][b] = typical_bc(flag[1], cst[1], f[gI], -dI);
                if (pass == 0) bc[1][b] = f[gI] - a->nxl[gI] * (-dI) / 2.0;
                f[G(I + 1, j, k)] = pass == 0 ? f[gI] + a->nx[gI] * dI : f[gI];
            }
        for (int i = 1; i <= I; ++i)
            for (int k = 1; k <= K; ++k) {
                const size_t b = (size_t)(i - 1) + (size_t)I * (k - 1);
                const size_t g1 = G(i, 1, k), gJ = G(i, J, k);
                const double d1 = a->dy[N(i, 1, k)], dJ = a->dy[N(i, J, k)];
                bc[2][b] = typical_bc(flag[2], cst[2], f[g1], d1);
                f[G(i, 0, k)] = pass == 0 ? f[g1] - a->ny[g1] * d1 : f[g1];
                bc[3][b] = typical_bc(flag[3], cst[3], f[gJ], -dJ);
                f[G(i, J + 1, k)] = pass == 0 ? f[gJ] - a->ny[gJ] * dJ : f[gJ];
            }
        for (int i = 1; i <= I; ++i)
            for (int j = 1; j <= J; ++j) {
                const size_t b = (size_t)(i - 1) + (size_t)I * (j - 1);
                const size_t g1 = G(i, j, 1), gK = G(i, j, K);
                const double d1 = a->dz[N(i, j, 1)], dK = a->dz[N(i, j, K)];
                bc[4][b] = typical_bc(flag[4], cst[4], f[g1], d1);
                f[G(i, j, 0)] = pass == 0 ? f[g1] - a->nz[g1] * d1 : f[g1];
                bc[5][b] = typical_bc(flag[5], cst[5], f[gK], -dK);
                f[G(i, j, K + 1)] = pass == 0 ? f[gK] + a->nz[gK] * dK : f[gK];
            }
    }
}

/* Clsvof_Scheme (355-798): NV sub-steps of dt/NV.  Sub-step kk sweeps
 * y, z, x when kk mod 3 = 1, z, x, y when 2, x, y, z when 0.  The first
 * sweep divides its fields by 1 - dtv/d (u_i - u_{i-1}); the later two add
 * dtv/d times the first sweep's fields times their own velocity
 * difference; the VOF is clipped to 0 and 1 within 1e-14 after each sweep.
 * Then the boundary planes, Interface_Reconstruct, the liquid normals, the
 * plane distances from the cell centres, and Redistance_Levelset.
 * Returns 0, or -1 when out of memory.                                      */
int oracle_clsvof_scheme(const struct oracle_clsvof_args *a)
{
    I = a->imax; J = a->jmax; K = a->kmax;
    const size_t ng = (size_t)(I + 2) * (J + 2) * (K + 2), nin = (size_t)I * J * K;
    double *buf = calloc(10 * ng + nin, sizeof(double));
    int *fix = calloc(nin, sizeof(int));
    if (!buf || !fix) { free(buf); free(fix); return -1; }
    double *nxx = buf, *nyy = buf + ng, *nzz = buf + 2 * ng, *dis = buf + 3 * ng;
    double *tvf[3] = {buf + 4 * ng, buf + 5 * ng, buf + 6 * ng};
    double *tls[3] = {buf + 7 * ng, buf + 8 * ng, buf + 9 * ng};
    double *aux = buf + 10 * ng;
    double *vfl = a->vofl, *phi = a->phil;
    const double *d[3] = {a->dx, a->dy, a->dz};
    const double *vel[3] = {a->u, a->v, a->w};
    const double *lvs_lo[3] = {a->lvs_bc[0], a->lvs_bc[2], a->lvs_bc[4]};
    const double dtv = a->dt / (double)NV;
    for (int kk = 1; kk <= NV; ++kk) {
        const int first = kk % 3 == 0 ? 0 : kk % 3 == 1 ? 1 : 2;
        for (int s = 0; s < 3; ++s) {
            const int ax = (first + s) % 3;
            memcpy(tvf[ax], vfl, ng * sizeof(double));
            memcpy(tls[ax], phi, ng * sizeof(double));
            oracle_interface_reconstruct(I, J, K, a->x, a->y, a->z, a->dx, a->dy, a->dz, vfl, phi, nxx, nyy, nzz,
                                         dis);
            sweep(ax, a->dx, a->dy, a->dz, a->x, a->y, a->z, vfl, phi, nxx, nyy, nzz, dis, vel[ax], a->bc_vel[ax],
                  lvs_lo[ax], dtv, tvf[ax], tls[ax]);
            for (int i = 1; i <= I; ++i)
                for (int j = 1; j <= J; ++j)
                    for (int k = 1; k <= K; ++k) {
                        const size_t g = G(i, j, k);
                        const size_t gm = G(i - (ax == 0), j - (ax == 1), k - (ax == 2));
                        const double dd = d[ax][N(i, j, k)], du = vel[ax][g] - vel[ax][gm];
                        if (s == 0) {
                            tvf[ax][g] = tvf[ax][g] / (1.0 - dtv / dd * du);
                            tls[ax][g] = tls[ax][g] / (1.0 - dtv / dd * du);
                        } else {
                            tvf[ax][g] = tvf[ax][g] + dtv / dd * tvf[first][g] * du;
                            tls[ax][g] = tls[ax][g] + dtv / dd * tls[first][g] * du;
                        }
                        if (tvf[ax][g] <= VOFEPS) tvf[ax][g] = 0.0;
                        if (tvf[ax][g] >= 1.0 - VOFEPS) tvf[ax][g] = 1.0;
                        vfl[g] = tvf[ax][g];
                        phi[g] = tls[ax][g];
                    }
        }
        boundary_lvs_vof(a);
        oracle_interface_reconstruct(I, J, K, a->x, a->y, a->z, a->dx, a->dy, a->dz, vfl, phi, nxx, nyy, nzz, dis);
        for (int i = 1; i <= I; ++i)
            for (int j = 1; j <= J; ++j)
                for (int k = 1; k <= K; ++k) {
                    const size_t g = G(i, j, k), c = N(i, j, k);
                    a->nxl[g] = nxx[g];
                    a->nyl[g] = nyy[g];
                    a->nzl[g] = nzz[g];
                    dis[g] = (0.5 * a->dx[c] * fabs(nxx[g]) + 0.5 * a->dy[c] * fabs(nyy[g]) +
                              0.5 * a->dz[c] * fabs(nzz[g])) - dis[g];
                }
        redistance(a->dx, a->dy, a->dz, vfl, phi, nxx, nyy, nzz, dis, aux, fix);
    }
    free(buf);
    free(fix);
    return 0;
}

/* The tail of one sub-step alone: Interface_Reconstruct, the liquid
 * normals, the centre distances and Redistance_Levelset (Clsvof.f90:767-780).
 * Returns 0, or -1 when out of memory. */
int oracle_clsvof_redistance(int imax, int jmax, int kmax, const double *x, const double *y, const double *z,
                             const double *dx, const double *dy, const double *dz, const double *vfl, double *phi,
                             double *nxl, double *nyl, double *nzl)
{
    I = imax; J = jmax; K = kmax;
    const size_t ng = (size_t)(I + 2) * (J + 2) * (K + 2), nin = (size_t)I * J * K;
    double *buf = calloc(4 * ng + nin, sizeof(double));
    int *fix = calloc(nin, sizeof(int));
    if (!buf || !fix) { free(buf); free(fix); return -1; }
    double *nxx = buf, *nyy = buf + ng, *nzz = buf + 2 * ng, *dis = buf + 3 * ng, *aux = buf + 4 * ng;
    oracle_interface_reconstruct(I, J, K, x, y, z, dx, dy, dz, vfl, phi, nxx, nyy, nzz, dis);
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                const size_t g = G(i, j, k), c = N(i, j, k);
                nxl[g] = nxx[g];
                nyl[g] = nyy[g];
                nzl[g] = nzz[g];
                dis[g] = (0.5 * dx[c] * fabs(nxx[g]) + 0.5 * dy[c] * fabs(nyy[g]) + 0.5 * dz[c] * fabs(nzz[g])) -
                         dis[g];
            }
    redistance(dx, dy, dz, vfl, phi, nxx, nyy, nzz, dis, aux, fix);
    free(buf);
    free(fix);
    return 0;
}
