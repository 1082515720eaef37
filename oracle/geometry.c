/*
 * geometry.c -- CPU restatement of SIMCOFlow's cut-cell geometry
 * preprocessing (src/CutCell.f90).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the CUDA geometry kernels and the
 * timed CPU baseline of their benchmark; nothing in the product links or
 * calls it.  Parity status: the reference (Fortran) cannot be built on this
 * machine, and its tests hold no golden values for these routines, so this
 * restatement is pinned by known-answer tests in tests/ (planar cuts with
 * exact apertures, the closed form of an open face, numbering invariants)
 * and by an independent vectorised restatement of the face aperture
 * (simcoflow3d_gb300/workloads.py face_geo_area), not by reference outputs.
 *
 * Loops and expressions keep the reference's order; built with
 * -ffp-contract=off.  Fortran x**2.d0 is written x*x.
 *
 * Indexing (column-major, i fastest): ghosted (0:I+1,0:J+1,0:K+1), interior
 * (1:I,1:J,1:K), ",3" arrays with the component as the last index.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "../include/scf_geometry.h"

static int I, J, K;
#define G(i, j, k) ((size_t)(i) + (size_t)(I + 2) * ((size_t)(j) + (size_t)(J + 2) * (size_t)(k)))
#define NG ((size_t)(I + 2) * (J + 2) * (K + 2))
#define N(i, j, k) ((size_t)((i) - 1) + (size_t)I * ((size_t)((j) - 1) + (size_t)J * (size_t)((k) - 1)))
#define NN ((size_t)I * J * K)
#define G3(i, j, k, c) (G(i, j, k) + NG * (size_t)((c) - 1))
#define N3(i, j, k, c) (N(i, j, k) + NN * (size_t)((c) - 1))

static const double EPSI = 1.0e-3;   /* CutCell.f90:11 */

/* FaceGeoCal (CutCell.f90:883-981): open part of a d1 x d2 face at offset d3
 * along the face normal, clipped by n.x + phi > 0.  Area = open fraction,
 * Cent = centroid in the face's (1,2) axes and d3.                          */
void oracle_face_geo_cal(double d1, double d2, double n1, double n2, double n3, double d3, double phi,
                         double *area, double cent[3])
{
    const double d11 = d1 / 2.0, d22 = d2 / 2.0;
    double node[7][2];   /* the reference's node(6,2), plus room for rounded corner
                            values of alternating sign (six vertices)        */
    double dpt[4];
    int temp = 0;
    memset(node, 0, sizeof node);
    dpt[0] = d11 * n1 - d22 * n2 + d3 * n3 + phi;
    dpt[1] = -(d11 * n1) - d22 * n2 + d3 * n3 + phi;
    dpt[2] = -(d11 * n1) + d22 * n2 + d3 * n3 + phi;
    dpt[3] = d11 * n1 + d22 * n2 + d3 * n3 + phi;
    if (dpt[0] > 0.0) { node[temp][0] = d11; node[temp][1] = -d22; temp++; }
    if (dpt[0] * dpt[1] < 0.0) { node[temp][0] = (d22 * n2 - d3 * n3 - phi) / n1; node[temp][1] = -d22; temp++; }
    if (dpt[1] > 0.0) { node[temp][0] = -d11; node[temp][1] = -d22; temp++; }
    if (dpt[1] * dpt[2] < 0.0) { node[temp][0] = -d11; node[temp][1] = (d11 * n1 - d3 * n3 - phi) / n2; temp++; }
    if (dpt[2] > 0.0) { node[temp][0] = -d11; node[temp][1] = d22; temp++; }
    if (dpt[2] * dpt[3] < 0.0) { node[temp][0] = (-(d22 * n2) - d3 * n3 - phi) / n1; node[temp][1] = d22; temp++; }
    if (dpt[3] > 0.0) { node[temp][0] = d11; node[temp][1] = d22; temp++; }
    if (dpt[3] * dpt[0] < 0.0) { node[temp][0] = d11; node[temp][1] = (-(d11 * n1) - d3 * n3 - phi) / n2; temp++; }
    node[temp][0] = node[0][0];
    node[temp][1] = node[0][1];
    double vol = 0.0;
    for (int k = 0; k < temp; ++k)
        vol = vol + 0.5 * (node[k][0] * node[k + 1][1] - node[k + 1][0] * node[k][1]);
    *area = fabs(vol / (d1 * d2));
    cent[0] = 0.0; cent[1] = 0.0; cent[2] = 0.0;
    if (*area > 0.0) {
        for (int k = 0; k < temp; ++k) {
            cent[0] = cent[0] + 1.0 / 6.0 / vol * (node[k][0] + node[k + 1][0]) *
                                    (node[k][0] * node[k + 1][1] - node[k + 1][0] * node[k][1]);
            cent[1] = cent[1] + 1.0 / 6.0 / vol * (node[k][1] + node[k + 1][1]) *
                                    (node[k][0] * node[k + 1][1] - node[k + 1][0] * node[k][1]);
        }
    }
    cent[2] = d3;
}

/* DefineCell (CutCell.f90:329-365) */
static void define_cell(scf_geo_cells *t)
{
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                const size_t g = G(i, j, k), n = N(i, j, k);
                if (t->vof[g] >= 1.0 - EPSI) {
                    t->cell_type[n] = 0;
                    t->vofl[g] = t->vofl[g] / t->vof[g];
                    t->vof[g] = 1.0;
                }
                if (t->vof[g] <= EPSI) {
                    t->cell_type[n] = 2;
                    t->vof[g] = 0.0;
                    t->vofl[g] = 0.0;
                }
                if (t->vof[g] >= EPSI && t->vof[g] <= 1.0 - EPSI) t->cell_type[n] = 1;
            }
}

/* CellGeoCal (CutCell.f90:369-671) */
static void cell_geo_cal(scf_geo_cells *t)
{
    const double tol = 1.0e-20;
    double *we = malloc(sizeof(double) * NN), *se = malloc(sizeof(double) * NN), *be = malloc(sizeof(double) * NN);
    double *ceE = malloc(sizeof(double) * NN * 3), *ceW = malloc(sizeof(double) * NN * 3);
    double *ceN = malloc(sizeof(double) * NN * 3), *ceS = malloc(sizeof(double) * NN * 3);
    double *ceT = malloc(sizeof(double) * NN * 3), *ceB = malloc(sizeof(double) * NN * 3);
#define C3(a, i, j, k, c) a[N3(i, j, k, c)]
    for (size_t q = 0; q < NN; ++q) { we[q] = 1.0; se[q] = 1.0; be[q] = 1.0; t->wllh[q] = 0.0; }
    for (size_t q = 0; q < NG; ++q) { t->eearea[q] = 1.0; t->nearea[q] = 1.0; t->tearea[q] = 1.0; }
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                const size_t g = G(i, j, k), n = N(i, j, k);
                const double dx = t->dx[n], dy = t->dy[n], dz = t->dz[n];
                const double nx = t->nx[g], ny = t->ny[g], nz = t->nz[g], phi = t->phi[g];
                double fc[3];
                t->cell_cent[N3(i, j, k, 1)] = 0.0;
                t->cell_cent[N3(i, j, k, 2)] = 0.0;
                t->cell_cent[N3(i, j, k, 3)] = 0.0;
                oracle_face_geo_cal(dx, dy, nx, ny, nz, dz / 2.0, phi, &t->tearea[g], fc);   /* top */
                C3(ceT, i, j, k, 1) = fc[0]; C3(ceT, i, j, k, 2) = fc[1]; C3(ceT, i, j, k, 3) = fc[2];
                oracle_face_geo_cal(dx, dy, nx, ny, nz, -dz / 2.0, phi, &be[n], fc);         /* bottom */
                C3(ceB, i, j, k, 1) = fc[0]; C3(ceB, i, j, k, 2) = fc[1]; C3(ceB, i, j, k, 3) = fc[2];
                oracle_face_geo_cal(dy, dz, ny, nz, nx, dx / 2.0, phi, &t->eearea[g], fc);   /* east */
                C3(ceE, i, j, k, 1) = fc[2]; C3(ceE, i, j, k, 2) = fc[0]; C3(ceE, i, j, k, 3) = fc[1];
                oracle_face_geo_cal(dy, dz, ny, nz, nx, -dx / 2.0, phi, &we[n], fc);         /* west */
                C3(ceW, i, j, k, 1) = fc[2]; C3(ceW, i, j, k, 2) = fc[0]; C3(ceW, i, j, k, 3) = fc[1];
                oracle_face_geo_cal(dz, dx, nz, nx, ny, dy / 2.0, phi, &t->nearea[g], fc);   /* north */
                C3(ceN, i, j, k, 1) = fc[1]; C3(ceN, i, j, k, 2) = fc[2]; C3(ceN, i, j, k, 3) = fc[0];
                oracle_face_geo_cal(dz, dx, nz, nx, ny, -dy / 2.0, phi, &se[n], fc);         /* south */
                C3(ceS, i, j, k, 1) = fc[1]; C3(ceS, i, j, k, 2) = fc[2]; C3(ceS, i, j, k, 3) = fc[0];
                const double a = (t->eearea[g] - we[n]) * dy * dz;
                const double b = (t->nearea[g] - se[n]) * dx * dz;
                const double c = (t->tearea[g] - be[n]) * dx * dy;
                t->wllh[n] = sqrt(a * a + b * b + c * c);
            }
    /* shared faces: east (i-1 | i) */
#pragma omp parallel for collapse(2) schedule(static)
    for (int j = 1; j <= J; ++j)
        for (int k = 1; k <= K; ++k)
            for (int i = 2; i <= I; ++i) {
                const double w = we[N(i, j, k)], e = t->eearea[G(i - 1, j, k)];
                const double avg = (w * w + e * e) / (w + e + tol);
                t->fce[G3(i - 1, j, k, 2)] = (C3(ceW, i, j, k, 2) * w + C3(ceE, i - 1, j, k, 2) * e) / (w + e + tol);
                t->fce[G3(i - 1, j, k, 3)] = (C3(ceW, i, j, k, 3) * w + C3(ceE, i - 1, j, k, 3) * e) / (w + e + tol);
                t->fce[G3(i - 1, j, k, 1)] = C3(ceE, i - 1, j, k, 1);
                t->eearea[G(i - 1, j, k)] = avg;
            }
    /* north (j-1 | j) */
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 1; i <= I; ++i)
        for (int k = 1; k <= K; ++k)
            for (int j = 2; j <= J; ++j) {
                const double s = se[N(i, j, k)], nn = t->nearea[G(i, j - 1, k)];
                const double avg = (s * s + nn * nn) / (s + nn + tol);
                t->fcn[G3(i, j - 1, k, 1)] = (C3(ceS, i, j, k, 1) * s + C3(ceN, i, j - 1, k, 1) * nn) / (s + nn + tol);
                t->fcn[G3(i, j - 1, k, 3)] = (C3(ceS, i, j, k, 3) * s + C3(ceN, i, j - 1, k, 3) * nn) / (s + nn + tol);
                t->fcn[G3(i, j - 1, k, 2)] = C3(ceN, i, j - 1, k, 2);
                t->nearea[G(i, j - 1, k)] = avg;
            }
    /* top (k-1 | k); the second component takes CeB(...,1), as in the reference */
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 2; k <= K; ++k) {
                const double b = be[N(i, j, k)], tt = t->tearea[G(i, j, k - 1)];
                const double avg = (b * b + tt * tt) / (b + tt + tol);
                t->fct[G3(i, j, k - 1, 1)] = (C3(ceB, i, j, k, 1) * b + C3(ceT, i, j, k - 1, 1) * tt) / (b + tt + tol);
                t->fct[G3(i, j, k - 1, 2)] = (C3(ceB, i, j, k, 1) * b + C3(ceT, i, j, k - 1, 2) * tt) / (b + tt + tol);
                t->fct[G3(i, j, k - 1, 3)] = C3(ceT, i, j, k - 1, 3);
                t->tearea[G(i, j, k - 1)] = avg;
            }
    /* cells with all faces below 1e-2 become solid where MoExCell is not allocated */
    if (!t->moexcell) {
        for (int i = 2; i <= I; ++i)
            for (int j = 2; j <= J; ++j)
                for (int k = 2; k <= K; ++k) {
                    double m = t->eearea[G(i - 1, j, k)];
                    const double c[5] = {t->eearea[G(i, j, k)], t->nearea[G(i, j - 1, k)], t->nearea[G(i, j, k)],
                                         t->tearea[G(i, j, k - 1)], t->tearea[G(i, j, k)]};
                    for (int q = 0; q < 5; ++q) m = fmax(m, c[q]);
                    if (m < 1.0e-2) t->cell_type[N(i, j, k)] = 2;
                }
    }
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                const int ct = t->cell_type[N(i, j, k)];
                if (ct == 2) {
                    t->eearea[G(i - 1, j, k)] = 0.0; t->eearea[G(i, j, k)] = 0.0;
                    t->nearea[G(i, j - 1, k)] = 0.0; t->nearea[G(i, j, k)] = 0.0;
                    t->tearea[G(i, j, k - 1)] = 0.0; t->tearea[G(i, j, k)] = 0.0;
                }
                if (ct == 1) {
                    if (i + 1 <= I && t->cell_type[N(i + 1, j, k)] == 2) t->eearea[G(i, j, k)] = 0.0;
                    if (j + 1 <= J && t->cell_type[N(i, j + 1, k)] == 2) t->nearea[G(i, j, k)] = 0.0;
                    if (k + 1 <= K && t->cell_type[N(i, j, k + 1)] == 2) t->tearea[G(i, j, k)] = 0.0;
                }
            }
    /* boundary planes of the face centres, in the reference's order */
    for (int c = 1; c <= 3; ++c)
        for (int k = 0; k <= K + 1; ++k)
            for (int j = 0; j <= J + 1; ++j) {
                t->fce[G3(0, j, k, c)] = t->fce[G3(1, j, k, c)];
            }
    for (int c = 1; c <= 3; ++c)
        for (int k = 0; k <= K + 1; ++k)
            for (int j = 0; j <= J + 1; ++j) t->fcn[G3(0, j, k, c)] = t->fcn[G3(1, j, k, c)];
    for (int c = 1; c <= 3; ++c)
        for (int k = 0; k <= K + 1; ++k)
            for (int j = 0; j <= J + 1; ++j) t->fct[G3(0, j, k, c)] = t->fct[G3(1, j, k, c)];
    for (int c = 1; c <= 3; ++c)
        for (int k = 0; k <= K + 1; ++k)
            for (int j = 0; j <= J + 1; ++j) t->fce[G3(I, j, k, c)] = t->fce[G3(I - 1, j, k, c)];
    for (int c = 1; c <= 3; ++c)
        for (int k = 0; k <= K + 1; ++k)
            for (int i = 0; i <= I + 1; ++i) t->fce[G3(i, 0, k, c)] = t->fce[G3(i, 1, k, c)];
    for (int c = 1; c <= 3; ++c)
        for (int k = 0; k <= K + 1; ++k)
            for (int i = 0; i <= I + 1; ++i) t->fcn[G3(i, 0, k, c)] = t->fcn[G3(i, 1, k, c)];
    for (int c = 1; c <= 3; ++c)
        for (int k = 0; k <= K + 1; ++k)
            for (int i = 0; i <= I + 1; ++i) t->fct[G3(i, 0, k, c)] = t->fct[G3(i, 1, k, c)];
    for (int c = 1; c <= 3; ++c)
        for (int k = 0; k <= K + 1; ++k)
            for (int i = 0; i <= I + 1; ++i) t->fcn[G3(i, J, k, c)] = t->fcn[G3(i, J - 1, k, c)];
    for (int c = 1; c <= 3; ++c)
        for (int j = 0; j <= J + 1; ++j)
            for (int i = 0; i <= I + 1; ++i) t->fce[G3(i, j, 0, c)] = t->fce[G3(i, j, 1, c)];
    for (int c = 1; c <= 3; ++c)
        for (int j = 0; j <= J + 1; ++j)
            for (int i = 0; i <= I + 1; ++i) t->fcn[G3(i, j, 0, c)] = t->fcn[G3(i, j, 1, c)];
    for (int c = 1; c <= 3; ++c)
        for (int j = 0; j <= J + 1; ++j)
            for (int i = 0; i <= I + 1; ++i) t->fct[G3(i, j, 0, c)] = t->fct[G3(i, j, 1, c)];
    for (int c = 1; c <= 3; ++c)
        for (int j = 0; j <= J + 1; ++j)
            for (int i = 0; i <= I + 1; ++i) t->fct[G3(i, j, K, c)] = t->fct[G3(i, j, K - 1, c)];
    /* full cells with a closed face */
    for (int i = 2; i <= I; ++i)
        for (int j = 2; j <= J; ++j)
            for (int k = 2; k <= K; ++k) {
                const size_t n = N(i, j, k);
                if (fabs(t->vof[G(i, j, k)] - 1.0) < EPSI) {
                    if (t->eearea[G(i - 1, j, k)] == 0.0 || t->eearea[G(i, j, k)] == 0.0) {
                        t->wllh[n] = t->dy[n] * t->dz[n];
                        t->delh[n] = t->dx[n] / 2.0;
                    }
                    if (t->nearea[G(i, j - 1, k)] == 0.0 || t->nearea[G(i, j, k)] == 0.0) {
                        t->wllh[n] = t->dx[n] * t->dz[n];
                        t->delh[n] = t->dy[n] / 2.0;
                    }
                    if (t->tearea[G(i, j, k - 1)] == 0.0 || t->tearea[G(i, j, k)] == 0.0) {
                        t->wllh[n] = t->dx[n] * t->dy[n];
                        t->delh[n] = t->dz[n] / 2.0;
                    }
                }
            }
#undef C3
    free(we); free(se); free(be); free(ceE); free(ceW); free(ceN); free(ceS); free(ceT); free(ceB);
}

/* GridPreprocess (CutCell.f90:62-325) */
static void grid_preprocess(scf_geo_cells *P, scf_geo_cells *U, scf_geo_cells *V, scf_geo_cells *W)
{
    define_cell(P); define_cell(U); define_cell(V); define_cell(W);
    cell_geo_cal(P); cell_geo_cal(U); cell_geo_cal(V); cell_geo_cal(W);
    /* face centres of velocity cells on stretched grids */
    for (int j = 1; j <= J; ++j)
        for (int k = 1; k <= K; ++k) {
            for (int i = 1; i <= I - 1; ++i)
                if (U->cell_type[N(i, j, k)] != 1 && U->cell_type[N(i + 1, j, k)] != 1)
                    if (fabs(U->dx[N(i, j, k)] - U->dx[N(i + 1, j, k)]) > 1.0e-10) {
                        U->fce[G3(i, j, k, 1)] = 0.5 * P->dx[N(i + 1, j, k)];
                        U->fcn[G3(i, j, k, 1)] = 0.0;
                        U->fct[G3(i, j, k, 1)] = 0.0;
                    }
            U->fcn[G3(I, j, k, 1)] = 0.0;
            U->fct[G3(I, j, k, 1)] = 0.0;
        }
    for (int i = 1; i <= I; ++i)
        for (int k = 1; k <= K; ++k) {
            for (int j = 1; j <= J - 1; ++j)
                if (V->cell_type[N(i, j, k)] != 1 && V->cell_type[N(i, j + 1, k)] != 1)
                    if (fabs(V->dy[N(i, j, k)] - V->dy[N(i, j + 1, k)]) > 1.0e-10) {
                        V->fcn[G3(i, j, k, 2)] = 0.5 * P->dy[N(i, j + 1, k)];
                        V->fce[G3(i, j, k, 2)] = 0.0;
                        V->fct[G3(i, j, k, 2)] = 0.0;
                    }
            V->fce[G3(i, J, k, 2)] = 0.0;
            V->fct[G3(i, J, k, 2)] = 0.0;
        }
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j) {
            for (int k = 1; k <= K - 1; ++k)
                if (W->cell_type[N(i, j, k)] != 1 && W->cell_type[N(i, j, k + 1)] != 1)
                    if (fabs(W->dz[N(i, j, k)] - W->dz[N(i, j, k + 1)]) > 1.0e-10) {
                        W->fct[G3(i, j, k, 3)] = 0.5 * P->dz[N(i, j, k + 1)];
                        W->fce[G3(i, j, k, 3)] = 0.0;
                        W->fcn[G3(i, j, k, 3)] = 0.0;
                    }
            W->fce[G3(i, j, K, 3)] = 0.0;
            W->fcn[G3(i, j, K, 3)] = 0.0;
        }
    /* velocity-cell faces from the pressure cells */
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                const size_t g = G(i, j, k), n = N(i, j, k);
                const double dx = P->dx[n], dy = P->dy[n], dz = P->dz[n];
                double fc[3];
                P->cell_cent[N3(i, j, k, 1)] = 0.0;
                P->cell_cent[N3(i, j, k, 2)] = 0.0;
                P->cell_cent[N3(i, j, k, 3)] = 0.0;
                const double vof = P->vof[g];
                if (vof < 1.0 && vof > 0.0) {
                    oracle_face_geo_cal(dy, dz, P->ny[g], P->nz[g], P->nx[g], 0.0, P->phi[g], &U->eearea[G(i - 1, j, k)], fc);
                    U->fce[G3(i - 1, j, k, 1)] = fc[2] + dx / 2.0;
                    U->fce[G3(i - 1, j, k, 2)] = fc[0]; U->fce[G3(i - 1, j, k, 3)] = fc[1];
                    oracle_face_geo_cal(dz, dx, P->nz[g], P->nx[g], P->ny[g], 0.0, P->phi[g], &V->nearea[G(i, j - 1, k)], fc);
                    V->fcn[G3(i, j - 1, k, 2)] = fc[2] + dy / 2.0;
                    V->fcn[G3(i, j - 1, k, 1)] = fc[1]; V->fcn[G3(i, j - 1, k, 3)] = fc[0];
                    oracle_face_geo_cal(dx, dy, P->nx[g], P->ny[g], P->nz[g], 0.0, P->phi[g], &W->tearea[G(i, j, k - 1)], fc);
                    W->fct[G3(i, j, k - 1, 3)] = fc[2] + dz / 2.0;
                    W->fct[G3(i, j, k - 1, 1)] = fc[0]; W->fct[G3(i, j, k - 1, 2)] = fc[1];
                } else if (vof > 0.5) {
                    U->fce[G3(i - 1, j, k, 1)] = dx / 2.0;
                    U->fce[G3(i - 1, j, k, 2)] = 0.0; U->fce[G3(i - 1, j, k, 3)] = 0.0;
                    U->eearea[G(i - 1, j, k)] = 1.0;
                    V->fcn[G3(i, j - 1, k, 2)] = dy / 2.0;
                    V->fcn[G3(i, j - 1, k, 1)] = 0.0; V->fcn[G3(i, j - 1, k, 3)] = 0.0;
                    V->nearea[G(i, j - 1, k)] = 1.0;
                    W->fct[G3(i, j, k - 1, 3)] = dz / 2.0;
                    W->fct[G3(i, j, k - 1, 1)] = 0.0; W->fct[G3(i, j, k - 1, 2)] = 0.0;
                    W->tearea[G(i, j, k - 1)] = 1.0;
                } else {
                    U->eearea[G(i - 1, j, k)] = 0.0;
                    for (int c = 1; c <= 3; ++c) U->fce[G3(i - 1, j, k, c)] = 0.0;
                    V->nearea[G(i, j - 1, k)] = 0.0;
                    for (int c = 1; c <= 3; ++c) V->fcn[G3(i, j - 1, k, c)] = 0.0;
                    W->tearea[G(i, j, k - 1)] = 0.0;
                    for (int c = 1; c <= 3; ++c) W->fct[G3(i, j, k - 1, c)] = 0.0;
                }
            }
    /* pressure-cell faces and velocity-cell centres from the velocity cells */
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                const size_t g = G(i, j, k), n = N(i, j, k);
                double fc[3], area;
                if (U->vof[g] < 1.0 && U->vof[g] > 0.0) {
                    oracle_face_geo_cal(U->dy[n], U->dz[n], U->ny[g], U->nz[g], U->nx[g], 0.0, U->phi[g], &area, fc);
                    P->fce[G3(i, j, k, 1)] = fc[2] + P->dx[n] / 2.0;
                    P->fce[G3(i, j, k, 2)] = fc[0]; P->fce[G3(i, j, k, 3)] = fc[1];
                    U->cell_cent[N3(i, j, k, 1)] = fc[2];
                    U->cell_cent[N3(i, j, k, 2)] = fc[0];
                    U->cell_cent[N3(i, j, k, 3)] = fc[1];
                } else if (U->vof[g] > 0.5) {
                    P->eearea[g] = 1.0;
                    P->fce[G3(i, j, k, 1)] = P->dx[n] / 2.0;
                    P->fce[G3(i, j, k, 2)] = 0.0; P->fce[G3(i, j, k, 3)] = 0.0;
                    for (int c = 1; c <= 3; ++c) U->cell_cent[N3(i, j, k, c)] = 0.0;
                } else {
                    P->eearea[g] = 0.0;
                    for (int c = 1; c <= 3; ++c) P->fce[G3(i, j, k, c)] = 0.0;
                    for (int c = 1; c <= 3; ++c) U->cell_cent[N3(i, j, k, c)] = 0.0;
                }
                if (V->vof[g] < 1.0 && V->vof[g] > 0.0) {
                    oracle_face_geo_cal(V->dz[n], V->dx[n], V->nz[g], V->nx[g], V->ny[g], 0.0, V->phi[g], &area, fc);
                    P->fcn[G3(i, j, k, 1)] = fc[1]; P->fcn[G3(i, j, k, 3)] = fc[0];
                    P->fcn[G3(i, j, k, 2)] = fc[2] + P->dy[n] / 2.0;
                    V->cell_cent[N3(i, j, k, 1)] = fc[1];
                    V->cell_cent[N3(i, j, k, 2)] = fc[2];
                    V->cell_cent[N3(i, j, k, 3)] = fc[0];
                } else if (V->vof[g] > 0.5) {
                    P->nearea[g] = 1.0;
                    P->fcn[G3(i, j, k, 1)] = 0.0; P->fcn[G3(i, j, k, 3)] = 0.0;
                    P->fcn[G3(i, j, k, 2)] = P->dy[n] / 2.0;
                    for (int c = 1; c <= 3; ++c) V->cell_cent[N3(i, j, k, c)] = 0.0;
                } else {
                    P->nearea[g] = 0.0;
                    for (int c = 1; c <= 3; ++c) P->fcn[G3(i, j, k, c)] = 0.0;
                    for (int c = 1; c <= 3; ++c) V->cell_cent[N3(i, j, k, c)] = 0.0;
                }
                if (W->vof[g] < 1.0 && W->vof[g] > 0.0) {
                    oracle_face_geo_cal(W->dx[n], W->dy[n], W->nx[g], W->ny[g], W->nz[g], 0.0, W->phi[g], &area, fc);
                    P->fct[G3(i, j, k, 1)] = fc[0]; P->fct[G3(i, j, k, 2)] = fc[1];
                    P->fct[G3(i, j, k, 3)] = fc[2] + P->dz[n] / 2.0;
                    W->cell_cent[N3(i, j, k, 1)] = fc[0];
                    W->cell_cent[N3(i, j, k, 2)] = fc[1];
                    W->cell_cent[N3(i, j, k, 3)] = fc[2];
                } else if (W->vof[g] > 0.5) {
                    P->tearea[g] = 1.0;
                    P->fct[G3(i, j, k, 1)] = 0.0; P->fct[G3(i, j, k, 2)] = 0.0;
                    P->fct[G3(i, j, k, 3)] = P->dz[n] / 2.0;
                    for (int c = 1; c <= 3; ++c) W->cell_cent[N3(i, j, k, c)] = 0.0;
                } else {
                    P->tearea[g] = 0.0;
                    for (int c = 1; c <= 3; ++c) P->fct[G3(i, j, k, c)] = 0.0;
                    for (int c = 1; c <= 3; ++c) W->cell_cent[N3(i, j, k, c)] = 0.0;
                }
            }
}

/* DefineMomentumExchangeCell (CutCell.f90:673-749) */
static void define_momentum_exchange_cell(const scf_geo_cells *P, scf_geo_cells *U, scf_geo_cells *V,
                                          scf_geo_cells *W)
{
    for (int i = 1; i <= I; ++i)
        for (int j = 1; j <= J; ++j)
            for (int k = 1; k <= K; ++k) {
                const size_t n = N(i, j, k);
                const int pc = P->cell_type[n];
                if (U->cell_type[n] == 1) {
                    if (i < I) { if (pc == 2 || P->cell_type[N(i + 1, j, k)] == 2) U->moexcell[n] = 1; }
                    else if (pc == 2) U->moexcell[n] = 1;
                }
                if (V->cell_type[n] == 1) {
                    if (j < J) { if (pc == 2 || P->cell_type[N(i, j + 1, k)] == 2) V->moexcell[n] = 1; }
                    else if (pc == 2) V->moexcell[n] = 1;
                }
                if (W->cell_type[n] == 1) {
                    if (k < K) { if (pc == 2 || P->cell_type[N(i, j, k + 1)] == 2) W->moexcell[n] = 1; }
                    else if (pc == 2) W->moexcell[n] = 1;
                }
            }
}

/* NumberExternalCell (CutCell.f90:753-786); PosNu has bounds
 * (I-iu, J-iv, K-iw) and is numbered with k fastest.                         */
static void number_external_cell(int iu, int iv, int iw, scf_geo_cells *t)
{
    const int ni = I - iu, nj = J - iv;
    int ctr = 0;
    for (int i = 1; i <= I - iu; ++i)
        for (int j = 1; j <= J - iv; ++j)
            for (int k = 1; k <= K - iw; ++k) {
                const size_t q = (size_t)(i - 1) + (size_t)ni * ((size_t)(j - 1) + (size_t)nj * (size_t)(k - 1));
                if (t->cell_type[N(i, j, k)] != 2) t->posnu[q] = ctr++;
                else t->posnu[q] = -1;
            }
    t->ext_cell = ctr - 1;
}

/* The sequence of Main.f90:203-214 (and SolidBody.f90:815-822) without
 * NewCellFace.  Returns 0, or 1 for grids below 2 cells in a direction.    */
int oracle_grid_preprocess(int imax, int jmax, int kmax, scf_geo_cells *p, scf_geo_cells *u, scf_geo_cells *v,
                           scf_geo_cells *w)
{
    if (imax < 2 || jmax < 2 || kmax < 2) return 1;
    I = imax; J = jmax; K = kmax;
    grid_preprocess(p, u, v, w);
    define_momentum_exchange_cell(p, u, v, w);
    number_external_cell(0, 0, 0, p);
    number_external_cell(1, 0, 0, u);
    number_external_cell(0, 1, 0, v);
    number_external_cell(0, 0, 1, w);
    return 0;
}
