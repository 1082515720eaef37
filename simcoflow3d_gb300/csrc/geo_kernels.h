// geo_kernels.h -- device view of one cut-cell family and the launchers of
// the geometry preprocessing (k_geometry.cu).
#pragma once
#include <algorithm>
#include "scf_common.cuh"

// Cells per thread segment of the column-marching face kernel.
constexpr int GEO_KSEG = 32;

// One cell family on the device, in the host arrays' layouts (scf_geometry.h):
// ghosted arrays of d.ng cells, interior arrays of d.n cells, ",3" arrays
// with the component as the slowest index.
struct GeoFam {
    const double *dx, *dy, *dz;           // interior
    const double *phi, *nx, *ny, *nz;     // ghosted
    double *vof, *vofl;                   // ghosted
    int *ct;                              // interior
    double *ee, *ne, *te;                 // ghosted
    double *fce, *fcn, *fct;              // ghosted x 3
    double *cent;                         // interior x 3
    double *wllh, *delh;                  // interior
    int *moex;                            // interior; nullptr: not allocated
    int *posnu;                           // (I-iu, J-iv, K-iw)
    int iu, iv, iw;
};

// Grid-stride loop over the interior cells (i, j, k 1-based).
#define INTERIOR_LOOP(d)                                                                     \
    for (int q_ = blockIdx.x * blockDim.x + threadIdx.x, i = 0, j = 0, k = 0;                 \
         q_ < (d).n && ((i = q_ % (d).I + 1), (j = (q_ / (d).I) % (d).J + 1),                 \
                        (k = q_ / ((d).I * (d).J) + 1), true);                               \
         q_ += gridDim.x * blockDim.x)

// DefineCell + CellGeoCal of one family; when ev is given, ev[0] and ev[1]
// are recorded around the face kernel.
void launch_cell_geo(const GeoFam &t, const Dims &d, int *exact_count, cudaStream_t st, int *launches,
                     cudaEvent_t *ev = nullptr);
// The rest of GridPreprocess and DefineMomentumExchangeCell.
void launch_grid_preprocess_tail(const GeoFam &P, const GeoFam &U, const GeoFam &V, const GeoFam &W, const Dims &d,
                                 int *exact_count, cudaStream_t st, int *launches);
// NumberExternalCell of one family; colbuf holds (I-iu)*(J-iv) ints.
void launch_posnu(const GeoFam &t, const Dims &d, int *colbuf, int *total, cudaStream_t st, int *launches);
