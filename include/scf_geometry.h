/*
 * scf_geometry.h -- C ABI of the GB300 cut-cell geometry preprocessing for
 * SIMCOFlow.
 *
 * One call replaces the geometry sequence that SIMCOFlow runs at start-up
 * (src/Main.f90:203-214) and after every motion of a solid body
 * (src/SolidBody.f90:815-822):
 *
 *   GridPreprocess(PGrid,UGrid,VGrid,WGrid, PCell,UCell,VCell,WCell)
 *       (src/CutCell.f90:62-325, with DefineCell 329-365, CellGeoCal
 *        369-671 and FaceGeoCal 883-981)
 *   DefineMomentumExchangeCell(PCell, UCell,VCell,WCell)   (673-749)
 *   NumberExternalCell(0,0,0,PCell), (1,0,0,UCell), (0,1,0,VCell),
 *       (0,0,1,WCell)                                      (753-786)
 *
 * Every array argument is a HOST pointer to the first element of a Fortran
 * array, column-major (i fastest), with the bounds of the reference's test
 * drivers (src/Test/Dambreak/Dambreak.f90:228-413): "ghosted" arrays are
 * (0:I+1, 0:J+1, 0:K+1), "interior" arrays (1:I, 1:J, 1:K), and arrays with a
 * trailing ",3" have a last index 1..3.  Arrays marked in/out are read and
 * written in place, like the reference's intent(inout) derived-type
 * members: entries the reference leaves untouched keep the caller's values.
 *
 * Results are bit-identical to a strict IEEE FP64 evaluation of the
 * reference's expressions in their order (no fused multiply-add).
 */
#ifndef SCF_GEOMETRY_H
#define SCF_GEOMETRY_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One cell family (PCell with PGrid, UCell with UGrid, ...). */
typedef struct scf_geo_cells {
    const double *dx, *dy, *dz;        /* TGrid%dx, dy, dz, interior            */
    const double *phi;                 /* TCell%phi (solid level set), ghosted   */
    const double *nx, *ny, *nz;        /* TCell%nx, ny, nz, ghosted              */
    double *vof, *vofl;                /* TCell%vof, vofL, ghosted, in/out
                                          (DefineCell rewrites full and empty
                                          cells)                                */
    int32_t *cell_type;                /* TCell%Cell_Type, interior, out         */
    double *eearea, *nearea, *tearea;  /* TCell%EEArea, NEArea, TEArea,
                                          ghosted, in/out                       */
    double *fce, *fcn, *fct;           /* TCell%FCE, FCN, FCT, ghosted ,3,
                                          in/out                                */
    double *cell_cent;                 /* TCell%Cell_Cent, interior ,3, in/out   */
    double *wllh;                      /* TCell%WlLh, interior, in/out           */
    double *delh;                      /* TCell%delh, interior, in/out           */
    int32_t *moexcell;                 /* TCell%MoExCell, interior, in/out; NULL
                                          when the member is not allocated (the
                                          reference's PCell): CellGeoCal then
                                          turns cells whose six faces are all
                                          below 1e-2 into solid cells           */
    int32_t *posnu;                    /* TCell%PosNu: (I,J,K) for PCell,
                                          (I-1,J,K) UCell, (I,J-1,K) VCell,
                                          (I,J,K-1) WCell; out                  */
    int32_t ext_cell;                  /* TCell%ExtCell, out                     */
} scf_geo_cells;

typedef struct scf_geo_stats {
    int32_t gpu_launches;     /* kernels launched by the call                      */
    int32_t exact_faces;      /* face polygons evaluated in full (the rest were
                                 entirely open or closed)                         */
    double  ms_h2d;           /* host->device copies                               */
    double  ms_device;        /* the kernels                                       */
    double  ms_d2h;           /* device->host copies                               */
    double  ms_total;         /* whole call                                        */
    int64_t bytes_h2d, bytes_d2h;
    double  ms_faces;         /* CUDA-event time of the four CellGeoCal face
                                 kernels (k_geo_faces), part of ms_device        */
    int64_t bytes_faces;      /* their algorithmic bytes: each array they read
                                 or write counted once per cell                 */
} scf_geo_stats;

typedef struct scf_geo_ctx scf_geo_ctx;

/* A context holds one device's buffers for one grid size (I, J, K >= 2);
 * keep it across time steps.                                                 */
int scf_geo_create(scf_geo_ctx **ctx, int32_t imax, int32_t jmax, int32_t kmax, int32_t device);
int scf_geo_destroy(scf_geo_ctx *ctx);

/* The whole sequence, host arrays in and out.  p, u, v, w are the PCell,
 * UCell, VCell and WCell families; p->moexcell is normally NULL.  Returns
 * SCF_OK (0) or an scf_status code (scf_projection.h).                      */
int scf_grid_preprocess(scf_geo_ctx *ctx, scf_geo_cells *p, scf_geo_cells *u, scf_geo_cells *v,
                        scf_geo_cells *w, scf_geo_stats *stats);

/* The same call split: copy the inputs (every array above) to the device,
 * run the sequence on the device copies (repeatable; each run starts from
 * the staged inputs), copy the results back into the families' arrays.     */
int scf_geo_stage(scf_geo_ctx *ctx, const scf_geo_cells *p, const scf_geo_cells *u,
                  const scf_geo_cells *v, const scf_geo_cells *w);
int scf_geo_run(scf_geo_ctx *ctx, scf_geo_stats *stats);
int scf_geo_fetch(scf_geo_ctx *ctx, scf_geo_cells *p, scf_geo_cells *u, scf_geo_cells *v,
                  scf_geo_cells *w);

/* Message of the last failure on this context. */
int scf_geo_last_error(scf_geo_ctx *ctx, char *buf, size_t n);

#ifdef __cplusplus
}
#endif
#endif
