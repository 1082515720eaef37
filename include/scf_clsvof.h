/*
 * scf_clsvof.h -- the CLSVOF interface transport on GB300.
 *
 * scf_clsvof_step replaces Clsvof_Scheme (src/Clsvof.f90:355-798), the
 * coupled level-set / volume-of-fluid advection of the liquid that
 * Solver.f90 calls once per time step: six sub-steps of dt/6, each with
 * three split directional sweeps (X_Sweep 817-948, Y_Sweep 950-1083,
 * Z_Sweep 1085-1214, each after Interface_Reconstruct 1216-1309) in the
 * order y z x, z x y, x y z, then BoundaryConditionLvsVof (2087-2221),
 * Interface_Reconstruct and Redistance_Levelset (1689-1889).
 *
 * scf_clsvof_uvw_liquid_field replaces ComputeUVWLiquidField
 * (src/Clsvof.f90:174-298), which derives the U, V, W cells' liquid fields
 * from the P cells' after the transport.
 *
 * Arrays are Fortran column-major (i fastest).  "ghosted" means
 * (0:I+1,0:J+1,0:K+1), "interior" (1:I,1:J,1:K); wall planes are (J,K) for
 * the W and E faces, (I,K) for S and N, (I,J) for B and T, in that face
 * order.  I, J, K >= 3.
 *
 * Every function returns an int status (scf_status of scf_projection.h).
 */
#ifndef SCF_CLSVOF_H
#define SCF_CLSVOF_H

#include <stddef.h>
#include <stdint.h>
#include "scf_projection.h"

#ifdef __cplusplus
extern "C" {
#endif

/* What the step reads and does not change. */
typedef struct scf_clsvof_in {
    const double *x, *y, *z;       /* PGrid%x, %y, %z: cell centres, interior   */
    const double *dx, *dy, *dz;    /* PGrid%dx, %dy, %dz, interior              */
    const double *u, *v, *w;       /* TVar%u, %v, %w: face velocities, ghosted  */
    const double *nx, *ny, *nz;    /* PCell%nx, %ny, %nz (the fluid normals,
                                      which the ghost level set steps by), ghosted */
    const double *bc_u_w;          /* BCu%VarW (J,K)                            */
    const double *bc_v_s;          /* BCv%VarS (I,K)                            */
    const double *bc_w_b;          /* BCw%VarB (I,J)                            */
    int32_t lvs_flag[6], vof_flag[6];  /* BCLvs%flag, BCVof%flag: 0 Dirichlet   */
    double lvs_const[6], vof_const[6]; /* BCLvs%const, BCVof%const              */
    double dt;                     /* the time step; sub-steps are dt/6         */
} scf_clsvof_in;

/* What the step advances (host arrays, read by stage, written by fetch). */
typedef struct scf_clsvof_state {
    double *vofl, *phil;           /* PCell%vofL, %phiL, ghosted                */
    double *nxl, *nyl, *nzl;       /* PCell%nxL, %nyL, %nzL, ghosted (the
                                      interior is written; the W and E level-set
                                      planes read the x component)            */
    double *lvs_bc[6];             /* BCLvs%VarW ... %VarT: the W, S, B planes
                                      feed the sweeps' wall fluxes; all six are
                                      rewritten each sub-step                 */
    double *vof_bc[6];             /* BCVof%VarW ... %VarT, written             */
} scf_clsvof_state;

typedef struct scf_clsvof_stats {
    double ms_h2d, ms_run, ms_d2h, ms_total;   /* CUDA-event times               */
    int64_t bytes_h2d, bytes_d2h;
    int32_t steps;                 /* time steps run by the last call            */
    int32_t gpu_launches;          /* kernels launched by the last run           */
    double ms_kernels[4];          /* with scf_clsvof_set_timing: the summed
                                      times of k_reconstruct, k_sweep, k_walls
                                      and the three redistancing kernels       */
} scf_clsvof_stats;

typedef struct scf_clsvof_ctx scf_clsvof_ctx;

int scf_clsvof_create(scf_clsvof_ctx **ctx, int32_t imax, int32_t jmax, int32_t kmax, int32_t device);
int scf_clsvof_destroy(scf_clsvof_ctx *ctx);

/* Copies the inputs and the state to the device.                           */
int scf_clsvof_stage(scf_clsvof_ctx *ctx, const scf_clsvof_in *in, const scf_clsvof_state *state);
/* Runs `steps` Clsvof_Scheme steps on the device-resident state.           */
int scf_clsvof_run(scf_clsvof_ctx *ctx, int32_t steps, scf_clsvof_stats *stats);
/* Copies the state back.                                                   */
int scf_clsvof_fetch(scf_clsvof_ctx *ctx, scf_clsvof_state *state, scf_clsvof_stats *stats);
/* With on != 0, scf_clsvof_run times every kernel with CUDA events (and
 * synchronises after each step) to fill stats->ms_kernels.                 */
int scf_clsvof_set_timing(scf_clsvof_ctx *ctx, int32_t on);
/* stage + run(1) + fetch: one Clsvof_Scheme call with host arrays.         */
int scf_clsvof_step(scf_clsvof_ctx *ctx, const scf_clsvof_in *in, scf_clsvof_state *state,
                    scf_clsvof_stats *stats);

/* One velocity family's cells for ComputeUVWLiquidField.                  */
typedef struct scf_clsvof_vcell {
    const double *dx, *dy, *dz;    /* UGrid%dx ... (or V, W), interior          */
    double *phil, *nxl, *nyl, *nzl;    /* UCell%phiL, %nxL, %nyL, %nzL, ghosted:
                                      (0:I-1,0:J-1,0:K-1) is written             */
    double *vofl;                  /* UCell%vofL, ghosted: the interior is written */
} scf_clsvof_vcell;

/* ComputeUVWLiquidField (src/Clsvof.f90:174-298), which Solver.f90:209 calls
 * after Clsvof_Scheme: the U, V, W cells' liquid level set, normals and
 * fraction from the P cells' state on the device (after the last run, or
 * as staged).  cells[0..2] = U, V, W; their arrays are read (to keep what
 * is not written) and written back.  The clamp vof + vofL <= 1 of
 * ComputeVelocityCellLiquidField acts on values the loops then overwrite
 * in the reference, so it is not applied.                                  */
int scf_clsvof_uvw_liquid_field(scf_clsvof_ctx *ctx, const scf_clsvof_vcell cells[3], scf_clsvof_stats *stats);

/* The device copies of vofL and phiL (ghosted) after the last run, for
 * callers that keep the fields on the GPU (0 if not staged).               */
int scf_clsvof_device_fields(scf_clsvof_ctx *ctx, double **vofl, double **phil);

int scf_clsvof_last_error(scf_clsvof_ctx *ctx, char *buf, size_t n);

#ifdef __cplusplus
}
#endif
#endif
