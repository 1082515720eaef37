/*
 * scf_predictor.h -- the implicit solves of the momentum predictor on GB300.
 *
 * scf_predict_solves replaces the part of PredictingUVW
 * (src/PredictUVW.f90:691-802) that starts once the convective and diffusive
 * fluxes are known:
 *   - for each of u, v, w: SetMatrix (PredictUVW.f90:856-1164) and
 *     SetVectors (1166-1292) build the momentum system and PU/PV/PW%Dp;
 *   - HYPRE PCG + BoomerAMG solves it (SetBasicSolver, 821-854);
 *   - DeltaGetValues (1294-1336) scatters the solution into Pred%u/v/w;
 *   - then the Dp ghost planes are copied (766-788), and
 *     PredictorVelocityBoundaryCondition (3796-3894) and
 *     PredictorVelocityInternalCellCondition (3896-3914) run.
 *
 * All arrays are Fortran column-major (i fastest), as allocated by the
 * reference's drivers (src/Test/Dambreak/Dambreak.f90:228-413).  "ghosted"
 * means (0:I+1,0:J+1,0:K+1), "interior" (1:I,1:J,1:K).
 *
 * The momentum matrix is not symmetric: its rows are divided by the cell
 * density, and the cut-cell terms EDF weigh the two sides of a face
 * differently.  The GPU therefore solves it with BiCGStab on the
 * Jacobi-scaled system (rows divided by their diagonal), either in FP64
 * throughout or as FP32 BiCGStab inside FP64 iterative refinement.  The
 * stopping test is the FP64 residual of the scaled system relative to its
 * right-hand side.  The matrix rows, right-hand sides and Dp are formed
 * with the reference's own FP64 operations in its order, and Dp is returned
 * bit for bit.
 */
#ifndef SCF_PREDICTOR_H
#define SCF_PREDICTOR_H

#include <stddef.h>
#include <stdint.h>
#include "scf_projection.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One velocity component's inputs (iu, iv, iw = the component's unit flags).
 * TGrid, TCell, TCellO are UGrid/UCell/UCellO for u, and so on.          */
typedef struct scf_mom_in {
    const double  *grid_dx, *grid_dy, *grid_dz;  /* TGrid%dx,dy,dz, interior          */
    const double  *vof, *vofl;                   /* TCell%vof, vofL, ghosted          */
    const double  *eta_e, *eta_n, *eta_t;        /* TCell%EtaE, EtaN, EtaT, ghosted   */
    const int32_t *cell_type;                    /* TCell%Cell_Type, interior         */
    const int32_t *posnu;                        /* TCell%PosNu, (I-iu,J-iv,K-iw)     */
    int32_t        extcell;                      /* TCell%ExtCell                     */
    const double  *vof_old;                      /* TCellO%vof, ghosted               */
    /* the component's slices (last index iu+2iv+3iw) of the face arrays:
     * DFEW/EDFEW (0:I+1,1:J,1:K), DFNS/EDFNS (1:I,0:J+1,1:K),
     * DFTB/EDFTB (1:I,1:J,0:K+1)                                             */
    const double  *df_ew, *df_ns, *df_tb;
    const double  *edf_ew, *edf_ns, *edf_tb;
    const double  *fric;                         /* UFric/VFric/WFric, interior       */
    const double  *flux_div;                     /* FluxDiv(:,:,:,c), interior        */
    const double  *tvar;                         /* TVar%u / v / w, ghosted           */
    int32_t        bc_flag[6];                   /* BC%flag (W,E,S,N,B,T); 1 = Neumann */
    const double  *bc_var[6];                    /* BC%VarW,VarE (J,K), VarS,VarN (I,K),
                                                    VarB,VarT (I,J)                    */
} scf_mom_in;

typedef struct scf_mom_opts {
    double  dt;
    double  rho_a_ref, rho_w_ref;   /* roa/Roref, row/Roref (PredictUVW.f90:161-163)  */
    double  fr;                     /* Froude number (StateVariables.f90:80)           */
    double  gx, gy, gz, g;          /* gravity vector and its magnitude                */
    double  beta_vis;               /* Crank-Nicolson weight, 0.5 (PredictUVW.f90:35)  */
    double  rel_tol;                /* stopping test, scaled FP64 residual             */
    int32_t max_iter;               /* BiCGStab iterations (all refinement rounds)     */
    int32_t precision;              /* SCF_PREC_FP64 or SCF_PREC_MIXED                 */
    int32_t kernel_timing;          /* 1: CUDA events around each BiCGStab stencil
                                       kernel (stats.ms_kernels)                       */
} scf_mom_opts;

typedef struct scf_mom_stats {
    int32_t iterations[3];          /* BiCGStab iterations per component              */
    int32_t rounds[3];              /* refinement rounds (1 in FP64 mode)             */
    int32_t converged[3];
    double  rel_residual[3];        /* final FP64 scaled residual / scaled rhs        */
    double  ms_assemble;            /* SetMatrix + SetVectors of the three systems    */
    double  ms_solve;
    double  ms_tail;                /* scatter, Dp ghosts, boundary and solid cells   */
    double  ms_h2d, ms_d2h, ms_total;
    int64_t bytes_h2d, bytes_d2h;
    int32_t gpu_launches;
    /* with kernel_timing: summed device time of the four passes of the
     * BiCGStab iterations (U: p update; P: v = A p; S: t = A s; X: x and r),
     * and how many iterations they cover                                    */
    int32_t timed_iterations;
    double  ms_kernels[4];
} scf_mom_stats;

typedef struct scf_mom_ctx scf_mom_ctx;

/* A context for an (imax, jmax, kmax) grid on CUDA device `device`; it holds
 * the device copies of the inputs of the three components and the solver's
 * work arrays.                                                              */
int scf_mom_create(scf_mom_ctx **ctx, int32_t imax, int32_t jmax, int32_t kmax, int32_t device);
int scf_mom_destroy(scf_mom_ctx *ctx);

/* Copies the inputs of u, v, w (in[0..2]) to the device.                   */
int scf_mom_stage(scf_mom_ctx *ctx, const scf_mom_in in[3]);
/* Assembles and solves the three systems and applies the tail of
 * PredictingUVW on the device.                                             */
int scf_mom_run(scf_mom_ctx *ctx, const scf_mom_opts *opts, scf_mom_stats *stats);
/* Writes the results into the host arrays (ghosted): Pred%u/v/w only at the
 * entries the reference writes (the other entries keep their values), and
 * PU/PV/PW%Dp whole.  Any pointer may be NULL.                             */
int scf_mom_fetch(scf_mom_ctx *ctx, double *pred_u, double *pred_v, double *pred_w, double *pu_dp,
                  double *pv_dp, double *pw_dp);

/* stage + run + fetch, the drop-in for the solve part of PredictingUVW.    */
int scf_predict_solves(scf_mom_ctx *ctx, const scf_mom_in in[3], const scf_mom_opts *opts, double *pred_u,
                       double *pred_v, double *pred_w, double *pu_dp, double *pv_dp, double *pw_dp,
                       scf_mom_stats *stats);

/* Device pointers (ghosted FP64) of the results of the last run: Pred%u/v/w
 * and PU/PV/PW%Dp.  Pred holds only the entries the reference writes (zero
 * elsewhere).  Valid until the context is destroyed; any output may be NULL. */
int scf_mom_device_fields(scf_mom_ctx *ctx, const double **pred_u, const double **pred_v, const double **pred_w,
                          const double **pu_dp, const double **pv_dp, const double **pw_dp);

/* The message of the context's last failed call (empty if none).         */
int scf_mom_last_error(scf_mom_ctx *ctx, char *buf, size_t n);

#ifdef __cplusplus
}
#endif
#endif
