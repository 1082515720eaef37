/*
 * scf_projection.h -- C ABI of the GB300 pressure projection for SIMCOFlow.
 *
 * The library replaces two pieces of SIMCOFlow's projection step:
 *
 *   - PoissonEquationSolver (src/ProjectionP.f90:33-121): GFM/cut-cell face
 *     coefficients, the 7-point pressure system, its solve (HYPRE PCG +
 *     BoomerAMG in the reference) and the scatter of the pressure with its
 *     ghost values;
 *   - the velocity correction of UpdatePUVW (src/ComputePUVW.f90:179-384):
 *     u = u* - grad(p) * PoCoef, p = Pp, BoundaryConditionVarNew with the
 *     TypicalBC rule, and the Dirichlet-face mass correction.
 *
 * Every array argument is a HOST pointer to the Fortran array's first element,
 * laid out column-major (i fastest).  "ghosted" arrays have bounds
 * (0:I+1, 0:J+1, 0:K+1); "interior" arrays (1:I, 1:J, 1:K); PoCoef is
 * (1:I, 1:J, 1:K, 1:6) with faces ordered W,S,B,E,N,T (ComputePUVW.f90:78).
 * Boundary arrays follow BCBase (BoundaryFunction.f90:31-46): VarW/VarE are
 * (J,K), VarS/VarN (I,K), VarB/VarT (I,J); face flags are ordered
 * W,E,S,N,B,T with 0 = Dirichlet and 1 = Neumann (BoundaryFunction.f90:48-59).
 *
 * The library borrows host arrays for the duration of a call and keeps no
 * host pointer.  A context owns one CUDA device's mirrors of the inputs, the
 * assembled operator, the multigrid hierarchy and the last pressure (used as
 * the warm start when requested).  Calls on one context are synchronous and
 * must come from one host thread at a time.
 *
 * Every function returns an int status (SCF_OK = 0).  The reference ignores
 * every HYPRE error code and halts with `pause` on a non-dominant row
 * (ProjectionP.f90:102-106,463-474); here each failure is a status.
 */
#ifndef SCF_PROJECTION_H
#define SCF_PROJECTION_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SCF_ABI_VERSION 2

/* ---- status codes ------------------------------------------------------- */
enum scf_status {
    SCF_OK = 0,
    SCF_ERR_BAD_ARG = 1,            /* null pointer, bad size or option      */
    SCF_ERR_NOT_CONVERGED = 2,      /* iteration or time cap reached         */
    SCF_ERR_NONFINITE = 3,          /* NaN/Inf in the system or the iterate  */
    SCF_ERR_CUDA = 4,               /* CUDA runtime error                    */
    SCF_ERR_OUT_OF_MEMORY = 5,      /* device allocation failed              */
    SCF_ERR_BAD_INPUT = 6,          /* inputs outside the reference's model  */
    SCF_ERR_UNDEFINED_IN_REFERENCE = 7, /* the reference code path has no
                                       defined result (see scf_opts)         */
    SCF_ERR_NO_DEVICE = 8,          /* no usable CUDA device                 */
    SCF_ERR_NO_SOLVE = 9            /* call needs a previous solve           */
};

/* ---- options ------------------------------------------------------------ */
enum scf_precision {
    SCF_PREC_FP64 = 0,   /* FP64 CG with an FP64 multigrid preconditioner     */
    SCF_PREC_MIXED = 1   /* CG in double-float arithmetic (FP32 pairs, about
                            48 significand bits; FP64 true residual at the end
                            of each round) with an FP32 multigrid V-cycle as
                            the preconditioner; FP64 coarsest solve           */
};

typedef struct scf_opts {
    int32_t precision;        /* enum scf_precision (default SCF_PREC_FP64)     */
    double  rel_tol;          /* stop when ||b-Ax||_2/||b||_2 <= rel_tol, with
                                 the FP64 operator (default 1e-10)             */
    int32_t max_iter;         /* cap on CG iterations, all rounds (default 500) */
    int32_t max_rounds;       /* cap on CG restarts from the true FP64 residual
                                 (when the recursive residual has drifted from
                                 it near the rounding floor), default 12       */
    double  inner_rtol;       /* reserved (default 1e-4; not used)             */
    int32_t smoother_degree;  /* Chebyshev degree per pre/post smoothing (3),
                                 1..8; the polynomial damps the interval
                                 [2/r, 2] of D^-1 A, r = max(6, 2 degree)     */
    int32_t coarse_max_cells; /* coarsen until a level has <= this many cells
                                 (default 64); solved densely in FP64          */
    double  rho_l, rho_g;     /* liquid/gas densities (StateVariables.f90:9)   */
    double  rho_ref;          /* reference density Roref (ProjectionP.f90:53);
                                 <= 0 means rho_l, as the reference passes row */
    double  epsi;             /* cut-cell threshold (CutCell.f90:11), 1e-3      */
    double  gfm_tol;          /* GFM lambda guard (ProjectionP.f90:18), 1e-30  */
    double  stale_init;       /* value of the reference's uninitialised BetaW/
                                 BetaD before their first assignment in a
                                 Compute1DGFMCoefficient call; the reference's
                                 debug build (-finit-real=nan) gives NaN       */
    int32_t warm_start;       /* 0: x0 = 0 as the reference (ProjectionP.f90:
                                 548); 1: start from the context's last p      */
    int32_t north_mass_fix;   /* the reference's North-face mass correction
                                 (ComputePUVW.f90:323-341) loops j twice with a
                                 stale k and indexes PGrid out of bounds.
                                 0: return SCF_ERR_UNDEFINED_IN_REFERENCE when
                                 that branch is taken; 1: apply the evident
                                 intent (j = Jmax, loop over i and k)          */
    int32_t check_inputs;     /* 1 (default): reject inputs outside the
                                 reference's model with SCF_ERR_BAD_INPUT      */
    int32_t device;           /* CUDA device ordinal (default 0)               */
    double  time_limit_s;     /* wall-clock cap on one solve (default 60 s)    */
    int32_t smoother_lines;   /* Jacobi blocks of the Chebyshev smoother:
                                 0 = single cells; 1 = segments of 8 cells
                                 along k, solved exactly (tridiagonal), which
                                 keeps strong k-couplings (z-stretched grids,
                                 thin layers) inside the blocks; 2 (default)
                                 = segments on FP32 V-cycles of grids whose
                                 smallest z spacing is at most half the larger
                                 of the (smallest) x and y spacings, single
                                 cells otherwise                              */
} scf_opts;

/* ---- per-call statistics -------------------------------------------------- */
typedef struct scf_stats {
    int32_t iterations;       /* CG iterations (all rounds)                    */
    int32_t rounds;           /* CG rounds: 1 + restarts from the true residual */
    int32_t converged;        /* 1 if rel_residual <= rel_tol                  */
    int32_t singular;         /* 1 if the system is all-Neumann (p defined up to
                                 a constant; the zero-mean solution is returned)*/
    int32_t levels;           /* multigrid levels                              */
    int32_t gpu_launches;     /* kernels launched by this call                 */
    double  rel_residual;     /* ||b-Ax||_2/||b||_2, FP64 operator             */
    double  rhs_norm;         /* ||b||_2                                       */
    double  ms_assemble;      /* coefficients + operator + rhs + hierarchy     */
    double  ms_solve;         /* CG (incl. V-cycles)                           */
    double  ms_correct;       /* scatter, velocity correction, BCs             */
    double  ms_h2d, ms_d2h;   /* host<->device copies inside the call; in
                                 scf_update_puvw ms_h2d covers the solve's
                                 inputs (the correction's inputs are copied
                                 on a second stream while the solve runs)    */
    double  ms_total;         /* device time of the whole call                 */
    int64_t bytes_h2d, bytes_d2h;
} scf_stats;

/* ---- inputs --------------------------------------------------------------- */
/* Everything PoissonEquationSolver reads (ProjectionP.f90:33-50).            */
typedef struct scf_poisson_in {
    const double  *pgrid_dx, *pgrid_dy, *pgrid_dz;   /* PGrid%dx,dy,dz interior */
    const double  *ugrid_dx, *vgrid_dy, *wgrid_dz;   /* UGrid%dx, VGrid%dy,
                                                        WGrid%dz interior      */
    const double  *pcell_phil, *pcell_vofl, *pcell_vof;        /* ghosted      */
    const double  *pcell_eearea, *pcell_nearea, *pcell_tearea; /* ghosted      */
    const int32_t *pcell_cell_type;                  /* interior               */
    const int32_t *pcell_posnu;                      /* interior, NumberExternal-
                                                        Cell numbering         */
    int32_t        pcell_extcell;                    /* PCell%ExtCell          */
    const double  *vof_old;                          /* PCellO%vof, ghosted    */
    const double  *pred_u, *pred_v, *pred_w;         /* TPred%u,v,w (u*), ghosted */
    const double  *pu_dp, *pv_dp, *pw_dp;            /* PU/PV/PW%Dp, ghosted   */
    int32_t        bcp_flag[6];                      /* BCp%flag (W,E,S,N,B,T) */
    const double  *bcp_var[6];                       /* BCp%VarW..VarT         */
    double         dt;
} scf_poisson_in;

/* What the correction block of UpdatePUVW reads besides the solve's inputs
 * (ComputePUVW.f90:181-232,255-384; BoundaryFunction.f90:69-513,760-781).
 * The BC procedure pointers are taken to be the TypicalBC routines
 * (BCU*, BCV*, BCW*, BCP*), i.e. Dirichlet = const and Neumann =
 * interior - const*d/2 with the reference's per-face spacing factors.      */
typedef struct scf_correct_in {
    const int32_t *ucell_moexcell, *ucell_cell_type; /* interior               */
    const int32_t *vcell_moexcell, *vcell_cell_type;
    const int32_t *wcell_moexcell, *wcell_cell_type;
    int32_t bcu_flag[6], bcv_flag[6], bcw_flag[6];   /* BCu/BCv/BCw%flag       */
    double  bcu_const[6], bcv_const[6], bcw_const[6], bcp_const[6]; /* %Const  */
} scf_correct_in;

/* Optional outputs of BoundaryConditionVarNew: the BC objects' Var arrays
 * after the call (field-major: u, v, w, p; faces W,E,S,N,B,T).  Any pointer
 * may be NULL.                                                               */
typedef struct scf_bc_out {
    double *var[4][6];
} scf_bc_out;

/* ---- context --------------------------------------------------------------- */
typedef struct scf_ctx scf_ctx;

/* Fills *opts with the defaults listed above (reference constants). */
void scf_opts_default(scf_opts *opts);

/* Replaces the per-call HYPRE set-up of SetBasicSolver/SetPoissonMatrix
 * (ProjectionP.f90:267-320): allocates the device state for an I x J x K
 * grid once.  Sizes must be >= 2 in every direction.                        */
int scf_ctx_create(scf_ctx **ctx, int32_t imax, int32_t jmax, int32_t kmax,
                   const scf_opts *opts);
int scf_ctx_destroy(scf_ctx *ctx);
/* Replaces the options of an existing context (sizes unchanged). */
int scf_ctx_set_opts(scf_ctx *ctx, const scf_opts *opts);

/* Drop-in for PoissonEquationSolver (ProjectionP.f90:33-121).
 *   pocoef : (I,J,K,6) FP64 output, PoCoef; may be NULL.
 *   pp     : ghosted FP64 output, Proj%Pp after DeltaPressureGetValues and
 *            DeltaPressureBoundaryCondition; may be NULL.  Ghost edges and
 *            corners, which the reference never writes, are 0 (UpdatePUVW
 *            zeroes Proj%Pp before the call, ComputePUVW.f90:102).
 * For an all-Neumann system the zero-mean (over active cells) solution is
 * returned; the reference's constant is HYPRE's.                            */
int scf_poisson_solve(scf_ctx *ctx, const scf_poisson_in *in,
                      double *pocoef, double *pp, scf_stats *stats);

/* Drop-in for the projection part of UpdatePUVW (ComputePUVW.f90:127-129,
 * 179-384): PoissonEquationSolver, the velocity correction, p = Pp,
 * BoundaryConditionVarNew and the Dirichlet-face mass correction.
 *   u, v, w, p : TVar%u,v,w,p, ghosted, in/out (values the reference leaves
 *                alone are left alone; the BCs read them).
 *   bc         : optional Var outputs, may be NULL.                         */
int scf_update_puvw(scf_ctx *ctx, const scf_poisson_in *in,
                    const scf_correct_in *corr, double *u, double *v,
                    double *w, double *p, scf_bc_out *bc, scf_stats *stats);

/* The same projection split into its host->device, device-only and
 * device->host parts, for callers that keep inputs resident between calls
 * (scf_update_puvw == stage_inputs + run_projection + fetch_outputs).      */
int scf_stage_inputs(scf_ctx *ctx, const scf_poisson_in *in,
                     const scf_correct_in *corr, const double *u,
                     const double *v, const double *w, const double *p);
int scf_run_projection(scf_ctx *ctx, scf_stats *stats);
int scf_fetch_outputs(scf_ctx *ctx, double *u, double *v, double *w,
                      double *p, double *pocoef, double *pp, scf_bc_out *bc);

/* ---- loss and adjoint gradient ---------------------------------------------
 * For the differentiable harness (no counterpart call in the reference; the
 * loss restates PrintDragLiftCoef's pressure force, Solver.f90:684-706).
 *   J[0] = sum_c g_c p_c   (g interior, e.g. -nz*WlLh on cut cells)
 *   J[1] = 1/2 sum over active cells of (D u)^2, u the corrected velocity of
 *          ComputePUVW.f90:181-232 before the boundary routines, D the
 *          divergence of SetPoissonVectors (ProjectionP.f90:521-526).
 * rho_cell: optional ghosted per-cell density field; face coefficients then
 * use the GFM face density lam*rho_a + (1-lam)*rho_b (ProjectionP.f90:155-
 * 235 with per-cell densities; identical to the reference, up to rounding,
 * when rho is each cell's phase density).  NULL: the reference's two
 * densities.  All-Neumann pressure boundaries only.
 * scf_loss_backward returns dJ/du*, dJ/dv*, dJ/dw* (ghosted, indexed like
 * the u*, v*, w* arrays) and dJ/drho (ghosted) of J[0] + J[1], by one
 * adjoint solve with the same operator.  Any output may be NULL.           */
int scf_loss_forward(scf_ctx *ctx, const scf_poisson_in *in, const scf_correct_in *corr,
                     const double *rho_cell, const double *g, double *J, scf_stats *stats);
int scf_loss_backward(scf_ctx *ctx, double *grad_u, double *grad_v, double *grad_w,
                      double *grad_rho, scf_stats *stats);

/* ---- diagnostics used by the parity tests ----------------------------------
 * All act on the operator of the last staged inputs (assembled on demand). */
/* y = A x on active cells, with the FP64 operator as stored on the device;
 * x and y are ghosted FP64 host arrays (ghost/solid entries of y are 0).    */
int scf_debug_apply(scf_ctx *ctx, const double *x, double *y);
/* z = M r: one V-cycle of the last run's multigrid hierarchy, in the
 * context's precision.  r and z are ghosted FP64 host arrays; z is 0 off the
 * active cells.  Needs a previous run.                                      */
int scf_debug_precondition(scf_ctx *ctx, const double *r, double *z);
/* Device operator: diag and the E/N/T couplings of each cell (interior
 * arrays; coupling = |off-diagonal| of row c towards c+e, 0 if none), and
 * the right-hand side b (interior, 0 on solid cells).  Any may be NULL.     */
int scf_debug_operator(scf_ctx *ctx, double *diag, double *cpl_e,
                       double *cpl_n, double *cpl_t, double *rhs);
/* FP32 forms of the device operator of a SCF_PREC_MIXED context (interior
 * arrays, solid cells included): hi = FP32 rounding (to nearest) of diag,
 * the E/N/T couplings and the extra diagonal part; lo = FP32 rounding of the
 * FP64 value minus hi, for diag and couplings (the double-float operator of
 * the CG); extra = the FP64 extra diagonal part (Dirichlet and solid-face
 * terms).  Any output may be NULL.                                         */
int scf_debug_operator_f32(scf_ctx *ctx, float *diag_hi, float *e_hi, float *n_hi,
                           float *t_hi, float *extra_hi, float *diag_lo, float *e_lo,
                           float *n_lo, float *t_lo, double *extra);

/* Times `reps` back-to-back launches of one kernel class of the last run's
 * state with CUDA events on the context's stream and reports the mean device
 * time per launch and the algorithmic bytes one launch moves (each array
 * touched once per cell).  kernel: SCF_K_SMOOTH (fine-level Chebyshev step
 * of the V-cycle, in its precision), SCF_K_SPMV (FP64 CG operator apply with
 * its dot product), SCF_K_RESTRICT (fine residual + restriction),
 * SCF_K_PROLONG (prolongation + first post-smoothing step; on large FP32
 * levels fused with the next step), SCF_K_CGUPDATE (FP64 x/r update with
 * its dot product), SCF_K_SMOOTH2 (two fused fine-level Chebyshev steps of
 * a SCF_PREC_MIXED context).  Needs a previous run.                        */
enum scf_kernel_class {
    SCF_K_SMOOTH = 0, SCF_K_SPMV = 1, SCF_K_RESTRICT = 2, SCF_K_PROLONG = 3, SCF_K_CGUPDATE = 4,
    SCF_K_SMOOTH2 = 5
};
int scf_debug_time_kernel(scf_ctx *ctx, int kernel, int reps, double *ms_per_launch,
                          double *bytes_per_launch);

/* Live per-kernel timing of real projections.  While enabled, every
 * fine-level launch of the kernel classes above inside a solve is bracketed
 * by CUDA events on the context's stream (at most 512 launches per solve);
 * the elapsed times accumulate per class across runs.  Enabling or disabling
 * resets the totals.  _read returns the total device milliseconds, the
 * number of timed launches and the mean algorithmic bytes of a timed launch
 * (each array a launch reads or writes counted once per cell; the smoother's
 * first and last steps move one array less); any output may be NULL.      */
int scf_kernel_timing(scf_ctx *ctx, int enable);
int scf_kernel_timing_read(scf_ctx *ctx, int kernel, double *ms_total, long long *launches,
                           double *bytes_per_launch);

/* ---- allocation-free operator apply ---------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory during a time step -- GPU-resident hosts that serve every device
 * buffer from their own preallocated arena, or jobs running at a fixed memory
 * budget on a shared GPU, where a late cudaMalloc may fail and, since it
 * synchronises the device, stalls their asynchronous work.
 *
 * Computes y = A x on the interior cells and x_dot_ax = sum x*(A x), with
 * A given by its diagonal and E/N/T couplings (the layout scf_debug_operator
 * reports, here as ghosted device arrays with a zero ghost layer).  Every
 * pointer is caller-owned DEVICE memory; x_dot_ax may be NULL.  Work is
 * queued on `stream` (a cudaStream_t; NULL = legacy default stream) and the
 * call returns without waiting for it.
 *
 * Scratch: a file-scope device array of SCF_NOALLOC_PARTIALS + 1 doubles
 * (32 KiB) that every device loading the library holds until exit.  The
 * first call on a device looks up that array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls share the array and it keeps the last call's contents; calls
 * that overlap on the GPU race on it.  Grids with more than
 * SCF_NOALLOC_MAX_CELLS ghosted cells are rejected with SCF_ERR_BAD_ARG.    */
#define SCF_NOALLOC_PARTIALS 4096
#define SCF_NOALLOC_MAX_CELLS 2147483647LL
int scf_apply_operator_noalloc(int32_t imax, int32_t jmax, int32_t kmax,
                               const double *diag, const double *cpl_e,
                               const double *cpl_n, const double *cpl_t,
                               const double *x, double *y, double *x_dot_ax,
                               void *stream);

/* ---- misc -------------------------------------------------------------- */
const char *scf_status_string(int status);
/* Copies the context's last error message (NUL-terminated) into buf.       */
int scf_last_error(const scf_ctx *ctx, char *buf, size_t len);
/* Pins a caller-owned host array and maps it into the device's address
 * space (cudaHostRegister, mapped and portable); undo with
 * scf_host_unregister.  The library moves page-locked, mapped arrays with
 * copy kernels that load from (and store to) host memory directly, and
 * other arrays with cudaMemcpyAsync.                                       */
int scf_host_register(void *ptr, size_t bytes);
int scf_host_unregister(void *ptr);
int scf_abi_version(void);

/* ---- test hooks (no counterpart in the reference) ------------------------
 * Every device buffer of this library (projection, geometry, predictor,
 * transport and output contexts) is allocated through one counting wrapper.
 * scf_debug_fail_device_alloc(n) makes the n-th device allocation from now
 * fail with SCF_ERR_OUT_OF_MEMORY, as a full GPU would, without calling
 * cudaMalloc for it (n = 0: off); the hook is process-wide and one-shot.
 * scf_debug_device_buffers() returns how many device buffers the library
 * holds, so a test can check that a failed create leaks none.             */
int     scf_debug_fail_device_alloc(int64_t nth);
int64_t scf_debug_device_buffers(void);

/* Large FP32 V-cycle levels can apply their Chebyshev steps in fused pairs,
 * one pass over the level for two steps.  on = 1 (the default): on levels of
 * at least 2^22 cells whose grid of 32 x 8 x planes blocks fills the GPU
 * twice; on = 2: on every FP32 level of at least 2^18 cells; on = 0: one
 * step per pass.  All give the same bits.  planes: k-planes per thread block
 * of the fused kernel (0: the default, 32).  Process-wide; applies from the
 * next solve of every context.                                             */
int scf_debug_smoother_pairs(int on, int planes);
/* Process-wide counts of fused-pair launches: those of the TMA-staged
 * kernel, and those that ran as two one-step launches instead because a
 * tensor map could not be encoded (none expected).  Either pointer may be
 * NULL.                                                                    */
int scf_debug_smoother_pair_counts(int64_t *tma_launches, int64_t *fallbacks);

#ifdef __cplusplus
}
#endif
#endif /* SCF_PROJECTION_H */
