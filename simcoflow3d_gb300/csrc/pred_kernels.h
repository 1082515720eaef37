// pred_kernels.h -- device-side types and launchers of the momentum
// predictor's implicit solves (include/scf_predictor.h).
//
// Layout: every per-cell array of the solver lives on the ghosted grid of
// the component, (I+2)(J+2)(K+2) cells, i fastest, so the 7-point stencil
// needs no bounds checks.  Rows outside the reference's loop range
// (i = I for u, j = J for v, k = K for w), rows of solid cells and the ghost
// layer are identity rows with a zero right-hand side: their unknowns stay
// exactly 0 and couple to nothing.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace pred {

// Staged inputs of one component (device pointers; layouts of scf_mom_in).
struct MomDev {
    const double *dx, *dy, *dz;
    const double *vof, *vofl, *eta_e, *eta_n, *eta_t, *vof_old, *tvar;
    const double *df_ew, *df_ns, *df_tb, *edf_ew, *edf_ns, *edf_tb;
    const double *fric, *flux_div;
    const int32_t *cell_type, *posnu;
    const double *bc[6];
    int flag[6];
};

struct MomParams {
    double dt, rho_a, rho_w, fr, gx, gy, gz, g, beta_vis;
    double rfr2;    // 1 / (fr * fr), the same IEEE quotient the rows would form
    int flags[6];   // the component's BC%flag (1 = Neumann)
};

// The Jacobi-scaled system of one component: row c reads
//   x(c) - sum_d m_d(c) x(nb_d(c)) = b(c),   d = W,S,B,E,N,T,
// with m_d = a_d / aP and b = rhs / aP (0 on identity rows).
struct MomSys {
    double *m[6];
    float *m32[6];   // FP32 copies (mixed precision only; may be null)
    double *b;
    double *dp;      // PU/PV/PW%Dp, ghosted
};

struct Dims {
    int I, J, K;          // interior sizes of the pressure grid
    long long sy, sz, ng; // ghosted strides and size
};

// Scalars of one BiCGStab run, in device memory.
struct BcgScalars {
    double rho, alpha, omega, beta;
    double rr, bb;        // ||r||^2 and ||b||^2
    double target;        // stop when rr <= target (the device-side stopping test)
    int breakdown;        // 1: r0.v = 0 or an invalid beta in the last step
    int done;             // 1: converged or broken down; later passes return at once
    int iters;            // iterations run since the last set_target / residual
    int pad;
};

// Assembly (k_predictor.cu, compiled without FMA contraction).
void mom_assemble(const MomDev &in, const MomParams &o, int comp, const Dims &d, const MomSys &S, bool want32,
                  cudaStream_t st);
// Checks of the row numbering: counts[0] = active cells of the loop range,
// counts[1] = cells whose PosNu is -1 exactly when they are solid is false.
void mom_check_numbering(const MomDev &in, int comp, const Dims &d, unsigned long long *counts, cudaStream_t st);
// Tail of PredictingUVW for component c (0 = u): its Dp ghost planes, its
// velocity BC planes and the solid cells of the plane the BC writes.  Each
// component's tail touches only its own arrays, so it may run right after
// that component's solve.
void mom_tail_comp(const MomDev &in, const Dims &d, int c, double *pred, double *dp, cudaStream_t st,
                   int *launches);

// BiCGStab kernels (k_bicgstab.cu).  x, r, r0, p, v, t: ghosted T arrays.
template <typename T>
struct BcgVecs {
    T *x, *r, *r0, *p, *v, *t;
};
struct Reduce {
    double *partials;     // 4 per block
    int nblocks;
};
// ev (optional, 7 events): recorded around the four passes U, P, S, X.
template <typename T>
void bcg_iteration(const Dims &d, const T *const m[6], BcgVecs<T> &V, bool first, Reduce &R, BcgScalars *sc,
                   cudaStream_t st, cudaEvent_t *ev = nullptr);
// r = b - A x with the FP64 couplings (x = NULL: x = 0, r = b) into r64
// and/or r32 (rounded); ||r||^2 into sc->rr, the stored vector's norm^2 into
// sc->rho, and with want_bb ||b||^2 into sc->bb; resets alpha, omega, beta.
void resid64(const Dims &d, const double *const m[6], const double *b, const double *x, double *r64, float *r32,
             bool want_bb, Reduce &R, BcgScalars *sc, cudaStream_t st);
// x += e (FP32 correction), pointwise.
void xadd(const Dims &d, double *x, const float *e, cudaStream_t st);
// sc->target = target; clears done and iters.
void set_target(BcgScalars *sc, double target, cudaStream_t st);
// Launch shape of the per-cell kernels (assembly checks).
dim3 interior_block();
dim3 interior_grid(const Dims &d);
// Launch shape of the solver kernels (KZ-cell column segments); Reduce
// holds one partial per dot per block of this grid.
dim3 solver_block();
dim3 solver_grid(const Dims &d);

}  // namespace pred
