// scf_kernels.h -- argument blocks and launchers shared by the .cu files.
#pragma once
#include "scf_common.cuh"

// Cells per thread segment of the column-marching assembly kernels.
constexpr int SCF_KSEG = 32;

// Inputs of the assembly (device mirrors of scf_poisson_in) plus scratch.
struct AsmArgs {
    Dims d;
    const double *pdx, *pdy, *pdz, *udx, *vdy, *wdz;      // interior
    const double *phil, *vofl, *vof, *ee, *ne, *te;       // ghosted
    const double *vofo, *us, *vs, *ws, *dpu, *dpv, *dpw;  // ghosted
    const int *ct, *pos;                                  // interior
    int ext_cell;
    int flag[6];
    const double *bvar[6];
    double dt, betap, betam, epsi, tol, stale_init;
    double *pocoef;                                       // (I,J,K,6)
    // stale-coefficient bookkeeping
    unsigned *stale_count;
    unsigned stale_cap;
    long long *stale_list;
    double *col_val;        // [I*J][12]
    unsigned short *col_mask;
    double *grp_val;        // [groups][12]
    unsigned short *grp_mask;
    unsigned *flags;
    unsigned char *phase;   // ghosted, 1 wet / 2 dry / 0 neither
    double rdt;             // 1/dt
};

// Level-0 operator outputs (ghosted layout).
struct OpArgs {
    double *diag, *dinv, *cE, *cN, *cT, *extra, *b;
    unsigned char *active;
    float *diag32, *cE32, *cN32, *cT32, *extra32;  // mixed only (FP32 levels derive 1/diag)
    float *diag_lo, *cE_lo, *cN_lo, *cT_lo;        // mixed only: v - (double)(float)v
};

// rho: per-cell densities (ghosted) or nullptr for the reference's two-phase
// coefficients.
int launch_assemble(const AsmArgs &a, const OpArgs &o, bool mixed, const double *rho, double rho_ref,
                    cudaStream_t st, unsigned *stale_count_host, int *launches);

// ---- solver --------------------------------------------------------------
template <typename T>
struct MgLevel {
    int n0, n1, n2, sy, sz, tot;
    int f0, f1, f2;                 // coarsening factors towards the next level
    T *diag, *dinv, *cE, *cN, *cT, *extra;
    unsigned char *active;
    T *x, *xb, *d, *b;              // x/xb ping-pong, Chebyshev update, rhs
    unsigned *flags;                // the context's device error flags
    LevelView<T> view() const
    {
        LevelView<T> v;
        v.n0 = n0; v.n1 = n1; v.n2 = n2; v.sy = sy; v.sz = sz;
        v.diag = diag; v.dinv = dinv; v.cE = cE; v.cN = cN; v.cT = cT;
        return v;
    }
};

struct ChebCoef {
    int degree;
    double first;        // 1/theta
    double c1[8], c2[8]; // steps 1..degree-1
    int lines = 0;       // Jacobi blocks: 0 single cells, 1 segments of LINE_SEG cells along k
};
constexpr int LINE_SEG = 8;

struct Reducer {
    double *partials;    // >= max blocks of any reducing launch
    double *scal;        // ScfScalar slots
    int max_blocks;
};

// Coarsening and the coarsest dense inverse.
template <typename T>
void mg_coarsen(const MgLevel<T> &F, MgLevel<T> &C, cudaStream_t st, int *launches);
template <typename T>
void mg_coarse_inverse(const MgLevel<T> &L, double *ainv, int *map, int n, bool singular, cudaStream_t st,
                       int *launches);
// Live per-launch timing: CUDA events on the launching stream around the
// fine-level launches of the kernel classes below (the same numbering as the
// public scf_kernel_class).  Pairs beyond CAP in one solve go untimed.
enum KClass { KC_SMOOTH = 0, KC_SPMV = 1, KC_RESTRICT = 2, KC_PROLONG = 3, KC_CGUPDATE = 4, KC_SMOOTH2 = 5,
              KC_NUM = 6 };
// Pairs [0, EAGER) time eagerly launched kernels (reset after every
// harvest); pairs [EAGER, CAP) belong to the captured CG-iteration graph,
// whose event-record nodes fire on every replay.
struct KTimer {
    static constexpr int CAP = 512;
    static constexpr int EAGER = 384;
    cudaEvent_t ev[2 * CAP];
    int cls[CAP];
    double bytes[CAP];     // algorithmic bytes of the launch (< 0: the class's model)
    int n = 0;             // eager pairs in use
    int ng = EAGER;        // next graph pair while capturing
    bool on = false;
    bool capturing = false;
    int begin(int c, cudaStream_t st, double b = -1.0)
    {
        if (!on) return -1;
        int id;
        if (capturing) {
            if (ng >= CAP) return -1;
            id = ng++;
        } else {
            if (n >= EAGER) return -1;
            id = n++;
        }
        cls[id] = c;
        bytes[id] = b;
        record(ev[2 * id], st);
        return id;
    }
    void end(int id, cudaStream_t st)
    {
        if (id >= 0) record(ev[2 * id + 1], st);
    }
    void record(cudaEvent_t e, cudaStream_t st)
    {
        if (capturing) cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
        else cudaEventRecord(e, st);
    }
};
inline int kt_begin(KTimer *kt, int c, cudaStream_t st, double bytes = -1.0)
{
    return kt ? kt->begin(c, st, bytes) : -1;
}
inline void kt_end(KTimer *kt, int id, cudaStream_t st)
{
    if (kt) kt->end(id, st);
}

// One V-cycle: level 0 rhs in L[0].b, result in *z (== L[0].x or L[0].xb).
// first_done: level 0's first Chebyshev step was already written to L[0].x
// (fused into the CG update).  coarse_ready: an event the coarsest solve
// waits for (the dense inverse formed on another stream), or nullptr.
template <typename T>
T *mg_vcycle(MgLevel<T> *L, int nlev, const ChebCoef &cc, const double *ainv, const int *map, int ncoarse,
             bool singular, bool first_done, cudaStream_t st, int *launches, KTimer *kt = nullptr,
             cudaEvent_t coarse_ready = nullptr);

// Single launches of the fine-level kernels, for timing.
template <typename T>
void probe_smooth(MgLevel<T> &F, const ChebCoef &cc, cudaStream_t st);
template <typename T>
void probe_restrict(MgLevel<T> &F, MgLevel<T> &C, cudaStream_t st);
template <typename T>
void probe_prolong(MgLevel<T> &F, MgLevel<T> &C, const ChebCoef &cc, cudaStream_t st);
void probe_spmv(const LevelView<double> &A, const double *p, double *q, Reducer &R, cudaStream_t st);
cudaError_t probe_smooth2(MgLevel<float> &F, const ChebCoef &cc, cudaStream_t st);   // n0 even

// Large FP32 levels smooth two Chebyshev steps per pass (on: 1, the
// default) or one (0); planes: k-planes per block of the two-step kernel
// (0: the default).
void set_smoother_pairs(int on, int planes);
int smoother_pairs_state();          // changes whenever the setting does
void smoother_pair_counts(long long *tma, long long *fallback);
cudaError_t pair_smem_attr();        // the two-step kernel's shared-memory opt-in

// Fine operator of the mixed solver's CG in double-float form: hi parts are
// the FP32 level-0 copy, lo parts the rounding remainders written by the
// assembly (diag, cE, cN, cT).
struct DfOp {
    LevelView<float> hi;
    const float *dlo, *elo, *nlo, *tlo;
};
void df_spmv_dot(const DfOp &A, const float2 *p, float2 *q, Reducer &R, bool singular, cudaStream_t st,
                 int *launches, KTimer *kt = nullptr);
void df_cg_update(const DfOp &A, float2 *x, float2 *r, const float2 *p, const float2 *q, float *rlow, float *x0,
                  double first, Reducer &R, cudaStream_t st, int *launches, KTimer *kt = nullptr);
void df_pupdate(const DfOp &A, const float *z, float2 *p, const double *scal, bool first, cudaStream_t st,
                int *launches);
// (r, z) in FP64 from the double-float r and the FP32 z; beta into the scalars
void df_dot_rz(const DfOp &A, const float2 *r, const float *z, Reducer &R, cudaStream_t st, int *launches);
void df_from_double(const double *src, float2 *dst, int n, cudaStream_t st, int *launches);
// the residual r (FP64, whole padded array) to double-float in place, with
// its FP32 hi part written to rlow
void df_round_start(double *r, float *rlow, int n, cudaStream_t st, int *launches);
void df_to_double(const float2 *src, double *dst, int n, cudaStream_t st, int *launches);
// alpha and the mean of A p from the two-lane partials of an SpMV
void reduce_alpha(Reducer &R, int nblocks, bool singular, cudaStream_t st, int *launches);
// beta = (r, z) / (previous (r, z)) from one-lane partials; (r, z) kept
void reduce_beta(Reducer &R, int nblocks, cudaStream_t st, int *launches);

// CG building blocks on the fine level (FP64 vectors, ghosted layout).
void cg_spmv_dot(const LevelView<double> &A, const double *p, double *q, Reducer &R, bool singular,
                 cudaStream_t st, int *launches, KTimer *kt = nullptr);
template <typename T>
void cg_update(const LevelView<double> &A, double *x, double *r, const double *p, const double *q, T *rlow,
               const LevelView<T> &L0, T *x0, double first, Reducer &R, cudaStream_t st, int *launches,
               KTimer *kt = nullptr);
template <typename T>
void cg_dot_rz(const LevelView<double> &A, const double *r, const T *rlow, const T *z, Reducer &R, cudaStream_t st,
               int *launches);
template <typename T>
void cg_pupdate(const LevelView<double> &A, const T *z, double *p, const double *scal, bool first, cudaStream_t st,
                int *launches);
void reduce_to(Reducer &R, int nblocks, int slot, cudaStream_t st, int *launches);
// Right-hand side prologue: for an all-Neumann system the mean of b over the
// active cells is removed (S_COUNT, S_MEAN); then S_BB = (b, b).
void rhs_prologue(const LevelView<double> &A, const unsigned char *active, double *b, bool singular, Reducer &R,
                  cudaStream_t st, int *launches);
// r = b - A x, S_RR = (r, r); for an all-Neumann system also S_MEANX = mean
// of x over the active cells (removed from the scattered pressure).
void final_residual(const LevelView<double> &A, const unsigned char *active, const double *b, const double *x,
                    double *r, bool singular, Reducer &R, cudaStream_t st, int *launches);
// x -= S_MEANX on the active cells
void shift_solution(const LevelView<double> &A, const unsigned char *active, double *x, const double *scal,
                    cudaStream_t st, int *launches);
void copy_to_low(const LevelView<double> &A, const double *src, float *dst, cudaStream_t st, int *launches);

// sums of two partial arrays: mode 0 sum+count (S_SUM, S_COUNT, S_MEAN),
// 1 (S_RR, S_MEANX), 2 loss terms (S_JP, S_JD)
void reduce2_to(Reducer &R, int nblocks, int mode, cudaStream_t st, int *launches);
// S_MEAN = mean of v over the active cells
void active_mean(const LevelView<double> &A, const unsigned char *active, const double *v, Reducer &R,
                 cudaStream_t st, int *launches);

// ---- loss and adjoint --------------------------------------------------------
struct AdjArgs {
    Dims d;
    const double *us, *vs, *ws, *pp, *pfwd, *pocoef;
    const int *umoex, *uct, *vmoex, *vct, *wmoex, *wct, *ct;
    const double *ee, *ne, *te, *pdx, *pdy, *pdz;
    const double *gw;            // pressure-loss weights, ghosted
    double *r;                   // divergence of the corrected velocity, ghosted
    const unsigned char *phase;
    const double *phil;
    double tol;
};
void launch_pocoef_rho(const AsmArgs &a, const double *rho, double rho_ref, cudaStream_t st, int *launches);
// rho = rho_g on dry cells, rho_l elsewhere (the reference's two densities)
void fill_phase_density(const unsigned char *phase, double *rho, int ng, double rho_l, double rho_g, cudaStream_t st,
                        int *launches);
void launch_adj_divergence(const AdjArgs &A, Reducer &R, cudaStream_t st, int *launches);
void launch_adj_rhs(const AdjArgs &A, const double *scal, double *b, cudaStream_t st, int *launches);
void launch_adj_grad(const AdjArgs &A, const double *lam, const double *rho, double rho_ref, double *gu, double *gv,
                     double *gw, double *grho, cudaStream_t st, int *launches);

// ---- correction ------------------------------------------------------------
struct CorrArgs {
    Dims d;
    const double *x;                 // solution, ghosted (0 on solid/ghost)
    const int *ct;
    double *pp;                      // Proj%Pp, ghosted
    const double *pocoef;
    const double *us, *vs, *ws;      // u*
    const int *umoex, *uct, *vmoex, *vct, *wmoex, *wct;
    double *u, *v, *w, *p;           // TVar, ghosted
    const double *pdx, *pdy, *pdz;
    const double *ee, *ne, *te;
    int bcp_flag[6];
    int flag[4][6];
    double cst[4][6];
    double *bcvar[4][6];             // device planes (always written)
    double *tmp[4];                  // plane scratch for the top face
    int north_fix;
    unsigned *flags;
};

void launch_scatter(const CorrArgs &c, cudaStream_t st, int *launches);
void launch_correct(const CorrArgs &c, cudaStream_t st, int *launches);
