// scf_api.cu -- C ABI of the GB300 projection (include/scf_projection.h).
//
// Host orchestration: device mirrors of the Fortran arrays, assembly, the
// multigrid hierarchy, the preconditioned CG loop and the correction.  All
// work of a context runs on one CUDA stream; calls are synchronous.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <vector>
#include "scf_kernels.h"
#include "../../include/scf_projection.h"
#include "scf_devmem.h"
#include "scf_stage.h"

namespace {

struct DevBuf {
    std::vector<void *> ptrs;
    ~DevBuf() { release(); }
    void release()
    {
        for (void *p : ptrs) scf_mem::dev_free(p);
        ptrs.clear();
    }
};

}  // namespace

struct scf_ctx {
    Dims d;
    scf_opts opts;
    cudaStream_t st = nullptr;
    cudaStream_t cst = nullptr;   // copies of the correction's inputs, overlapping the solve
    cudaEvent_t corr_ready = nullptr;
    // the coarsest level's dense inverse is formed on its own stream (one SM)
    // while the first V-cycle's downward sweep runs on the others
    cudaStream_t ist = nullptr;
    cudaEvent_t inv_start = nullptr, inv_ready = nullptr;
    bool inv_pending = false;     // the next V-cycle must wait for inv_ready
    bool corr_pending = false;    // st must wait for corr_ready before the correction
    char err[512] = {0};
    DevBuf mem, mgmem;
    // inputs (device)
    double *pdx, *pdy, *pdz, *udx, *vdy, *wdz;
    double *phil, *vofl, *vof, *ee, *ne, *te, *vofo, *us, *vs, *ws, *dpu, *dpv, *dpw;
    int *ct, *pos;
    int *umoex, *uct, *vmoex, *vct, *wmoex, *wct;
    double *tu, *tv, *tw, *tp;
    double *bvar[6];
    int ext_cell = -1;
    int bcp_flag[6];
    double dt = 0.0;
    scf_correct_in corr;
    bool have_corr = false;
    bool staged = false;
    bool solved = false;      // a projection has run (hierarchy and vectors exist)
    bool warm_ok = false;     // x holds the last solution (warm start)
    bool assembled = false;
    // assembly scratch
    double *pocoef;
    unsigned *stale_count, *flags;
    long long *stale_list;
    unsigned stale_cap;
    double *col_val, *grp_val;
    unsigned short *col_mask, *grp_mask;
    unsigned char *phase;
    // level-0 operator, FP64
    double *diag, *dinv, *cE, *cN, *cT, *extra, *b;
    unsigned char *active;
    float *diag32, *cE32, *cN32, *cT32, *extra32;
    float *diag_lo, *cE_lo, *cN_lo, *cT_lo;   // double-float remainders of the FP64 operator (mixed)
    // CG vectors
    double *x, *r, *p, *q;
    double *xbest;             // best round-end iterate of a solve that restarts
    KTimer kt;                 // live per-launch timing (scf_kernel_timing)
    // captured CG iteration (V-cycle, direction update, SpMV, x/r update)
    cudaGraphExec_t iter_exec = nullptr;
    unsigned long long iter_key = 0;
    int iter_launches = 0;     // kernels in one replay
    bool graphs_ok = true;     // cleared if capture is not available
    double aniso_z = 1.0;      // (larger of the x, y spacings / smallest z spacing)^2 of the staged grid
    unsigned mg_gen = 0;       // bumped whenever the hierarchy is reallocated
    bool kt_events = false;
    double kt_ms[KC_NUM] = {0}, kt_launches[KC_NUM] = {0}, kt_bytes[KC_NUM] = {0};
    // multigrid
    int nlev = 0;
    int mg_precision = -1;
    MgLevel<double> L64[32];
    MgLevel<float> L32[32];
    double *ainv;
    int *map;
    int ncoarse = 0;
    Reducer R;
    // correction
    double *pp;
    double *bcvar[4][6];
    // host pinned scratch
    double *h_scal = nullptr;
    unsigned *h_u32 = nullptr;
    cudaEvent_t ev[8];
    int launches = 0;
    // loss and adjoint (allocated on first use)
    DevBuf adjmem;
    double *adj_rho = nullptr, *adj_g = nullptr, *adj_r = nullptr, *adj_pfwd = nullptr;
    double *adj_gu = nullptr, *adj_gv = nullptr, *adj_gw = nullptr, *adj_grho = nullptr;
    bool use_rho = false;          // assemble with per-cell densities
    bool have_loss = false;        // a loss forward has run on the current state
    bool rho_given_last = false;   // the last loss forward used a density field
};

namespace {

void set_err(scf_ctx *c, const char *fmt, ...)
{
    if (!c) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof(c->err), fmt, ap);
    va_end(ap);
}

#define CK(call)                                                                           \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            set_err(ctx, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return e_ == cudaErrorMemoryAllocation ? SCF_ERR_OUT_OF_MEMORY : SCF_ERR_CUDA;  \
        }                                                                                  \
    } while (0)

template <typename P>
int dalloc(scf_ctx *ctx, DevBuf &mem, P **ptr, size_t count)
{
    void *p = nullptr;
    size_t bytes = count * sizeof(P);
    if (bytes == 0) bytes = 16;
    cudaError_t e = scf_mem::dev_malloc(&p, bytes);
    if (e != cudaSuccess) {
        set_err(ctx, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
        return SCF_ERR_OUT_OF_MEMORY;
    }
    cudaMemset(p, 0, bytes);
    mem.ptrs.push_back(p);
    *ptr = (P *)p;
    return SCF_OK;
}

#define DALLOC(mem, ptr, n)                          \
    do {                                             \
        int rc_ = dalloc(ctx, mem, &(ptr), (size_t)(n)); \
        if (rc_) return rc_;                         \
    } while (0)

bool is_singular(const scf_ctx *ctx)
{
    for (int q = 0; q < 6; ++q)
        if (ctx->bcp_flag[q] == 0) return false;
    return true;
}

template <typename T>
int alloc_level(scf_ctx *ctx, MgLevel<T> &L, int n0, int n1, int n2, bool own_op)
{
    L.n0 = n0; L.n1 = n1; L.n2 = n2;
    L.flags = ctx->flags;
    L.sy = n0 + 2;
    L.sz = L.sy * (n1 + 2);
    L.tot = L.sz * (n2 + 2);
    if (own_op) {
        DALLOC(ctx->mgmem, L.diag, L.tot);
        DALLOC(ctx->mgmem, L.dinv, L.tot);
        DALLOC(ctx->mgmem, L.cE, L.tot);
        DALLOC(ctx->mgmem, L.cN, L.tot);
        DALLOC(ctx->mgmem, L.cT, L.tot);
        DALLOC(ctx->mgmem, L.extra, L.tot);
        DALLOC(ctx->mgmem, L.active, L.tot);
        DALLOC(ctx->mgmem, L.b, L.tot);
    }
    DALLOC(ctx->mgmem, L.x, L.tot);
    DALLOC(ctx->mgmem, L.xb, L.tot);
    DALLOC(ctx->mgmem, L.d, L.tot);
    return SCF_OK;
}

// Level sizes and factors; fills ctx->nlev.
void plan_levels(scf_ctx *ctx, int dims[][3], int fac[][3])
{
    int n0 = ctx->d.I, n1 = ctx->d.J, n2 = ctx->d.K;
    int cmax = ctx->opts.coarse_max_cells;
    int l = 0;
    dims[0][0] = n0; dims[0][1] = n1; dims[0][2] = n2;
    while ((long long)n0 * n1 * n2 > cmax && (n0 > 2 || n1 > 2 || n2 > 2) && l < 30) {
        fac[l][0] = n0 > 2 ? 2 : 1;
        fac[l][1] = n1 > 2 ? 2 : 1;
        fac[l][2] = n2 > 2 ? 2 : 1;
        n0 = (n0 + fac[l][0] - 1) / fac[l][0];
        n1 = (n1 + fac[l][1] - 1) / fac[l][1];
        n2 = (n2 + fac[l][2] - 1) / fac[l][2];
        ++l;
        dims[l][0] = n0; dims[l][1] = n1; dims[l][2] = n2;
    }
    fac[l][0] = fac[l][1] = fac[l][2] = 1;
    ctx->nlev = l + 1;
}

template <typename T>
int build_levels(scf_ctx *ctx, MgLevel<T> *L, int dims[][3], int fac[][3])
{
    for (int l = 0; l < ctx->nlev; ++l) {
        int rc = alloc_level<T>(ctx, L[l], dims[l][0], dims[l][1], dims[l][2], l > 0);
        if (rc) return rc;
        L[l].f0 = fac[l][0]; L[l].f1 = fac[l][1]; L[l].f2 = fac[l][2];
    }
    return SCF_OK;
}

int ensure_mg(scf_ctx *ctx)
{
    const int prec = ctx->opts.precision;
    if (ctx->mg_precision == prec) return SCF_OK;
    if (ctx->ist) cudaStreamSynchronize(ctx->ist);   // no inverse in flight into the buffers freed here
    ctx->inv_pending = false;
    ctx->mgmem.release();
    ctx->mg_gen++;
    if (ctx->iter_exec) { cudaGraphExecDestroy(ctx->iter_exec); ctx->iter_exec = nullptr; }
    int dims[32][3], fac[32][3];
    plan_levels(ctx, dims, fac);
    int rc;
    if (prec == SCF_PREC_FP64) {
        rc = build_levels<double>(ctx, ctx->L64, dims, fac);
        if (rc) return rc;
        MgLevel<double> &L0 = ctx->L64[0];
        L0.diag = ctx->diag; L0.dinv = ctx->dinv; L0.cE = ctx->cE; L0.cN = ctx->cN; L0.cT = ctx->cT;
        L0.extra = ctx->extra; L0.active = ctx->active; L0.b = ctx->r;
    } else {
        rc = build_levels<float>(ctx, ctx->L32, dims, fac);
        if (rc) return rc;
        MgLevel<float> &L0 = ctx->L32[0];
        DALLOC(ctx->mgmem, ctx->diag32, L0.tot);
        DALLOC(ctx->mgmem, ctx->cE32, L0.tot);
        DALLOC(ctx->mgmem, ctx->cN32, L0.tot);
        DALLOC(ctx->mgmem, ctx->cT32, L0.tot);
        DALLOC(ctx->mgmem, ctx->extra32, L0.tot);
        DALLOC(ctx->mgmem, ctx->diag_lo, L0.tot);
        DALLOC(ctx->mgmem, ctx->cE_lo, L0.tot);
        DALLOC(ctx->mgmem, ctx->cN_lo, L0.tot);
        DALLOC(ctx->mgmem, ctx->cT_lo, L0.tot);
        DALLOC(ctx->mgmem, L0.b, L0.tot);
        L0.diag = ctx->diag32; L0.dinv = nullptr; L0.cE = ctx->cE32; L0.cN = ctx->cN32; L0.cT = ctx->cT32;
        L0.extra = ctx->extra32; L0.active = ctx->active;
        // the two-step smoother's shared memory (set here, outside any capture)
        CK(pair_smem_attr());
    }
    // coarsest dense map
    const int last = ctx->nlev - 1;
    const int c0 = dims[last][0], c1 = dims[last][1], c2 = dims[last][2];
    ctx->ncoarse = c0 * c1 * c2;
    std::vector<int> hmap;
    const int sy = c0 + 2, sz = sy * (c1 + 2);
    for (int k = 1; k <= c2; ++k)
        for (int j = 1; j <= c1; ++j)
            for (int i = 1; i <= c0; ++i) hmap.push_back(i + sy * j + sz * k);
    DALLOC(ctx->mgmem, ctx->map, hmap.size());
    DALLOC(ctx->mgmem, ctx->ainv, (size_t)ctx->ncoarse * ctx->ncoarse);
    CK(cudaMemcpy(ctx->map, hmap.data(), hmap.size() * sizeof(int), cudaMemcpyHostToDevice));
    ctx->mg_precision = prec;
    return SCF_OK;
}

int check_flags(scf_ctx *ctx)
{
    CK(cudaMemcpyAsync(ctx->h_u32, ctx->flags, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    const unsigned f = *ctx->h_u32;
    if (!f) return SCF_OK;
    if (f & FLAG_NONFINITE) { set_err(ctx, "non-finite value in the assembled system (flags 0x%x)", f); return SCF_ERR_NONFINITE; }
    if (f & FLAG_BAD_POSNU) { set_err(ctx, "PosNu is not -1 exactly on the Cell_Type==2 cells, or exceeds ExtCell"); return SCF_ERR_BAD_INPUT; }
    if (f & FLAG_STALE_OVERFLOW) { set_err(ctx, "too many cells with a carried GFM coefficient"); return SCF_ERR_BAD_INPUT; }
    if (ctx->opts.check_inputs) {
        if (f & FLAG_NEITHER_ACTIVE) { set_err(ctx, "an active cell (Cell_Type/=2) is neither wet nor dry (vof <= epsi)"); return SCF_ERR_BAD_INPUT; }
        if (f & FLAG_BAD_DIAG) { set_err(ctx, "an active row has a non-positive diagonal (all faces closed)"); return SCF_ERR_BAD_INPUT; }
    }
    return SCF_OK;
}

AsmArgs asm_args(scf_ctx *ctx)
{
    AsmArgs a;
    a.d = ctx->d;
    a.pdx = ctx->pdx; a.pdy = ctx->pdy; a.pdz = ctx->pdz;
    a.udx = ctx->udx; a.vdy = ctx->vdy; a.wdz = ctx->wdz;
    a.phil = ctx->phil; a.vofl = ctx->vofl; a.vof = ctx->vof; a.ee = ctx->ee; a.ne = ctx->ne; a.te = ctx->te;
    a.vofo = ctx->vofo; a.us = ctx->us; a.vs = ctx->vs; a.ws = ctx->ws;
    a.dpu = ctx->dpu; a.dpv = ctx->dpv; a.dpw = ctx->dpw;
    a.ct = ctx->ct; a.pos = ctx->pos; a.ext_cell = ctx->ext_cell;
    for (int q = 0; q < 6; ++q) { a.flag[q] = ctx->bcp_flag[q]; a.bvar[q] = ctx->bvar[q]; }
    const double rho_ref = ctx->opts.rho_ref > 0.0 ? ctx->opts.rho_ref : ctx->opts.rho_l;
    a.dt = ctx->dt;
    a.betap = 1.0 / (ctx->opts.rho_l / rho_ref);
    a.betam = 1.0 / (ctx->opts.rho_g / rho_ref);
    a.epsi = ctx->opts.epsi;
    a.tol = ctx->opts.gfm_tol;
    a.stale_init = ctx->opts.stale_init;
    a.pocoef = ctx->pocoef;
    a.stale_count = ctx->stale_count; a.stale_cap = ctx->stale_cap; a.stale_list = ctx->stale_list;
    a.col_val = ctx->col_val; a.col_mask = ctx->col_mask; a.grp_val = ctx->grp_val; a.grp_mask = ctx->grp_mask;
    a.flags = ctx->flags;
    a.phase = ctx->phase;
    a.rdt = 1.0 / ctx->dt;
    return a;
}

LevelView<double> fine_view(scf_ctx *ctx)
{
    LevelView<double> v;
    v.n0 = ctx->d.I; v.n1 = ctx->d.J; v.n2 = ctx->d.K;
    v.sy = ctx->d.gx; v.sz = ctx->d.gx * ctx->d.gy;
    v.diag = ctx->diag; v.dinv = ctx->dinv; v.cE = ctx->cE; v.cN = ctx->cN; v.cT = ctx->cT;
    return v;
}

int assemble(scf_ctx *ctx)
{
    int rc = ensure_mg(ctx);
    if (rc) return rc;
    CK(cudaMemsetAsync(ctx->flags, 0, sizeof(unsigned), ctx->st));
    AsmArgs a = asm_args(ctx);
    OpArgs o;
    o.diag = ctx->diag; o.dinv = ctx->dinv; o.cE = ctx->cE; o.cN = ctx->cN; o.cT = ctx->cT;
    o.extra = ctx->extra; o.b = ctx->b; o.active = ctx->active;
    const bool mixed = ctx->opts.precision == SCF_PREC_MIXED;
    o.diag32 = ctx->diag32; o.cE32 = ctx->cE32; o.cN32 = ctx->cN32; o.cT32 = ctx->cT32;
    o.diag_lo = ctx->diag_lo; o.cE_lo = ctx->cE_lo; o.cN_lo = ctx->cN_lo; o.cT_lo = ctx->cT_lo;
    o.extra32 = ctx->extra32;
    const double rho_ref = ctx->opts.rho_ref > 0.0 ? ctx->opts.rho_ref : ctx->opts.rho_l;
    int e = launch_assemble(a, o, mixed, ctx->use_rho ? ctx->adj_rho : nullptr, rho_ref, ctx->st, ctx->h_u32,
                            &ctx->launches);
    if (e) { set_err(ctx, "assembly launch: %s", cudaGetErrorString((cudaError_t)e)); return SCF_ERR_CUDA; }
    rc = check_flags(ctx);
    if (rc) return rc;
    ctx->assembled = true;
    return SCF_OK;
}

template <typename T>
int build_hierarchy(scf_ctx *ctx, MgLevel<T> *L)
{
    for (int l = 0; l + 1 < ctx->nlev; ++l) mg_coarsen<T>(L[l], L[l + 1], ctx->st, &ctx->launches);
    CK(cudaEventRecord(ctx->inv_start, ctx->st));
    CK(cudaStreamWaitEvent(ctx->ist, ctx->inv_start, 0));
    mg_coarse_inverse<T>(L[ctx->nlev - 1], ctx->ainv, ctx->map, ctx->ncoarse, is_singular(ctx), ctx->ist,
                         &ctx->launches);
    CK(cudaEventRecord(ctx->inv_ready, ctx->ist));
    ctx->inv_pending = true;
    return SCF_OK;
}

// Stream order after the coarsest inverse, outside any capture.
int join_inverse(scf_ctx *ctx)
{
    if (ctx->inv_pending) {
        CK(cudaStreamWaitEvent(ctx->st, ctx->inv_ready, 0));
        ctx->inv_pending = false;
    }
    return SCF_OK;
}

ChebCoef cheb_coef(int degree, int lines)
{
    ChebCoef cc;
    cc.lines = lines;
    if (degree < 1) degree = 1;
    if (degree > 8) degree = 8;
    cc.degree = degree;
    // interval [lmax/r, lmax]: lmax = 2 bounds the spectrum of D^-1 A
    // (Gershgorin); higher degrees damp a wider band, r = max(6, 2 degree)
    const double lmax = 2.0, lmin = lmax / (degree > 3 ? 2.0 * degree : 6.0);
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin), sigma = theta / delta;
    cc.first = 1.0 / theta;
    double rho = 1.0 / sigma;
    for (int s = 1; s < degree; ++s) {
        const double rn = 1.0 / (2.0 * sigma - rho);
        cc.c1[s] = rn * rho;
        cc.c2[s] = 2.0 * rn / delta;
        rho = rn;
    }
    return cc;
}

double read_scal(scf_ctx *ctx, int slot)
{
    cudaMemcpyAsync(ctx->h_scal, ctx->R.scal + slot, sizeof(double), cudaMemcpyDeviceToHost, ctx->st);
    cudaStreamSynchronize(ctx->st);
    return ctx->h_scal[0];
}

// Algorithmic bytes of one fine-level launch of a kernel class: each array
// counted once per cell; FP32 levels derive 1/diag, FP64 levels read dinv.
double kernel_bytes(const scf_ctx *ctx, int kernel)
{
    const bool mixed = ctx->opts.precision == SCF_PREC_MIXED;
    const double s = mixed ? 4.0 : 8.0;
    const double n = (double)ctx->d.n;
    switch (kernel) {
    case SCF_K_SMOOTH: return (mixed ? 9.0 : 10.0) * s * n;               // b,x,d,diag,[dinv],cE,cN,cT in; x,d out
    case SCF_K_SPMV: return 6.0 * 8.0 * n;                                // p,diag,cE,cN,cT in; q out
    case SCF_K_RESTRICT: return 6.0 * s * n + s * n / 8.0;                // b,x,diag,cE,cN,cT in; coarse b out
    case SCF_K_PROLONG: return (mixed ? 8.0 : 9.0) * s * n + s * n / 8.0; // + coarse e; x,d out
    case SCF_K_CGUPDATE: return (mixed ? 60.0 : 64.0) * n;                // x,r,p,q,diag|dinv in; x,r,[rlow],x0 out
    case SCF_K_SMOOTH2:                                                  // b,x,d,diag,cE,cN,cT in; x out
        return mixed && ctx->d.I % 2 == 0 ? 8.0 * s * n : -1.0;        // (rows of whole pairs: even I)
    default: return -1.0;
    }
}

// Adds the elapsed times of event pairs [a, b) to the per-class totals.
void kt_add(scf_ctx *ctx, int a, int b)
{
    for (int i = a; i < b; ++i) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, ctx->kt.ev[2 * i], ctx->kt.ev[2 * i + 1]) == cudaSuccess) {
            const int c = ctx->kt.cls[i];
            ctx->kt_ms[c] += ms;
            ctx->kt_launches[c] += 1.0;
            ctx->kt_bytes[c] += ctx->kt.bytes[i] >= 0.0 ? ctx->kt.bytes[i] : kernel_bytes(ctx, c);
        }
    }
    cudaGetLastError();
}

// Eagerly recorded pairs (after the stream has been synchronised).
void kt_harvest(scf_ctx *ctx)
{
    if (!ctx->kt.on || ctx->kt.n == 0) return;
    cudaEventSynchronize(ctx->kt.ev[2 * ctx->kt.n - 1]);
    kt_add(ctx, 0, ctx->kt.n);
    ctx->kt.n = 0;
}

// The pairs of the captured iteration graph, after one replay has finished.
void kt_harvest_graph(scf_ctx *ctx)
{
    if (ctx->kt.on && ctx->kt.ng > KTimer::EAGER) kt_add(ctx, KTimer::EAGER, ctx->kt.ng);
}

// Line blocks for the smoother: always (1), never (0), or (2) on FP32
// V-cycles of grids whose smallest z spacing is at most half the larger of
// the x and y spacings, where the k-couplings outweigh the weaker in-plane
// ones at least fourfold.  (FP64 V-cycles are bound by FP64 arithmetic, and
// the line solve's division per cell costs more there than the iterations it
// saves.)
bool use_lines(const scf_ctx *ctx)
{
    if (ctx->opts.smoother_lines == 1) return true;
    if (ctx->opts.smoother_lines == 0) return false;
    return ctx->opts.precision == SCF_PREC_MIXED && ctx->aniso_z >= 4.0;
}

ChebCoef cheb_for(const scf_ctx *ctx) { return cheb_coef(ctx->opts.smoother_degree, use_lines(ctx) ? 1 : 0); }

// The CG update writes level 0's first (point-Jacobi) smoothing step of the
// next V-cycle when the hierarchy has more than one level; with line blocks
// the V-cycle forms that step itself.
bool fuse_first(const scf_ctx *ctx) { return ctx->nlev > 1 && !use_lines(ctx); }

template <typename T>
T *precondition(scf_ctx *ctx, MgLevel<T> *L, const ChebCoef &cc, bool first_done)
{
    // the first V-cycle after a new hierarchy waits for the coarsest inverse
    // just before its coarsest solve
    cudaEvent_t ready = ctx->inv_pending ? ctx->inv_ready : nullptr;
    ctx->inv_pending = false;
    return mg_vcycle<T>(L, ctx->nlev, cc, ctx->ainv, ctx->map, ctx->ncoarse, is_singular(ctx), first_done,
                        ctx->st, &ctx->launches, ctx->kt.on ? &ctx->kt : nullptr, ready);
}

// Fine operator of the mixed CG in double-float form.
DfOp df_view(scf_ctx *ctx)
{
    DfOp D;
    D.hi = ctx->L32[0].view();
    D.dlo = ctx->diag_lo; D.elo = ctx->cE_lo; D.nlo = ctx->cN_lo; D.tlo = ctx->cT_lo;
    return D;
}

// beta from (r, z): FP64 vectors, or (mixed) the double-float r with the
// FP32 z, both in FP64 arithmetic.
template <typename T>
void cg_beta(scf_ctx *ctx, const T *z)
{
    if constexpr (sizeof(T) == 4)
        df_dot_rz(df_view(ctx), (const float2 *)ctx->r, z, ctx->R, ctx->st, &ctx->launches);
    else
        cg_dot_rz<double>(fine_view(ctx), ctx->r, ctx->r, z, ctx->R, ctx->st, &ctx->launches);
}

// New search direction p = z + beta p: FP64 vectors, or (mixed) double-float
// vectors held in the same buffers.
template <typename T>
void cg_direction(scf_ctx *ctx, const T *z, bool first)
{
    if constexpr (sizeof(T) == 4)
        df_pupdate(df_view(ctx), z, (float2 *)ctx->p, ctx->R.scal, first, ctx->st, &ctx->launches);
    else
        cg_pupdate<double>(fine_view(ctx), z, ctx->p, ctx->R.scal, first, ctx->st, &ctx->launches);
}

// SpMV with (p, Ap) and the x/r update with (r, r); the update also writes
// level 0's first smoothing step when fuse_first() holds.
template <typename T>
void cg_step(scf_ctx *ctx, MgLevel<T> *L, const ChebCoef &cc, bool singular, KTimer *kt)
{
    const bool fuse = fuse_first(ctx);
    if constexpr (sizeof(T) == 4) {
        const DfOp D = df_view(ctx);
        df_spmv_dot(D, (const float2 *)ctx->p, (float2 *)ctx->q, ctx->R, singular, ctx->st, &ctx->launches, kt);
        df_cg_update(D, (float2 *)ctx->x, (float2 *)ctx->r, (const float2 *)ctx->p, (const float2 *)ctx->q,
                     L[0].b, fuse ? L[0].x : nullptr, cc.first, ctx->R, ctx->st, &ctx->launches, kt);
    } else {
        const LevelView<double> A = fine_view(ctx);
        cg_spmv_dot(A, ctx->p, ctx->q, ctx->R, singular, ctx->st, &ctx->launches, kt);
        cg_update<double>(A, ctx->x, ctx->r, ctx->p, ctx->q, nullptr, L[0].view(), fuse ? L[0].x : nullptr,
                          cc.first, ctx->R, ctx->st, &ctx->launches, kt);
    }
}

// The part of a CG iteration after the stopping test: precondition, new
// search direction, SpMV with (p, Ap) and the x/r update with (r, r).  Its
// kernel sequence is fixed for a context, so it is captured once as a CUDA
// graph and replayed (one launch instead of ~50, which matters on the small
// coarse levels); the capture is redone when anything it bakes in changes.
template <typename T>
void iteration_kernels(scf_ctx *ctx, MgLevel<T> *L, const ChebCoef &cc, bool singular)
{
    KTimer *kt = ctx->kt.on ? &ctx->kt : nullptr;
    T *z = precondition<T>(ctx, L, cc, fuse_first(ctx));
    cg_beta<T>(ctx, z);
    cg_direction<T>(ctx, z, false);
    cg_step<T>(ctx, L, cc, singular, kt);
}

template <typename T>
void run_iteration(scf_ctx *ctx, MgLevel<T> *L, const ChebCoef &cc, bool singular)
{
    const unsigned long long key = 1ull + (unsigned long long)ctx->mg_gen * 1000003ull +
                                   (unsigned long long)cc.degree * 131ull + (singular ? 7ull : 0ull) +
                                   (ctx->kt.on ? 3ull : 0ull) + (sizeof(T) == 4 ? 11ull : 0ull) +
                                   (unsigned long long)ctx->nlev * 17ull + (cc.lines ? 5ull : 0ull) +
                                   (unsigned long long)smoother_pairs_state() * 7919ull;
    if (ctx->inv_pending) join_inverse(ctx);   // (a captured V-cycle cannot wait on it)
    if (ctx->graphs_ok && (!ctx->iter_exec || ctx->iter_key != key)) {
        if (ctx->iter_exec) { cudaGraphExecDestroy(ctx->iter_exec); ctx->iter_exec = nullptr; }
        cudaGraph_t g = nullptr;
        const int before = ctx->launches;
        ctx->kt.ng = KTimer::EAGER;
        ctx->kt.capturing = ctx->kt.on;
        bool ok = cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) iteration_kernels<T>(ctx, L, cc, singular);
        ok = (cudaStreamEndCapture(ctx->st, &g) == cudaSuccess) && ok && g;
        ctx->kt.capturing = false;
        ctx->iter_launches = ctx->launches - before;
        ctx->launches = before;
        if (ok) ok = cudaGraphInstantiate(&ctx->iter_exec, g, 0) == cudaSuccess;
        if (g) cudaGraphDestroy(g);
        if (!ok) {
            cudaGetLastError();
            if (ctx->iter_exec) { cudaGraphExecDestroy(ctx->iter_exec); ctx->iter_exec = nullptr; }
            ctx->graphs_ok = false;
            ctx->kt.ng = KTimer::EAGER;
        } else {
            ctx->iter_key = key;
        }
    }
    if (ctx->graphs_ok && ctx->iter_exec && cudaGraphLaunch(ctx->iter_exec, ctx->st) == cudaSuccess) {
        ctx->launches += ctx->iter_launches;
        return;
    }
    cudaGetLastError();
    ctx->kt.ng = KTimer::EAGER;
    iteration_kernels<T>(ctx, L, cc, singular);
}

// Iterations without a new smallest CG residual after which a round of the
// solve ends (the tolerance is below what FP64 can reach for the system).
constexpr int kStallWindow = 50;

template <typename T>
int solve_impl(scf_ctx *ctx, MgLevel<T> *L, scf_stats *stats)
{
    const LevelView<double> A = fine_view(ctx);
    const bool singular = is_singular(ctx);
    const bool mixed = sizeof(T) == 4;
    float *rlow = mixed ? (float *)L[0].b : nullptr;
    const ChebCoef cc = cheb_for(ctx);
    auto t0 = std::chrono::steady_clock::now();
    rhs_prologue(A, ctx->active, ctx->b, singular, ctx->R, ctx->st, &ctx->launches);
    {
        const int rh = build_hierarchy<T>(ctx, L);
        if (rh) return rh;
    }
    const double bb = read_scal(ctx, S_BB);
    const double bn = std::sqrt(bb);
    stats->rhs_norm = bn;
    stats->singular = singular ? 1 : 0;
    stats->levels = ctx->nlev;
    int its = 0;
    double rel = 0.0;
    if (!(bn > 0.0)) {
        CK(cudaMemsetAsync(ctx->x, 0, sizeof(double) * ctx->d.ng, ctx->st));
        CK(cudaMemsetAsync(ctx->R.scal + S_MEANX, 0, sizeof(double), ctx->st));
        stats->iterations = 0;
        stats->rounds = 1;
        stats->rel_residual = 0.0;
        stats->converged = 1;
        return std::isfinite(bb) ? SCF_OK : SCF_ERR_NONFINITE;
    }
    if (ctx->opts.warm_start && ctx->warm_ok) {
        final_residual(A, ctx->active, ctx->b, ctx->x, ctx->r, false, ctx->R, ctx->st, &ctx->launches);
    } else {
        CK(cudaMemsetAsync(ctx->x, 0, sizeof(double) * ctx->d.ng, ctx->st));
        CK(cudaMemcpyAsync(ctx->r, ctx->b, sizeof(double) * ctx->d.ng, cudaMemcpyDeviceToDevice, ctx->st));
    }
    const double tol = ctx->opts.rel_tol;
    int restarts = 0;
    bool stalled = false, have_best = false;
    double best_rel = HUGE_VAL;
    const int ng = ctx->d.ng;
    // x is zero before a cold first round; the double-float zero has the
    // same bits as the FP64 zero, so that x needs no conversion
    bool x_zero = !(ctx->opts.warm_start && ctx->warm_ok);
    for (;;) {
        if (mixed) {
            // x and r (FP64 here) become double-float for the round, and r's
            // FP32 copy is the V-cycle's right-hand side
            if (!x_zero) df_from_double(ctx->x, (float2 *)ctx->x, ng, ctx->st, &ctx->launches);
            df_round_start(ctx->r, rlow, ng, ctx->st, &ctx->launches);
        }
        x_zero = false;
        T *z = precondition<T>(ctx, L, cc, false);
        cg_beta<T>(ctx, z);
        cg_direction<T>(ctx, z, true);
        bool conv = false;
        stalled = false;
        double best = HUGE_VAL;
        int best_it = its;
        bool replayed = false;
        if (its < ctx->opts.max_iter) {
            ++its;
            cg_step<T>(ctx, L, cc, singular, ctx->kt.on ? &ctx->kt : nullptr);
        }
        while (true) {
            const double rr = read_scal(ctx, S_RR);
            if (replayed) kt_harvest_graph(ctx);
            if (!std::isfinite(rr)) {
                set_err(ctx, "CG residual became non-finite at iteration %d", its);
                stats->iterations = its;
                return SCF_ERR_NONFINITE;
            }
            if (std::sqrt(rr) <= tol * bn) { conv = true; break; }
            // Below the rounding floor of the system (where the recursive
            // residual has left the true one behind) the recursion turns
            // around and grows: stop at a tenfold rise over the smallest
            // residual of this round, or after a long stretch without a new
            // smallest one, and restart from the true residual.
            if (rr < best) { best = rr; best_it = its; }
            else if (rr > 100.0 * best || its - best_it >= kStallWindow) { stalled = true; break; }
            const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (el > ctx->opts.time_limit_s || its >= ctx->opts.max_iter) break;
            run_iteration<T>(ctx, L, cc, singular);
            replayed = ctx->graphs_ok && ctx->iter_exec;
            ++its;
        }
        // true FP64 residual (the refinement check); for an all-Neumann
        // system also the mean of x, removed below
        if (mixed) df_to_double((const float2 *)ctx->x, ctx->x, ng, ctx->st, &ctx->launches);
        final_residual(A, ctx->active, ctx->b, ctx->x, ctx->r, singular, ctx->R, ctx->st, &ctx->launches);
        rel = std::sqrt(read_scal(ctx, S_RR)) / bn;
        if (rel <= tol || !(conv || stalled) || its >= ctx->opts.max_iter || restarts >= ctx->opts.max_rounds)
            break;
        // recursive residual drifted away from the true one: restart from the
        // true residual, keeping the best round-end iterate
        if (rel < best_rel) {
            best_rel = rel;
            CK(cudaMemcpyAsync(ctx->xbest, ctx->x, sizeof(double) * ctx->d.ng, cudaMemcpyDeviceToDevice, ctx->st));
            have_best = true;
        }
        ++restarts;
    }
    if (have_best && rel > best_rel) {
        CK(cudaMemcpyAsync(ctx->x, ctx->xbest, sizeof(double) * ctx->d.ng, cudaMemcpyDeviceToDevice, ctx->st));
        final_residual(A, ctx->active, ctx->b, ctx->x, ctx->r, singular, ctx->R, ctx->st, &ctx->launches);
        rel = std::sqrt(read_scal(ctx, S_RR)) / bn;
    }
    if (singular) shift_solution(A, ctx->active, ctx->x, ctx->R.scal, ctx->st, &ctx->launches);
    kt_harvest(ctx);
    if (mixed) {
        // the two-step smoother's bounded waits for its own copies
        CK(cudaMemcpyAsync(ctx->h_u32, ctx->flags, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        if (*ctx->h_u32 & FLAG_WAIT_TIMEOUT) {
            set_err(ctx, "a smoother kernel gave up waiting for its shared-memory copies");
            return SCF_ERR_CUDA;
        }
    }
    stats->iterations = its;
    stats->rounds = restarts + 1;
    stats->rel_residual = rel;
    stats->converged = rel <= tol ? 1 : 0;
    if (!stats->converged) {
        set_err(ctx, "not converged: relative residual %.3e after %d iterations (tolerance %.1e)%s", rel, its, tol,
                stalled ? "; the residual stopped decreasing at the rounding floor" : "");
        return SCF_ERR_NOT_CONVERGED;
    }
    return SCF_OK;
}

CorrArgs corr_args(scf_ctx *ctx)
{
    CorrArgs a;
    a.d = ctx->d;
    a.x = ctx->x; a.ct = ctx->ct; a.pp = ctx->pp; a.pocoef = ctx->pocoef;
    a.us = ctx->us; a.vs = ctx->vs; a.ws = ctx->ws;
    a.umoex = ctx->umoex; a.uct = ctx->uct; a.vmoex = ctx->vmoex; a.vct = ctx->vct;
    a.wmoex = ctx->wmoex; a.wct = ctx->wct;
    a.u = ctx->tu; a.v = ctx->tv; a.w = ctx->tw; a.p = ctx->tp;
    a.pdx = ctx->pdx; a.pdy = ctx->pdy; a.pdz = ctx->pdz;
    a.ee = ctx->ee; a.ne = ctx->ne; a.te = ctx->te;
    for (int q = 0; q < 6; ++q) {
        a.bcp_flag[q] = ctx->bcp_flag[q];
        a.flag[0][q] = ctx->corr.bcu_flag[q]; a.flag[1][q] = ctx->corr.bcv_flag[q];
        a.flag[2][q] = ctx->corr.bcw_flag[q]; a.flag[3][q] = ctx->bcp_flag[q];
        a.cst[0][q] = ctx->corr.bcu_const[q]; a.cst[1][q] = ctx->corr.bcv_const[q];
        a.cst[2][q] = ctx->corr.bcw_const[q]; a.cst[3][q] = ctx->corr.bcp_const[q];
        for (int f = 0; f < 4; ++f) a.bcvar[f][q] = ctx->bcvar[f][q];
    }
    a.north_fix = ctx->opts.north_mass_fix;
    a.flags = ctx->flags;
    return a;
}

size_t plane_size(const Dims &d, int face)
{
    const int axis = face >> 1;
    return axis == 0 ? (size_t)d.J * d.K : axis == 1 ? (size_t)d.I * d.K : (size_t)d.I * d.J;
}

int check_ctx(scf_ctx *ctx)
{
    if (!ctx) return SCF_ERR_BAD_ARG;
    cudaError_t e = cudaSetDevice(ctx->opts.device);
    if (e != cudaSuccess) { set_err(ctx, "cudaSetDevice: %s", cudaGetErrorString(e)); return SCF_ERR_CUDA; }
    return SCF_OK;
}

int run(scf_ctx *ctx, bool with_correction, scf_stats *stats)
{
    scf_stats local;
    if (!stats) stats = &local;
    memset(stats, 0, sizeof(*stats));
    if (!ctx->staged) { set_err(ctx, "no inputs staged"); return SCF_ERR_NO_SOLVE; }
    if (with_correction && !ctx->have_corr) { set_err(ctx, "no correction inputs staged"); return SCF_ERR_BAD_ARG; }
    if (with_correction && ctx->bcp_flag[0] != 0 && ctx->bcp_flag[1] != 0 && ctx->bcp_flag[2] != 0 &&
        ctx->bcp_flag[3] == 0 && !ctx->opts.north_mass_fix) {
        set_err(ctx, "the reference's North-face mass correction (ComputePUVW.f90:323-341) has no defined "
                     "result (stale k, PGrid indexed out of bounds); set opts.north_mass_fix = 1 for the "
                     "evident intent");
        return SCF_ERR_UNDEFINED_IN_REFERENCE;
    }
    ctx->launches = 0;
    cudaEventRecord(ctx->ev[0], ctx->st);
    int rc = assemble(ctx);
    if (rc) return rc;
    cudaEventRecord(ctx->ev[1], ctx->st);
    if (ctx->opts.precision == SCF_PREC_FP64)
        rc = solve_impl<double>(ctx, ctx->L64, stats);
    else
        rc = solve_impl<float>(ctx, ctx->L32, stats);
    cudaEventRecord(ctx->ev[2], ctx->st);
    if (rc && rc != SCF_ERR_NOT_CONVERGED) return rc;
    const int solve_rc = rc;
    ctx->solved = true;
    ctx->warm_ok = true;
    CorrArgs ca = corr_args(ctx);
    if (ctx->corr_pending) {
        CK(cudaStreamWaitEvent(ctx->st, ctx->corr_ready, 0));
        ctx->corr_pending = false;
    }
    launch_scatter(ca, ctx->st, &ctx->launches);
    if (with_correction) launch_correct(ca, ctx->st, &ctx->launches);
    cudaEventRecord(ctx->ev[3], ctx->st);
    CK(cudaEventSynchronize(ctx->ev[3]));
    CK(cudaGetLastError());
    float ms;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]); stats->ms_assemble = ms;
    cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]); stats->ms_solve = ms;
    cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]); stats->ms_correct = ms;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[3]); stats->ms_total = ms;
    stats->gpu_launches = ctx->launches;
    return solve_rc;
}

// Blocks of the copy kernels that bring the correction's inputs in on the
// second stream while the solve runs: enough to move them within the solve
// (about 1 GB in 16 ms at 256^3), few enough to leave the SMs to the solve.
constexpr int kSideCopyBlocks = 64;

// One input array to the device: by a copy kernel when the caller's array
// is page-locked and device-mapped, else by the copy engine (scf_stage.h).
template <typename P>
int h2d(scf_ctx *ctx, P *dst, const P *src, size_t n, int64_t *bytes, cudaStream_t st)
{
    if (!src) { set_err(ctx, "null input array"); return SCF_ERR_BAD_ARG; }
    CK(stage_h2d(dst, src, n * sizeof(P), st, st == ctx->st ? 0 : kSideCopyBlocks, nullptr, nullptr));
    *bytes += (int64_t)(n * sizeof(P));
    return SCF_OK;
}
#define H2D(dst, src, n)                                   \
    do {                                                   \
        int rc_ = h2d(ctx, dst, src, (size_t)(n), &bytes, ctx->st); \
        if (rc_) return rc_;                               \
    } while (0)

// defer_corr: the correction's inputs go to the device on the copy stream
// and overlap the assembly and solve; run() orders the correction after
// them.  Only for callers that keep the host arrays alive until the
// projection has finished (scf_update_puvw).
int stage(scf_ctx *ctx, const scf_poisson_in *in, const scf_correct_in *corr, const double *u, const double *v,
          const double *w, const double *p, int64_t *bytes_out, bool defer_corr = false)
{
    if (!in) { set_err(ctx, "null scf_poisson_in"); return SCF_ERR_BAD_ARG; }
    const Dims &d = ctx->d;
    int64_t bytes = 0;
    for (int q = 0; q < 6; ++q) {
        if (in->bcp_flag[q] != 0 && in->bcp_flag[q] != 1) { set_err(ctx, "BCp flag %d is %d (0 or 1 expected)", q + 1, in->bcp_flag[q]); return SCF_ERR_BAD_ARG; }
    }
    if (!(in->dt > 0.0) || !std::isfinite(in->dt)) { set_err(ctx, "dt must be positive and finite"); return SCF_ERR_BAD_ARG; }
    if (in->pcell_extcell < -1 || in->pcell_extcell >= d.n) { set_err(ctx, "ExtCell %d out of range", in->pcell_extcell); return SCF_ERR_BAD_ARG; }
    H2D(ctx->pdx, in->pgrid_dx, d.n); H2D(ctx->pdy, in->pgrid_dy, d.n); H2D(ctx->pdz, in->pgrid_dz, d.n);
    H2D(ctx->udx, in->ugrid_dx, d.n); H2D(ctx->vdy, in->vgrid_dy, d.n); H2D(ctx->wdz, in->wgrid_dz, d.n);
    H2D(ctx->phil, in->pcell_phil, d.ng); H2D(ctx->vofl, in->pcell_vofl, d.ng); H2D(ctx->vof, in->pcell_vof, d.ng);
    H2D(ctx->ee, in->pcell_eearea, d.ng); H2D(ctx->ne, in->pcell_nearea, d.ng); H2D(ctx->te, in->pcell_tearea, d.ng);
    H2D(ctx->ct, in->pcell_cell_type, d.n); H2D(ctx->pos, in->pcell_posnu, d.n);
    H2D(ctx->vofo, in->vof_old, d.ng);
    H2D(ctx->us, in->pred_u, d.ng); H2D(ctx->vs, in->pred_v, d.ng); H2D(ctx->ws, in->pred_w, d.ng);
    H2D(ctx->dpu, in->pu_dp, d.ng); H2D(ctx->dpv, in->pv_dp, d.ng); H2D(ctx->dpw, in->pw_dp, d.ng);
    for (int q = 0; q < 6; ++q) {
        ctx->bcp_flag[q] = in->bcp_flag[q];
        if (in->bcp_flag[q] == 0) H2D(ctx->bvar[q], in->bcp_var[q], plane_size(d, q));
    }
    ctx->ext_cell = in->pcell_extcell;
    ctx->dt = in->dt;
    {
        // tensor-product grid: the spacings along the first line of each axis
        double hx = HUGE_VAL, hy = HUGE_VAL, hz = HUGE_VAL;
        for (int i = 0; i < d.I; ++i) hx = std::min(hx, in->pgrid_dx[i]);
        for (int j = 0; j < d.J; ++j) hy = std::min(hy, in->pgrid_dy[(size_t)j * d.I]);
        for (int k = 0; k < d.K; ++k) hz = std::min(hz, in->pgrid_dz[(size_t)k * d.I * d.J]);
        const double h = std::max(hx, hy);
        ctx->aniso_z = (hz > 0.0 && std::isfinite(h)) ? (h / hz) * (h / hz) : 1.0;
    }
    ctx->have_corr = false;
    if (corr) {
        const int *fl[3] = {corr->bcu_flag, corr->bcv_flag, corr->bcw_flag};
        for (int f = 0; f < 3; ++f)
            for (int q = 0; q < 6; ++q)
                if (fl[f][q] != 0 && fl[f][q] != 1) { set_err(ctx, "velocity BC flag must be 0 or 1"); return SCF_ERR_BAD_ARG; }
        if ((u || v || w || p) && !(u && v && w && p)) { set_err(ctx, "null TVar array"); return SCF_ERR_BAD_ARG; }
        const cudaStream_t cs = defer_corr ? ctx->cst : ctx->st;
#define H2DC(dst, src, n)                                               \
    do {                                                                \
        int rc_ = h2d(ctx, dst, src, (size_t)(n), &bytes, cs);          \
        if (rc_) return rc_;                                            \
    } while (0)
        if (defer_corr) {   // the copy stream may not overwrite what a running call still reads
            CK(cudaEventRecord(ctx->corr_ready, ctx->st));
            CK(cudaStreamWaitEvent(ctx->cst, ctx->corr_ready, 0));
        }
        H2DC(ctx->umoex, corr->ucell_moexcell, d.n); H2DC(ctx->uct, corr->ucell_cell_type, d.n);
        H2DC(ctx->vmoex, corr->vcell_moexcell, d.n); H2DC(ctx->vct, corr->vcell_cell_type, d.n);
        H2DC(ctx->wmoex, corr->wcell_moexcell, d.n); H2DC(ctx->wct, corr->wcell_cell_type, d.n);
        if (u) { H2DC(ctx->tu, u, d.ng); H2DC(ctx->tv, v, d.ng); H2DC(ctx->tw, w, d.ng); H2DC(ctx->tp, p, d.ng); }
#undef H2DC
        if (defer_corr) {
            CK(cudaEventRecord(ctx->corr_ready, ctx->cst));
            ctx->corr_pending = true;
        }
        ctx->corr = *corr;
        ctx->have_corr = true;
    }
    ctx->staged = true;
    ctx->assembled = false;
    ctx->have_loss = false;
    if (bytes_out) *bytes_out = bytes;
    return SCF_OK;
}

template <typename P>
int d2h(scf_ctx *ctx, P *dst, const P *src, size_t n, int64_t *bytes)
{
    if (!dst) return SCF_OK;
    CK(stage_d2h(dst, src, n * sizeof(P), ctx->st, 0, nullptr, nullptr));
    *bytes += (int64_t)(n * sizeof(P));
    return SCF_OK;
}

int fetch(scf_ctx *ctx, double *u, double *v, double *w, double *p, double *pocoef, double *pp, scf_bc_out *bc,
          int64_t *bytes_out)
{
    const Dims &d = ctx->d;
    int64_t bytes = 0;
    int rc;
    if ((rc = d2h(ctx, u, ctx->tu, d.ng, &bytes))) return rc;
    if ((rc = d2h(ctx, v, ctx->tv, d.ng, &bytes))) return rc;
    if ((rc = d2h(ctx, w, ctx->tw, d.ng, &bytes))) return rc;
    if ((rc = d2h(ctx, p, ctx->tp, d.ng, &bytes))) return rc;
    if ((rc = d2h(ctx, pocoef, ctx->pocoef, (size_t)d.n * 6, &bytes))) return rc;
    if ((rc = d2h(ctx, pp, ctx->pp, d.ng, &bytes))) return rc;
    if (bc)
        for (int f = 0; f < 4; ++f)
            for (int q = 0; q < 6; ++q)
                if ((rc = d2h(ctx, bc->var[f][q], ctx->bcvar[f][q], plane_size(d, q), &bytes))) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    if (bytes_out) *bytes_out = bytes;
    return SCF_OK;
}

}  // namespace

// ===========================================================================
extern "C" {

void scf_opts_default(scf_opts *o)
{
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->precision = SCF_PREC_FP64;
    o->rel_tol = 1.0e-10;
    o->max_iter = 500;
    o->max_rounds = 12;
    o->inner_rtol = 1.0e-4;
    o->smoother_degree = 3;
    o->coarse_max_cells = 64;
    o->rho_l = 998.3;
    o->rho_g = 1.205;
    o->rho_ref = 0.0;
    o->epsi = 1.0e-3;
    o->gfm_tol = 1.0e-30;
    o->stale_init = std::nan("");
    o->warm_start = 0;
    o->north_mass_fix = 0;
    o->check_inputs = 1;
    o->device = 0;
    o->time_limit_s = 60.0;
    o->smoother_lines = 2;
}

static int validate_opts(scf_ctx *ctx, const scf_opts *o)
{
    if (o->precision != SCF_PREC_FP64 && o->precision != SCF_PREC_MIXED) { set_err(ctx, "bad precision"); return SCF_ERR_BAD_ARG; }
    if (!(o->rel_tol > 0.0) || o->max_iter < 1 || o->smoother_degree < 1 || o->smoother_degree > 8) { set_err(ctx, "bad solver options"); return SCF_ERR_BAD_ARG; }
    if (o->coarse_max_cells < 8 || o->coarse_max_cells > 128) { set_err(ctx, "coarse_max_cells must be in [8,128]"); return SCF_ERR_BAD_ARG; }
    if (o->smoother_lines < 0 || o->smoother_lines > 2) { set_err(ctx, "smoother_lines must be 0, 1 or 2"); return SCF_ERR_BAD_ARG; }
    if (!(o->rho_l > 0.0) || !(o->rho_g > 0.0)) { set_err(ctx, "densities must be positive"); return SCF_ERR_BAD_ARG; }
    return SCF_OK;
}

int scf_ctx_create(scf_ctx **out, int32_t imax, int32_t jmax, int32_t kmax, const scf_opts *opts)
{
    if (!out) return SCF_ERR_BAD_ARG;
    *out = nullptr;
    if (imax < 2 || jmax < 2 || kmax < 2) return SCF_ERR_BAD_ARG;
    const long long n = (long long)imax * jmax * kmax;
    const long long ng = (long long)(imax + 2) * (jmax + 2) * (kmax + 2);
    if (6 * n >= (1LL << 31) || ng >= (1LL << 31)) return SCF_ERR_BAD_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SCF_ERR_NO_DEVICE;
    scf_ctx *ctx = new scf_ctx();
    if (opts) ctx->opts = *opts; else scf_opts_default(&ctx->opts);
    int rc = validate_opts(ctx, &ctx->opts);
    if (rc) { delete ctx; return rc; }
    if (ctx->opts.device < 0 || ctx->opts.device >= ndev) { delete ctx; return SCF_ERR_BAD_ARG; }
    if (cudaSetDevice(ctx->opts.device) != cudaSuccess) { delete ctx; return SCF_ERR_CUDA; }
    Dims &d = ctx->d;
    d.I = imax; d.J = jmax; d.K = kmax;
    d.gx = imax + 2; d.gy = jmax + 2; d.gz = kmax + 2;
    d.ng = (int)ng; d.n = (int)n;
    auto fail = [&](int code) { scf_ctx_destroy(ctx); return code; };
#define A(ptr, cnt) do { if ((rc = dalloc(ctx, ctx->mem, &(ptr), (size_t)(cnt)))) return fail(rc); } while (0)
    A(ctx->pdx, n); A(ctx->pdy, n); A(ctx->pdz, n); A(ctx->udx, n); A(ctx->vdy, n); A(ctx->wdz, n);
    A(ctx->phil, ng); A(ctx->vofl, ng); A(ctx->vof, ng); A(ctx->ee, ng); A(ctx->ne, ng); A(ctx->te, ng);
    A(ctx->vofo, ng); A(ctx->us, ng); A(ctx->vs, ng); A(ctx->ws, ng);
    A(ctx->dpu, ng); A(ctx->dpv, ng); A(ctx->dpw, ng);
    A(ctx->ct, n); A(ctx->pos, n);
    A(ctx->umoex, n); A(ctx->uct, n); A(ctx->vmoex, n); A(ctx->vct, n); A(ctx->wmoex, n); A(ctx->wct, n);
    A(ctx->tu, ng); A(ctx->tv, ng); A(ctx->tw, ng); A(ctx->tp, ng);
    for (int q = 0; q < 6; ++q) A(ctx->bvar[q], plane_size(d, q));
    A(ctx->pocoef, 6 * n);
    A(ctx->stale_count, 1); A(ctx->flags, 4);
    ctx->stale_cap = (unsigned)(n < (1LL << 30) ? n : (1LL << 30));
    A(ctx->stale_list, ctx->stale_cap);
    // per-segment summaries of the coefficient kernel (segments of 32 cells)
    const long long ncol = (long long)imax * jmax * ((kmax + SCF_KSEG - 1) / SCF_KSEG), ngrp = (ncol + 63) / 64;
    A(ctx->col_val, 12 * ncol); A(ctx->col_mask, ncol); A(ctx->grp_val, 12 * ngrp); A(ctx->grp_mask, ngrp);
    A(ctx->phase, ng);
    A(ctx->diag, ng); A(ctx->dinv, ng); A(ctx->cE, ng); A(ctx->cN, ng); A(ctx->cT, ng); A(ctx->extra, ng);
    A(ctx->b, ng); A(ctx->active, ng);
    A(ctx->x, ng); A(ctx->r, ng); A(ctx->p, ng); A(ctx->q, ng); A(ctx->xbest, ng);
    A(ctx->pp, ng);
    for (int f = 0; f < 4; ++f)
        for (int q = 0; q < 6; ++q) A(ctx->bcvar[f][q], plane_size(d, q));
    Launch3 l = launch_interior(imax, jmax, kmax);
    ctx->R.max_blocks = (int)nblocks(l);
    A(ctx->R.partials, 2 * ctx->R.max_blocks + 1024);
    A(ctx->R.scal, S_NUM);
#undef A
    if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess) return fail(SCF_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&ctx->cst, cudaStreamNonBlocking) != cudaSuccess) return fail(SCF_ERR_CUDA);
    if (cudaEventCreateWithFlags(&ctx->corr_ready, cudaEventDisableTiming) != cudaSuccess) return fail(SCF_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&ctx->ist, cudaStreamNonBlocking) != cudaSuccess) return fail(SCF_ERR_CUDA);
    if (cudaEventCreateWithFlags(&ctx->inv_start, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->inv_ready, cudaEventDisableTiming) != cudaSuccess)
        return fail(SCF_ERR_CUDA);
    for (int e = 0; e < 8; ++e) cudaEventCreate(&ctx->ev[e]);
    if (cudaMallocHost(&ctx->h_scal, 64 * sizeof(double)) != cudaSuccess) return fail(SCF_ERR_OUT_OF_MEMORY);
    if (cudaMallocHost(&ctx->h_u32, 64 * sizeof(unsigned)) != cudaSuccess) return fail(SCF_ERR_OUT_OF_MEMORY);
    rc = ensure_mg(ctx);
    if (rc) return fail(rc);
    if (cudaDeviceSynchronize() != cudaSuccess) return fail(SCF_ERR_CUDA);
    *out = ctx;
    return SCF_OK;
}

int scf_ctx_destroy(scf_ctx *ctx)
{
    if (!ctx) return SCF_OK;
    cudaSetDevice(ctx->opts.device);
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    if (ctx->ist) cudaStreamSynchronize(ctx->ist);
    ctx->mgmem.release();
    ctx->adjmem.release();
    ctx->mem.release();
    for (int e = 0; e < 8; ++e)
        if (ctx->ev[e]) cudaEventDestroy(ctx->ev[e]);
    if (ctx->kt_events)
        for (int e = 0; e < 2 * KTimer::CAP; ++e) cudaEventDestroy(ctx->kt.ev[e]);
    if (ctx->iter_exec) cudaGraphExecDestroy(ctx->iter_exec);
    if (ctx->h_scal) cudaFreeHost(ctx->h_scal);
    if (ctx->h_u32) cudaFreeHost(ctx->h_u32);
    if (ctx->cst) { cudaStreamSynchronize(ctx->cst); cudaStreamDestroy(ctx->cst); }
    if (ctx->corr_ready) cudaEventDestroy(ctx->corr_ready);
    if (ctx->ist) cudaStreamDestroy(ctx->ist);
    if (ctx->inv_start) cudaEventDestroy(ctx->inv_start);
    if (ctx->inv_ready) cudaEventDestroy(ctx->inv_ready);
    if (ctx->st) cudaStreamDestroy(ctx->st);
    delete ctx;
    return SCF_OK;
}

int scf_ctx_set_opts(scf_ctx *ctx, const scf_opts *opts)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!opts) return SCF_ERR_BAD_ARG;
    rc = validate_opts(ctx, opts);
    if (rc) return rc;
    if (opts->device != ctx->opts.device) { set_err(ctx, "the device of a context cannot change"); return SCF_ERR_BAD_ARG; }
    const bool replan = opts->coarse_max_cells != ctx->opts.coarse_max_cells;
    ctx->opts = *opts;
    if (replan) ctx->mg_precision = -1;
    return ensure_mg(ctx);
}

int scf_stage_inputs(scf_ctx *ctx, const scf_poisson_in *in, const scf_correct_in *corr, const double *u,
                     const double *v, const double *w, const double *p)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    rc = stage(ctx, in, corr, u, v, w, p, nullptr);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    return SCF_OK;
}

int scf_run_projection(scf_ctx *ctx, scf_stats *stats)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    return run(ctx, ctx->have_corr, stats);
}

int scf_fetch_outputs(scf_ctx *ctx, double *u, double *v, double *w, double *p, double *pocoef, double *pp,
                      scf_bc_out *bc)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!ctx->solved) { set_err(ctx, "no projection has run"); return SCF_ERR_NO_SOLVE; }
    if ((u || v || w || p || bc) && !ctx->have_corr) { set_err(ctx, "the last run had no correction"); return SCF_ERR_BAD_ARG; }
    return fetch(ctx, u, v, w, p, pocoef, pp, bc, nullptr);
}

int scf_poisson_solve(scf_ctx *ctx, const scf_poisson_in *in, double *pocoef, double *pp, scf_stats *stats)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    scf_stats local;
    if (!stats) stats = &local;
    auto t0 = std::chrono::steady_clock::now();
    int64_t bi = 0, bo = 0;
    rc = stage(ctx, in, nullptr, nullptr, nullptr, nullptr, nullptr, &bi);
    if (rc) return rc;
    rc = run(ctx, false, stats);
    if (rc && rc != SCF_ERR_NOT_CONVERGED) return rc;
    const int solve_rc = rc;
    rc = fetch(ctx, nullptr, nullptr, nullptr, nullptr, pocoef, pp, nullptr, &bo);
    if (rc) return rc;
    stats->bytes_h2d = bi;
    stats->bytes_d2h = bo;
    stats->ms_h2d = 0.0;
    stats->ms_d2h = 0.0;
    stats->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return solve_rc;
}

int scf_update_puvw(scf_ctx *ctx, const scf_poisson_in *in, const scf_correct_in *corr, double *u, double *v,
                    double *w, double *p, scf_bc_out *bc, scf_stats *stats)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!corr || !u || !v || !w || !p) { set_err(ctx, "null correction argument"); return SCF_ERR_BAD_ARG; }
    scf_stats local;
    if (!stats) stats = &local;
    auto t0 = std::chrono::steady_clock::now();
    int64_t bi = 0, bo = 0;
    cudaEventRecord(ctx->ev[6], ctx->st);
    rc = stage(ctx, in, corr, u, v, w, p, &bi, true);
    if (rc) { cudaStreamSynchronize(ctx->cst); ctx->corr_pending = false; return rc; }
    cudaEventRecord(ctx->ev[7], ctx->st);
    rc = run(ctx, true, stats);
    if (rc && rc != SCF_ERR_NOT_CONVERGED) {
        // the caller's arrays may go away on return: finish the copies first
        cudaStreamSynchronize(ctx->cst);
        ctx->corr_pending = false;
        return rc;
    }
    const int solve_rc = rc;
    float h2d_ms = 0.f;
    cudaEventElapsedTime(&h2d_ms, ctx->ev[6], ctx->ev[7]);
    cudaEventRecord(ctx->ev[6], ctx->st);
    rc = fetch(ctx, u, v, w, p, nullptr, nullptr, bc, &bo);
    if (rc) return rc;
    cudaEventRecord(ctx->ev[7], ctx->st);
    cudaEventSynchronize(ctx->ev[7]);
    float d2h_ms = 0.f;
    cudaEventElapsedTime(&d2h_ms, ctx->ev[6], ctx->ev[7]);
    stats->ms_h2d = h2d_ms;
    stats->ms_d2h = d2h_ms;
    stats->bytes_h2d = bi;
    stats->bytes_d2h = bo;
    stats->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return solve_rc;
}

// ---------------------------------------------------------------------------
// loss and adjoint
namespace {

AdjArgs adj_args(scf_ctx *ctx)
{
    AdjArgs A;
    A.d = ctx->d;
    A.us = ctx->us; A.vs = ctx->vs; A.ws = ctx->ws;
    A.pp = ctx->pp; A.pfwd = ctx->adj_pfwd; A.pocoef = ctx->pocoef;
    A.umoex = ctx->umoex; A.uct = ctx->uct; A.vmoex = ctx->vmoex; A.vct = ctx->vct;
    A.wmoex = ctx->wmoex; A.wct = ctx->wct; A.ct = ctx->ct;
    A.ee = ctx->ee; A.ne = ctx->ne; A.te = ctx->te;
    A.pdx = ctx->pdx; A.pdy = ctx->pdy; A.pdz = ctx->pdz;
    A.gw = ctx->adj_g; A.r = ctx->adj_r;
    A.phase = ctx->phase; A.phil = ctx->phil; A.tol = ctx->opts.gfm_tol;
    return A;
}

int alloc_adj(scf_ctx *ctx)
{
    const int ng = ctx->d.ng;
    DALLOC(ctx->adjmem, ctx->adj_rho, ng);
    DALLOC(ctx->adjmem, ctx->adj_g, ng);
    DALLOC(ctx->adjmem, ctx->adj_r, ng);
    DALLOC(ctx->adjmem, ctx->adj_pfwd, ng);
    DALLOC(ctx->adjmem, ctx->adj_gu, ng);
    DALLOC(ctx->adjmem, ctx->adj_gv, ng);
    DALLOC(ctx->adjmem, ctx->adj_gw, ng);
    DALLOC(ctx->adjmem, ctx->adj_grho, ng);
    return SCF_OK;
}

// The adjoint's buffers, allocated on first use; all or none (a failed
// allocation releases the ones made, so a later call starts over).
int ensure_adj(scf_ctx *ctx)
{
    if (ctx->adj_grho) return SCF_OK;
    const int rc = alloc_adj(ctx);
    if (rc) {
        ctx->adjmem.release();
        ctx->adj_rho = ctx->adj_g = ctx->adj_r = ctx->adj_pfwd = nullptr;
        ctx->adj_gu = ctx->adj_gv = ctx->adj_gw = ctx->adj_grho = nullptr;
    }
    return rc;
}

}  // namespace

extern "C" int scf_loss_forward(scf_ctx *ctx, const scf_poisson_in *in, const scf_correct_in *corr,
                                const double *rho_cell, const double *g, double *J, scf_stats *stats)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!in || !corr || !g || !J) { set_err(ctx, "null argument"); return SCF_ERR_BAD_ARG; }
    for (int q = 0; q < 6; ++q)
        if (in->bcp_flag[q] != 1) {
            set_err(ctx, "the loss gradient supports all-Neumann pressure boundaries only");
            return SCF_ERR_BAD_ARG;
        }
    if ((rc = ensure_adj(ctx))) return rc;
    scf_stats local;
    if (!stats) stats = &local;
    rc = stage(ctx, in, corr, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (rc) return rc;
    const Dims &d = ctx->d;
    // g (interior) -> ghosted device array
    std::vector<double> gg(d.ng, 0.0);
    for (int k = 1; k <= d.K; ++k)
        for (int j = 1; j <= d.J; ++j)
            for (int i = 1; i <= d.I; ++i) gg[gidx(d, i, j, k)] = g[nidx(d, i, j, k)];
    CK(cudaMemcpyAsync(ctx->adj_g, gg.data(), sizeof(double) * d.ng, cudaMemcpyHostToDevice, ctx->st));
    if (rho_cell) {
        CK(cudaMemcpyAsync(ctx->adj_rho, rho_cell, sizeof(double) * d.ng, cudaMemcpyHostToDevice, ctx->st));
        ctx->use_rho = true;
    } else {
        ctx->use_rho = false;
    }
    CK(cudaStreamSynchronize(ctx->st));
    ctx->warm_ok = false;
    rc = run(ctx, false, stats);   // coefficients, operator, solve, scatter
    ctx->use_rho = false;
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->adj_pfwd, ctx->pp, sizeof(double) * d.ng, cudaMemcpyDeviceToDevice, ctx->st));
    AdjArgs A = adj_args(ctx);
    launch_adj_divergence(A, ctx->R, ctx->st, &ctx->launches);
    CK(cudaMemcpyAsync(ctx->h_scal, ctx->R.scal + S_JP, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    J[0] = ctx->h_scal[0];
    J[1] = ctx->h_scal[1];
    ctx->have_loss = true;
    ctx->rho_given_last = rho_cell != nullptr;
    return SCF_OK;
}

extern "C" int scf_loss_backward(scf_ctx *ctx, double *grad_u, double *grad_v, double *grad_w, double *grad_rho,
                                 scf_stats *stats)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!ctx->have_loss) { set_err(ctx, "scf_loss_backward needs a preceding scf_loss_forward"); return SCF_ERR_NO_SOLVE; }
    scf_stats local;
    if (!stats) stats = &local;
    memset(stats, 0, sizeof(*stats));
    const Dims &d = ctx->d;
    const LevelView<double> V = fine_view(ctx);
    AdjArgs A = adj_args(ctx);
    // adjoint right-hand side (P g + A_m r) into b, then the same solve
    active_mean(V, ctx->active, ctx->adj_g, ctx->R, ctx->st, &ctx->launches);
    launch_adj_rhs(A, ctx->R.scal, ctx->b, ctx->st, &ctx->launches);
    ctx->warm_ok = false;
    cudaEventRecord(ctx->ev[1], ctx->st);
    if (ctx->opts.precision == SCF_PREC_FP64)
        rc = solve_impl<double>(ctx, ctx->L64, stats);
    else
        rc = solve_impl<float>(ctx, ctx->L32, stats);
    cudaEventRecord(ctx->ev[2], ctx->st);
    if (rc) return rc;
    // densities for the derivative: the given field or the phase densities
    if (!ctx->rho_given_last) fill_phase_density(ctx->phase, ctx->adj_rho, d.ng, ctx->opts.rho_l, ctx->opts.rho_g,
                                                 ctx->st, &ctx->launches);
    const double rho_ref = ctx->opts.rho_ref > 0.0 ? ctx->opts.rho_ref : ctx->opts.rho_l;
    CK(cudaMemsetAsync(ctx->adj_gu, 0, sizeof(double) * d.ng, ctx->st));
    CK(cudaMemsetAsync(ctx->adj_gv, 0, sizeof(double) * d.ng, ctx->st));
    CK(cudaMemsetAsync(ctx->adj_gw, 0, sizeof(double) * d.ng, ctx->st));
    CK(cudaMemsetAsync(ctx->adj_grho, 0, sizeof(double) * d.ng, ctx->st));
    launch_adj_grad(A, ctx->x, ctx->adj_rho, rho_ref, ctx->adj_gu, ctx->adj_gv, ctx->adj_gw, ctx->adj_grho, ctx->st,
                    &ctx->launches);
    int64_t bo = 0;
    if ((rc = d2h(ctx, grad_u, ctx->adj_gu, d.ng, &bo))) return rc;
    if ((rc = d2h(ctx, grad_v, ctx->adj_gv, d.ng, &bo))) return rc;
    if ((rc = d2h(ctx, grad_w, ctx->adj_gw, d.ng, &bo))) return rc;
    if ((rc = d2h(ctx, grad_rho, ctx->adj_grho, d.ng, &bo))) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]);
    stats->ms_solve = ms;
    stats->bytes_d2h = bo;
    stats->gpu_launches = ctx->launches;
    return SCF_OK;
}

int scf_debug_apply(scf_ctx *ctx, const double *xh, double *yh)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!xh || !yh) return SCF_ERR_BAD_ARG;
    if (!ctx->staged) { set_err(ctx, "no inputs staged"); return SCF_ERR_NO_SOLVE; }
    if (!ctx->assembled) { ctx->launches = 0; rc = assemble(ctx); if (rc) return rc; }
    const Dims &d = ctx->d;
    // p <- x (ghost layer forced to zero), q <- A p
    std::vector<double> xz(xh, xh + d.ng);
    for (int k = 0; k < d.gz; ++k)
        for (int j = 0; j < d.gy; ++j)
            for (int i = 0; i < d.gx; ++i)
                if (i == 0 || j == 0 || k == 0 || i == d.gx - 1 || j == d.gy - 1 || k == d.gz - 1)
                    xz[gidx(d, i, j, k)] = 0.0;
    CK(cudaMemcpyAsync(ctx->p, xz.data(), sizeof(double) * d.ng, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemsetAsync(ctx->q, 0, sizeof(double) * d.ng, ctx->st));
    cg_spmv_dot(fine_view(ctx), ctx->p, ctx->q, ctx->R, false, ctx->st, &ctx->launches);
    CK(cudaMemcpyAsync(yh, ctx->q, sizeof(double) * d.ng, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return SCF_OK;
}

int scf_debug_precondition(scf_ctx *ctx, const double *rh, double *zh)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!rh || !zh) return SCF_ERR_BAD_ARG;
    if (!ctx->solved) { set_err(ctx, "no projection has run"); return SCF_ERR_NO_SOLVE; }
    const Dims &d = ctx->d;
    const ChebCoef cc = cheb_for(ctx);
    CK(cudaMemcpyAsync(ctx->r, rh, sizeof(double) * d.ng, cudaMemcpyHostToDevice, ctx->st));
    if (ctx->opts.precision == SCF_PREC_FP64) {
        const double *z = precondition<double>(ctx, ctx->L64, cc, false);
        CK(cudaMemcpyAsync(zh, z, sizeof(double) * d.ng, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
    } else {
        copy_to_low(fine_view(ctx), ctx->r, ctx->L32[0].b, ctx->st, &ctx->launches);
        const float *z = precondition<float>(ctx, ctx->L32, cc, false);
        std::vector<float> zf(d.ng);
        CK(cudaMemcpyAsync(zf.data(), z, sizeof(float) * d.ng, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        for (int c = 0; c < d.ng; ++c) zh[c] = zf[c];
    }
    ctx->warm_ok = false;  // r was overwritten
    return SCF_OK;
}

int scf_debug_operator(scf_ctx *ctx, double *diag, double *cpl_e, double *cpl_n, double *cpl_t, double *rhs)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!ctx->staged) { set_err(ctx, "no inputs staged"); return SCF_ERR_NO_SOLVE; }
    if (!ctx->assembled) { ctx->launches = 0; rc = assemble(ctx); if (rc) return rc; }
    const Dims &d = ctx->d;
    std::vector<double> tmp(d.ng);
    double *outs[5] = {diag, cpl_e, cpl_n, cpl_t, rhs};
    double *srcs[5] = {ctx->diag, ctx->cE, ctx->cN, ctx->cT, ctx->b};
    for (int q = 0; q < 5; ++q) {
        if (!outs[q]) continue;
        CK(cudaMemcpyAsync(tmp.data(), srcs[q], sizeof(double) * d.ng, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        for (int k = 1; k <= d.K; ++k)
            for (int j = 1; j <= d.J; ++j)
                for (int i = 1; i <= d.I; ++i) outs[q][nidx(d, i, j, k)] = tmp[gidx(d, i, j, k)];
    }
    return SCF_OK;
}

int scf_debug_operator_f32(scf_ctx *ctx, float *diag_hi, float *e_hi, float *n_hi, float *t_hi, float *extra_hi,
                           float *diag_lo, float *e_lo, float *n_lo, float *t_lo, double *extra)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (ctx->opts.precision != SCF_PREC_MIXED) { set_err(ctx, "not a mixed-precision context"); return SCF_ERR_BAD_ARG; }
    if (!ctx->staged) { set_err(ctx, "no inputs staged"); return SCF_ERR_NO_SOLVE; }
    if (!ctx->assembled) { ctx->launches = 0; rc = assemble(ctx); if (rc) return rc; }
    const Dims &d = ctx->d;
    std::vector<float> tmp(d.ng);
    float *outs[9] = {diag_hi, e_hi, n_hi, t_hi, extra_hi, diag_lo, e_lo, n_lo, t_lo};
    const float *srcs[9] = {ctx->diag32, ctx->cE32, ctx->cN32, ctx->cT32, ctx->extra32,
                            ctx->diag_lo, ctx->cE_lo, ctx->cN_lo, ctx->cT_lo};
    for (int q = 0; q < 9; ++q) {
        if (!outs[q]) continue;
        CK(cudaMemcpyAsync(tmp.data(), srcs[q], sizeof(float) * d.ng, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        for (int k = 1; k <= d.K; ++k)
            for (int j = 1; j <= d.J; ++j)
                for (int i = 1; i <= d.I; ++i) outs[q][nidx(d, i, j, k)] = tmp[gidx(d, i, j, k)];
    }
    if (extra) {
        std::vector<double> t64(d.ng);
        CK(cudaMemcpyAsync(t64.data(), ctx->extra, sizeof(double) * d.ng, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        for (int k = 1; k <= d.K; ++k)
            for (int j = 1; j <= d.J; ++j)
                for (int i = 1; i <= d.I; ++i) extra[nidx(d, i, j, k)] = t64[gidx(d, i, j, k)];
    }
    return SCF_OK;
}

int scf_debug_time_kernel(scf_ctx *ctx, int kernel, int reps, double *ms_per_launch, double *bytes_per_launch)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!ms_per_launch || !bytes_per_launch || reps < 1) return SCF_ERR_BAD_ARG;
    if (!ctx->solved) { set_err(ctx, "no projection has run"); return SCF_ERR_NO_SOLVE; }
    if (ctx->nlev < 2 && (kernel == SCF_K_RESTRICT || kernel == SCF_K_PROLONG)) return SCF_ERR_BAD_ARG;
    const bool mixed = ctx->opts.precision == SCF_PREC_MIXED;
    const ChebCoef cc = cheb_for(ctx);
    auto launch = [&]() {
        switch (kernel) {
        case SCF_K_SMOOTH:
            if (mixed) probe_smooth<float>(ctx->L32[0], cc, ctx->st); else probe_smooth<double>(ctx->L64[0], cc, ctx->st);
            break;
        case SCF_K_SPMV:
            if (mixed) {
                int dummy = 0;
                df_spmv_dot(df_view(ctx), (const float2 *)ctx->p, (float2 *)ctx->q, ctx->R, false, ctx->st, &dummy);
            } else {
                probe_spmv(fine_view(ctx), ctx->p, ctx->q, ctx->R, ctx->st);
            }
            break;
        case SCF_K_RESTRICT:
            if (mixed) probe_restrict<float>(ctx->L32[0], ctx->L32[1], ctx->st);
            else probe_restrict<double>(ctx->L64[0], ctx->L64[1], ctx->st);
            break;
        case SCF_K_PROLONG:
            if (mixed) probe_prolong<float>(ctx->L32[0], ctx->L32[1], cc, ctx->st);
            else probe_prolong<double>(ctx->L64[0], ctx->L64[1], cc, ctx->st);
            break;
        case SCF_K_SMOOTH2: probe_smooth2(ctx->L32[0], cc, ctx->st); break;
        default: {
            int dummy = 0;
            if (mixed)
                df_cg_update(df_view(ctx), (float2 *)ctx->x, (float2 *)ctx->r, (const float2 *)ctx->p,
                             (const float2 *)ctx->q, ctx->L32[0].b, ctx->L32[0].x, cc.first, ctx->R, ctx->st, &dummy);
            else
                cg_update<double>(fine_view(ctx), ctx->x, ctx->r, ctx->p, ctx->q, nullptr, ctx->L64[0].view(),
                                  ctx->L64[0].x, cc.first, ctx->R, ctx->st, &dummy);
        }
        }
    };
    const double bytes = kernel_bytes(ctx, kernel);
    if (bytes < 0.0) return SCF_ERR_BAD_ARG;
    launch();  // warm
    CK(cudaEventRecord(ctx->ev[4], ctx->st));
    for (int r = 0; r < reps; ++r) launch();
    CK(cudaEventRecord(ctx->ev[5], ctx->st));
    CK(cudaEventSynchronize(ctx->ev[5]));
    CK(cudaGetLastError());
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev[4], ctx->ev[5]);
    *ms_per_launch = ms / reps;
    *bytes_per_launch = bytes;
    if (kernel == SCF_K_CGUPDATE) ctx->warm_ok = false;  // x was modified
    return SCF_OK;
}

int scf_kernel_timing(scf_ctx *ctx, int enable)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (enable && !ctx->kt_events) {
        for (int i = 0; i < 2 * KTimer::CAP; ++i)
            if (cudaEventCreate(&ctx->kt.ev[i]) != cudaSuccess) {
                while (i-- > 0) cudaEventDestroy(ctx->kt.ev[i]);
                set_err(ctx, "cudaEventCreate failed");
                return SCF_ERR_CUDA;
            }
        ctx->kt_events = true;
    }
    ctx->kt.on = enable != 0;
    ctx->kt.n = 0;
    for (int c = 0; c < KC_NUM; ++c) ctx->kt_ms[c] = ctx->kt_launches[c] = ctx->kt_bytes[c] = 0.0;
    return SCF_OK;
}

int scf_kernel_timing_read(scf_ctx *ctx, int kernel, double *ms_total, long long *launches, double *bytes_per_launch)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (kernel < 0 || kernel >= KC_NUM) return SCF_ERR_BAD_ARG;
    if (ms_total) *ms_total = ctx->kt_ms[kernel];
    if (launches) *launches = (long long)ctx->kt_launches[kernel];
    if (bytes_per_launch)
        *bytes_per_launch = ctx->kt_launches[kernel] > 0.0 ? ctx->kt_bytes[kernel] / ctx->kt_launches[kernel]
                                                            : kernel_bytes(ctx, kernel);
    return SCF_OK;
}

const char *scf_status_string(int s)
{
    switch (s) {
    case SCF_OK: return "ok";
    case SCF_ERR_BAD_ARG: return "bad argument";
    case SCF_ERR_NOT_CONVERGED: return "not converged";
    case SCF_ERR_NONFINITE: return "non-finite value";
    case SCF_ERR_CUDA: return "CUDA error";
    case SCF_ERR_OUT_OF_MEMORY: return "out of device memory";
    case SCF_ERR_BAD_INPUT: return "input outside the reference's model";
    case SCF_ERR_UNDEFINED_IN_REFERENCE: return "reference path has no defined result";
    case SCF_ERR_NO_DEVICE: return "no CUDA device";
    case SCF_ERR_NO_SOLVE: return "no solve/staged inputs";
    default: return "unknown status";
    }
}

int scf_last_error(const scf_ctx *ctx, char *buf, size_t len)
{
    if (!ctx || !buf || len == 0) return SCF_ERR_BAD_ARG;
    snprintf(buf, len, "%s", ctx->err);
    return SCF_OK;
}

int scf_host_register(void *ptr, size_t bytes)
{
    if (!ptr || !bytes) return SCF_ERR_BAD_ARG;
    return cudaHostRegister(ptr, bytes, cudaHostRegisterMapped | cudaHostRegisterPortable) == cudaSuccess
               ? SCF_OK
               : SCF_ERR_CUDA;
}

int scf_host_unregister(void *ptr)
{
    if (!ptr) return SCF_ERR_BAD_ARG;
    return cudaHostUnregister(ptr) == cudaSuccess ? SCF_OK : SCF_ERR_CUDA;
}

int scf_abi_version(void) { return SCF_ABI_VERSION; }

int scf_debug_fail_device_alloc(int64_t nth)
{
    if (nth < 0) return SCF_ERR_BAD_ARG;
    scf_mem::fail_countdown.store(nth);
    return SCF_OK;
}

int64_t scf_debug_device_buffers(void) { return scf_mem::live.load(); }

int scf_debug_smoother_pairs(int on, int planes)
{
    if (planes < 0 || on < 0 || on > 2) return SCF_ERR_BAD_ARG;
    set_smoother_pairs(on, planes);
    return SCF_OK;
}

int scf_debug_smoother_pair_counts(int64_t *tma_launches, int64_t *fallbacks)
{
    long long t = 0, f = 0;
    smoother_pair_counts(&t, &f);
    if (tma_launches) *tma_launches = t;
    if (fallbacks) *fallbacks = f;
    return SCF_OK;
}

}  // extern "C"

namespace scf_mem {
std::atomic<long long> fail_countdown{0};
std::atomic<long long> live{0};
}  // namespace scf_mem

extern "C" int scf_ctx_device_fields(scf_ctx *ctx, const double **u, const double **v, const double **w,
                                     const double **p, const double **phil, const double **vofl, const double **vof)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (u) *u = ctx->tu;
    if (v) *v = ctx->tv;
    if (w) *w = ctx->tw;
    if (p) *p = ctx->tp;
    if (phil) *phil = ctx->phil;
    if (vofl) *vofl = ctx->vofl;
    if (vof) *vof = ctx->vof;
    return SCF_OK;
}
