// pred_api.cu -- C ABI of the momentum predictor's implicit solves
// (include/scf_predictor.h): device copies of the three components' inputs,
// the per-component assembly and BiCGStab solve, the tail of PredictingUVW,
// and the copies out.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <future>
#include <thread>
#include <vector>

#include "../../include/scf_predictor.h"
#include "pred_kernels.h"
#include "scf_devmem.h"
#include "scf_stage.h"

using namespace pred;

struct scf_mom_ctx {
    Dims d{};
    int device = 0;
    cudaStream_t st = nullptr;
    cudaStream_t cin = nullptr, cout = nullptr;   // copies in / out of the pipelined call
    cudaEvent_t staged_ev[3] = {}, done_ev[3] = {};
    cudaEvent_t ev[4] = {};
    cudaEvent_t kev[7] = {};   // around the BiCGStab passes (kernel_timing)
    std::vector<void *> mem;
    struct Comp {
        double *dx, *dy, *dz, *vof, *vofl, *eta_e, *eta_n, *eta_t, *vof_old, *tvar;
        double *df_ew, *df_ns, *df_tb, *edf_ew, *edf_ns, *edf_tb, *fric, *flux_div;
        int32_t *cell_type, *posnu;
        double *bc[6];
        int flag[6];
        int extcell;
    } comp[3];
    double *m[6] = {};
    float *m32[6] = {};
    double *b = nullptr;
    double *pred[3] = {}, *dp[3] = {};
    BcgVecs<double> V64{};
    BcgVecs<float> V32{};
    Reduce R{};
    BcgScalars *sc = nullptr, *sc_host = nullptr;
    unsigned long long *counts = nullptr, *counts_host = nullptr;
    bool staged = false, ran = false;
    char err[512] = {0};
};

namespace {

void mom_err(scf_mom_ctx *c, const char *fmt, ...)
{
    if (!c) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof(c->err), fmt, ap);
    va_end(ap);
}

#define MK(call)                                                                            \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            mom_err(ctx, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return e_ == cudaErrorMemoryAllocation ? SCF_ERR_OUT_OF_MEMORY : SCF_ERR_CUDA;   \
        }                                                                                   \
    } while (0)

template <typename P>
int malloc0(scf_mom_ctx *ctx, P **ptr, size_t count)
{
    void *p = nullptr;
    const size_t bytes = std::max<size_t>(count * sizeof(P), 16);
    cudaError_t e = scf_mem::dev_malloc(&p, bytes);
    if (e != cudaSuccess) {
        mom_err(ctx, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
        return SCF_ERR_OUT_OF_MEMORY;
    }
    ctx->mem.push_back(p);
    if (cudaMemset(p, 0, bytes) != cudaSuccess) return SCF_ERR_CUDA;
    *ptr = (P *)p;
    return SCF_OK;
}

struct Copy {
    void *dev;
    const void *host;
    size_t bytes;
};

// The arrays of one component in the order of scf_mom_in, with sizes.
std::vector<Copy> comp_copies(scf_mom_ctx *ctx, int c, const scf_mom_in &in)
{
    const Dims &d = ctx->d;
    const size_t n = (size_t)d.I * d.J * d.K, ng = (size_t)d.ng, D = sizeof(double), I4 = sizeof(int32_t);
    const size_t few = (size_t)(d.I + 2) * d.J * d.K, fns = (size_t)d.I * (d.J + 2) * d.K,
                 ftb = (size_t)d.I * d.J * (d.K + 2);
    const size_t npn = (size_t)(d.I - (c == 0)) * (d.J - (c == 1)) * (d.K - (c == 2));
    scf_mom_ctx::Comp &t = ctx->comp[c];
    const size_t bcn[6] = {(size_t)d.J * d.K, (size_t)d.J * d.K, (size_t)d.I * d.K,
                           (size_t)d.I * d.K, (size_t)d.I * d.J, (size_t)d.I * d.J};
    std::vector<Copy> v = {
        {t.dx, in.grid_dx, n * D},     {t.dy, in.grid_dy, n * D},       {t.dz, in.grid_dz, n * D},
        {t.vof, in.vof, ng * D},       {t.vofl, in.vofl, ng * D},       {t.eta_e, in.eta_e, ng * D},
        {t.eta_n, in.eta_n, ng * D},   {t.eta_t, in.eta_t, ng * D},     {t.cell_type, in.cell_type, n * I4},
        {t.posnu, in.posnu, npn * I4}, {t.vof_old, in.vof_old, ng * D}, {t.df_ew, in.df_ew, few * D},
        {t.df_ns, in.df_ns, fns * D},  {t.df_tb, in.df_tb, ftb * D},    {t.edf_ew, in.edf_ew, few * D},
        {t.edf_ns, in.edf_ns, fns * D}, {t.edf_tb, in.edf_tb, ftb * D}, {t.fric, in.fric, n * D},
        {t.flux_div, in.flux_div, n * D}, {t.tvar, in.tvar, ng * D}};
    for (int f = 0; f < 6; ++f) v.push_back({t.bc[f], in.bc_var[f], bcn[f] * D});
    return v;
}

MomDev dev_view(const scf_mom_ctx::Comp &t)
{
    MomDev m;
    m.dx = t.dx; m.dy = t.dy; m.dz = t.dz;
    m.vof = t.vof; m.vofl = t.vofl; m.eta_e = t.eta_e; m.eta_n = t.eta_n; m.eta_t = t.eta_t;
    m.vof_old = t.vof_old; m.tvar = t.tvar;
    m.df_ew = t.df_ew; m.df_ns = t.df_ns; m.df_tb = t.df_tb;
    m.edf_ew = t.edf_ew; m.edf_ns = t.edf_ns; m.edf_tb = t.edf_tb;
    m.fric = t.fric; m.flux_div = t.flux_div;
    m.cell_type = t.cell_type; m.posnu = t.posnu;
    for (int f = 0; f < 6; ++f) { m.bc[f] = t.bc[f]; m.flag[f] = t.flag[f]; }
    return m;
}

int read_scalars(scf_mom_ctx *ctx)
{
    MK(cudaMemcpyAsync(ctx->sc_host, ctx->sc, sizeof(BcgScalars), cudaMemcpyDeviceToHost, ctx->st));
    MK(cudaStreamSynchronize(ctx->st));
    return SCF_OK;
}

#define RS()                                   \
    do {                                       \
        const int rc_ = read_scalars(ctx);     \
        if (rc_ != SCF_OK) return rc_;         \
    } while (0)

struct SolveOut {
    int iterations = 0, rounds = 0, converged = 0;
    double rel = 0.0;
    const double *x = nullptr;
    int launches = 0;
    int timed = 0;
    double ms_k[4] = {0.0, 0.0, 0.0, 0.0};
};

float elapsed(cudaEvent_t a, cudaEvent_t b);
int check_inputs(scf_mom_ctx *ctx, const scf_mom_in in[3]);

// After a synchronised iteration: the three stencil kernels' times.
void add_kernel_times(scf_mom_ctx *ctx, SolveOut &out)
{
    out.ms_k[0] += elapsed(ctx->kev[0], ctx->kev[1]);
    out.ms_k[1] += elapsed(ctx->kev[1], ctx->kev[2]);
    out.ms_k[2] += elapsed(ctx->kev[3], ctx->kev[4]);
    out.ms_k[3] += elapsed(ctx->kev[5], ctx->kev[6]);
    ++out.timed;
}

// Iterations enqueued between two reads of the device scalars (the passes
// after convergence return at once, so a batch costs at most a few empty
// launches); 1 with kernel timing, whose events are read per iteration.
constexpr int BATCH = 4;

// Runs BiCGStab iterations on V until the device-side test stops them (done)
// or `cap` iterations ran; returns the iterations run.  `first`: the first
// one starts with p = r.
template <typename T>
int run_batches(scf_mom_ctx *ctx, const scf_mom_opts &o, const T *const m[6], BcgVecs<T> &V, bool first, int cap,
                SolveOut &out, int &rc)
{
    const Dims &d = ctx->d;
    const int batch = o.kernel_timing ? 1 : BATCH;
    int done_its = 0;
    rc = SCF_OK;
    while (done_its < cap) {
        const int nb = std::min(batch, cap - done_its);
        for (int q = 0; q < nb; ++q)
            bcg_iteration<T>(d, m, V, first && q == 0, ctx->R, ctx->sc, ctx->st,
                             o.kernel_timing ? ctx->kev : nullptr);
        first = false;
        out.launches += 7 * nb;
        if ((rc = read_scalars(ctx)) != SCF_OK) return done_its;
        done_its = ctx->sc_host->iters;
        if (o.kernel_timing) add_kernel_times(ctx, out);
        if (!std::isfinite(ctx->sc_host->rr)) {
            mom_err(ctx, "non-finite residual after %d iterations", out.iterations + done_its);
            rc = SCF_ERR_NONFINITE;
            return done_its;
        }
        if (ctx->sc_host->done) break;
    }
    return done_its;
}

// FP64 BiCGStab on the scaled system, restarted from the true residual
// when the recursive one says converged but the true one does not, or on a
// breakdown.
int solve_fp64(scf_mom_ctx *ctx, const scf_mom_opts &o, SolveOut &out)
{
    const Dims &d = ctx->d;
    BcgVecs<double> &V = ctx->V64;
    const double *const *m = ctx->m;
    const size_t bytes = (size_t)d.ng * sizeof(double);
    MK(cudaMemsetAsync(V.x, 0, bytes, ctx->st));
    resid64(d, m, ctx->b, nullptr, V.r, nullptr, true, ctx->R, ctx->sc, ctx->st);
    MK(cudaMemcpyAsync(V.r0, V.r, bytes, cudaMemcpyDeviceToDevice, ctx->st));
    out.launches += 2;
    RS();
    const double bb = ctx->sc_host->bb, target = o.rel_tol * o.rel_tol * bb;
    out.x = V.x;
    out.rounds = 1;
    double rr = ctx->sc_host->rr;
    if (bb == 0.0 || rr <= target) {
        out.converged = 1;
        out.rel = bb == 0.0 ? 0.0 : std::sqrt(rr / bb);
        return SCF_OK;
    }
    while (out.iterations < o.max_iter) {
        set_target(ctx->sc, target, ctx->st);
        int rc = SCF_OK;
        const int its = run_batches<double>(ctx, o, m, V, true, o.max_iter - out.iterations, out, rc);
        out.iterations += its;
        if (rc != SCF_OK) return rc;
        if (!ctx->sc_host->done) break;   // iteration cap
        // converged by the recursive residual, or broken down: check the
        // true residual and restart from it if needed
        resid64(d, m, ctx->b, V.x, V.r, nullptr, false, ctx->R, ctx->sc, ctx->st);
        out.launches += 2;
        RS();
        rr = ctx->sc_host->rr;
        if (!std::isfinite(rr)) {
            mom_err(ctx, "non-finite residual after %d iterations", out.iterations);
            return SCF_ERR_NONFINITE;
        }
        if (rr <= target) { out.converged = 1; break; }
        // a breakdown in the first iteration of a round leaves the residual
        // as it was, and a restart from it would break down again
        if (its == 0) break;
        MK(cudaMemcpyAsync(V.r0, V.r, bytes, cudaMemcpyDeviceToDevice, ctx->st));
        ++out.rounds;
    }
    out.rel = std::sqrt(rr / bb);
    return SCF_OK;
}

// FP32 BiCGStab inside FP64 iterative refinement: each round solves
// A e = r (r the FP64 residual rounded to FP32) to a relative 1e-6, then
// x += e and the residual is recomputed in FP64 from the FP64 rows.  The
// host reads the scalars only to stop.
int solve_mixed(scf_mom_ctx *ctx, const scf_mom_opts &o, SolveOut &out)
{
    const Dims &d = ctx->d;
    BcgVecs<float> &V = ctx->V32;
    const double *const *m = ctx->m;
    const float *const *m32 = ctx->m32;
    double *xa = ctx->V64.x;
    const size_t bytes32 = (size_t)d.ng * sizeof(float);
    MK(cudaMemsetAsync(xa, 0, (size_t)d.ng * sizeof(double), ctx->st));
    resid64(d, m, ctx->b, nullptr, nullptr, V.r, true, ctx->R, ctx->sc, ctx->st);
    out.launches += 2;
    RS();
    const double bb = ctx->sc_host->bb, target = o.rel_tol * o.rel_tol * bb;
    double rr = ctx->sc_host->rr;
    out.x = xa;
    if (bb == 0.0 || rr <= target) {
        out.converged = 1;
        out.rel = bb == 0.0 ? 0.0 : std::sqrt(rr / bb);
        return SCF_OK;
    }
    while (out.iterations < o.max_iter) {
        const double rho0 = ctx->sc_host->rho;
        const double inner = std::max(1e-12 * rho0, 0.25 * target);
        MK(cudaMemcpyAsync(V.r0, V.r, bytes32, cudaMemcpyDeviceToDevice, ctx->st));
        MK(cudaMemsetAsync(V.x, 0, bytes32, ctx->st));
        set_target(ctx->sc, inner, ctx->st);
        int rc = SCF_OK;
        const int its = run_batches<float>(ctx, o, m32, V, true, o.max_iter - out.iterations, out, rc);
        out.iterations += its;
        if (rc != SCF_OK) return rc;
        if (its == 0) break;   // breakdown at the round's first iteration: x unchanged, no progress possible
        xadd(d, xa, V.x, ctx->st);
        resid64(d, m, ctx->b, xa, nullptr, V.r, false, ctx->R, ctx->sc, ctx->st);
        out.launches += 3;
        ++out.rounds;
        RS();
        rr = ctx->sc_host->rr;
        if (!std::isfinite(rr)) {
            mom_err(ctx, "non-finite residual after %d iterations", out.iterations);
            return SCF_ERR_NONFINITE;
        }
        if (rr <= target) { out.converged = 1; break; }
    }
    out.x = xa;
    out.rel = std::sqrt(rr / bb);
    return SCF_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

}  // namespace

extern "C" int scf_mom_create(scf_mom_ctx **out, int32_t imax, int32_t jmax, int32_t kmax, int32_t device)
{
    if (!out) return SCF_ERR_BAD_ARG;
    *out = nullptr;
    if (imax < 2 || jmax < 2 || kmax < 2 || jmax > 65533 || kmax > 65533) return SCF_ERR_BAD_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return SCF_ERR_NO_DEVICE;
    scf_mom_ctx *ctx = new scf_mom_ctx();
    ctx->device = device;
    Dims &d = ctx->d;
    d.I = imax; d.J = jmax; d.K = kmax;
    d.sy = imax + 2;
    d.sz = (long long)(imax + 2) * (jmax + 2);
    d.ng = d.sz * (kmax + 2);
    auto fail = [&](int rc) {
        scf_mom_destroy(ctx);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->cin, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->cout, cudaStreamNonBlocking) != cudaSuccess)
        return fail(SCF_ERR_CUDA);
    for (int c = 0; c < 3; ++c)
        if (cudaEventCreateWithFlags(&ctx->staged_ev[c], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->done_ev[c], cudaEventDisableTiming) != cudaSuccess)
            return fail(SCF_ERR_CUDA);
    for (auto &e : ctx->ev)
        if (cudaEventCreate(&e) != cudaSuccess) return fail(SCF_ERR_CUDA);
    for (auto &e : ctx->kev)
        if (cudaEventCreate(&e) != cudaSuccess) return fail(SCF_ERR_CUDA);
    const size_t n = (size_t)imax * jmax * kmax, ng = (size_t)d.ng;
    const size_t few = (size_t)(imax + 2) * jmax * kmax, fns = (size_t)imax * (jmax + 2) * kmax,
                 ftb = (size_t)imax * jmax * (kmax + 2);
    const size_t bcn[6] = {(size_t)jmax * kmax, (size_t)jmax * kmax, (size_t)imax * kmax,
                           (size_t)imax * kmax, (size_t)imax * jmax, (size_t)imax * jmax};
    int rc = SCF_OK;
#define TRY(ptr, count)                                              \
    if ((rc = malloc0(ctx, &(ptr), (count))) != SCF_OK) return fail(rc);
    for (int c = 0; c < 3; ++c) {
        scf_mom_ctx::Comp &t = ctx->comp[c];
        TRY(t.dx, n) TRY(t.dy, n) TRY(t.dz, n)
        TRY(t.vof, ng) TRY(t.vofl, ng) TRY(t.eta_e, ng) TRY(t.eta_n, ng) TRY(t.eta_t, ng)
        TRY(t.vof_old, ng) TRY(t.tvar, ng)
        TRY(t.df_ew, few) TRY(t.df_ns, fns) TRY(t.df_tb, ftb)
        TRY(t.edf_ew, few) TRY(t.edf_ns, fns) TRY(t.edf_tb, ftb)
        TRY(t.fric, n) TRY(t.flux_div, n)
        TRY(t.cell_type, n)
        TRY(t.posnu, (size_t)(imax - (c == 0)) * (jmax - (c == 1)) * (kmax - (c == 2)))
        for (int f = 0; f < 6; ++f) TRY(t.bc[f], bcn[f])
        TRY(ctx->pred[c], ng) TRY(ctx->dp[c], ng)
    }
    for (int q = 0; q < 6; ++q) { TRY(ctx->m[q], ng) TRY(ctx->m32[q], ng) }
    TRY(ctx->b, ng)
    TRY(ctx->V64.x, ng) TRY(ctx->V64.r, ng) TRY(ctx->V64.r0, ng) TRY(ctx->V64.t, ng)
    TRY(ctx->V64.p, ng) TRY(ctx->V64.v, ng)
    TRY(ctx->V32.x, ng) TRY(ctx->V32.r, ng) TRY(ctx->V32.r0, ng) TRY(ctx->V32.t, ng)
    TRY(ctx->V32.p, ng) TRY(ctx->V32.v, ng)
    ctx->R.nblocks = (int)(solver_grid(d).x * solver_grid(d).y * solver_grid(d).z);
    TRY(ctx->R.partials, 4 * (size_t)ctx->R.nblocks)
    TRY(ctx->sc, 1)
    TRY(ctx->counts, 2)
#undef TRY
    if (cudaMallocHost(&ctx->sc_host, sizeof(BcgScalars)) != cudaSuccess) return fail(SCF_ERR_OUT_OF_MEMORY);
    if (cudaMallocHost(&ctx->counts_host, 2 * sizeof(unsigned long long)) != cudaSuccess)
        return fail(SCF_ERR_OUT_OF_MEMORY);
    *out = ctx;
    return SCF_OK;
}

extern "C" int scf_mom_destroy(scf_mom_ctx *ctx)
{
    if (!ctx) return SCF_OK;
    cudaSetDevice(ctx->device);
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    for (void *p : ctx->mem) scf_mem::dev_free(p);
    if (ctx->sc_host) cudaFreeHost(ctx->sc_host);
    if (ctx->counts_host) cudaFreeHost(ctx->counts_host);
    for (auto e : ctx->ev)
        if (e) cudaEventDestroy(e);
    for (auto e : ctx->kev)
        if (e) cudaEventDestroy(e);
    for (int c = 0; c < 3; ++c) {
        if (ctx->staged_ev[c]) cudaEventDestroy(ctx->staged_ev[c]);
        if (ctx->done_ev[c]) cudaEventDestroy(ctx->done_ev[c]);
    }
    if (ctx->cin) cudaStreamSynchronize(ctx->cin);
    if (ctx->cout) cudaStreamSynchronize(ctx->cout);
    if (ctx->cin) cudaStreamDestroy(ctx->cin);
    if (ctx->cout) cudaStreamDestroy(ctx->cout);
    if (ctx->st) cudaStreamDestroy(ctx->st);
    delete ctx;
    return SCF_OK;
}

extern "C" int scf_mom_stage(scf_mom_ctx *ctx, const scf_mom_in in[3])
{
    if (!ctx || !in) return SCF_ERR_BAD_ARG;
    ctx->err[0] = 0;
    const int rc = check_inputs(ctx, in);
    if (rc != SCF_OK) return rc;
    MK(cudaSetDevice(ctx->device));
    for (int c = 0; c < 3; ++c) {
        for (const Copy &cp : comp_copies(ctx, c, in[c]))
            MK(stage_h2d(cp.dev, cp.host, cp.bytes, ctx->st, 0, nullptr, nullptr));
        for (int f = 0; f < 6; ++f) ctx->comp[c].flag[f] = in[c].bc_flag[f];
        ctx->comp[c].extcell = in[c].extcell;
    }
    MK(cudaStreamSynchronize(ctx->st));
    ctx->staged = true;
    return SCF_OK;
}

namespace {

int check_opts(scf_mom_ctx *ctx, const scf_mom_opts &o)
{
    if (!(o.dt > 0.0) || !(o.rel_tol > 0.0) || o.max_iter < 1 || !(o.g != 0.0) || !(o.fr != 0.0) ||
        (o.precision != SCF_PREC_FP64 && o.precision != SCF_PREC_MIXED)) {
        mom_err(ctx, "bad options");
        return SCF_ERR_BAD_ARG;
    }
    return SCF_OK;
}

int check_inputs(scf_mom_ctx *ctx, const scf_mom_in in[3])
{
    for (int c = 0; c < 3; ++c) {
        for (const Copy &cp : comp_copies(ctx, c, in[c]))
            if (!cp.host) {
                mom_err(ctx, "component %d: a required input array is NULL", c);
                return SCF_ERR_BAD_ARG;
            }
        if (in[c].extcell < -1) {
            mom_err(ctx, "component %d: ExtCell %d", c, in[c].extcell);
            return SCF_ERR_BAD_ARG;
        }
    }
    return SCF_OK;
}

// The numbering DeltaGetValues relies on: PosNu = -1 exactly on solid
// cells, ExtCell + 1 numbered cells.
int check_numbering(scf_mom_ctx *ctx, int c, scf_mom_stats &s)
{
    MK(cudaMemsetAsync(ctx->counts, 0, 2 * sizeof(unsigned long long), ctx->st));
    mom_check_numbering(dev_view(ctx->comp[c]), c + 1, ctx->d, ctx->counts, ctx->st);
    MK(cudaMemcpyAsync(ctx->counts_host, ctx->counts, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                       ctx->st));
    MK(cudaStreamSynchronize(ctx->st));
    s.gpu_launches += 1;
    if (ctx->counts_host[1] != 0 || (long long)ctx->counts_host[0] != (long long)ctx->comp[c].extcell + 1) {
        mom_err(ctx, "component %d: %llu active cells for ExtCell %d, %llu PosNu/Cell_Type mismatches", c,
                ctx->counts_host[0], ctx->comp[c].extcell, ctx->counts_host[1]);
        return SCF_ERR_BAD_INPUT;
    }
    return SCF_OK;
}

// Assembly, solve, scatter and tail of component c on ctx->st.
int run_component(scf_mom_ctx *ctx, int c, const scf_mom_opts &o, scf_mom_stats &s)
{
    const Dims &d = ctx->d;
    MomParams P;
    P.dt = o.dt; P.rho_a = o.rho_a_ref; P.rho_w = o.rho_w_ref; P.fr = o.fr;
    P.gx = o.gx; P.gy = o.gy; P.gz = o.gz; P.g = o.g; P.beta_vis = o.beta_vis;
    P.rfr2 = 1.0 / (o.fr * o.fr);
    for (int f = 0; f < 6; ++f) P.flags[f] = ctx->comp[c].flag[f];
    const bool mixed = o.precision == SCF_PREC_MIXED;
    MomSys S;
    for (int q = 0; q < 6; ++q) { S.m[q] = ctx->m[q]; S.m32[q] = ctx->m32[q]; }
    S.b = ctx->b;
    S.dp = ctx->dp[c];
    const MomDev view = dev_view(ctx->comp[c]);
    MK(cudaEventRecord(ctx->ev[0], ctx->st));
    mom_assemble(view, P, c + 1, d, S, mixed, ctx->st);
    MK(cudaGetLastError());
    MK(cudaEventRecord(ctx->ev[1], ctx->st));
    s.gpu_launches += 1;
    SolveOut so;
    const int rc = mixed ? solve_mixed(ctx, o, so) : solve_fp64(ctx, o, so);
    if (rc != SCF_OK) return rc;
    MK(cudaGetLastError());
    MK(cudaMemcpyAsync(ctx->pred[c], so.x, (size_t)d.ng * sizeof(double), cudaMemcpyDeviceToDevice, ctx->st));
    MK(cudaEventRecord(ctx->ev[2], ctx->st));
    int tl = 0;
    mom_tail_comp(view, d, c, ctx->pred[c], ctx->dp[c], ctx->st, &tl);
    MK(cudaGetLastError());
    MK(cudaEventRecord(ctx->ev[3], ctx->st));
    MK(cudaEventSynchronize(ctx->ev[3]));
    s.ms_assemble += elapsed(ctx->ev[0], ctx->ev[1]);
    s.ms_solve += elapsed(ctx->ev[1], ctx->ev[2]);
    s.ms_tail += elapsed(ctx->ev[2], ctx->ev[3]);
    s.iterations[c] = so.iterations;
    s.rounds[c] = so.rounds;
    s.converged[c] = so.converged;
    s.rel_residual[c] = so.rel;
    s.gpu_launches += so.launches + tl;
    s.timed_iterations += so.timed;
    for (int q = 0; q < 4; ++q) s.ms_kernels[q] += so.ms_k[q];
    return SCF_OK;
}

int converged_or_report(scf_mom_ctx *ctx, const scf_mom_stats &s)
{
    for (int c = 0; c < 3; ++c)
        if (!s.converged[c]) {
            mom_err(ctx, "component %d: relative residual %.3e after %d iterations", c, s.rel_residual[c],
                    s.iterations[c]);
            return SCF_ERR_NOT_CONVERGED;
        }
    return SCF_OK;
}

// Copies of component c's results to the host on stream st: Dp whole, Pred
// on the box the reference writes (the loop range and the BC planes of the
// component's own axis).
cudaError_t fetch_component(scf_mom_ctx *ctx, int c, double *pred, double *dp, cudaStream_t st)
{
    const Dims &d = ctx->d;
    if (dp) {
        const cudaError_t e = cudaMemcpyAsync(dp, ctx->dp[c], (size_t)d.ng * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return e;
    }
    if (!pred) return cudaSuccess;
    const int x0 = c == 0 ? 0 : 1, y0 = c == 1 ? 0 : 1, z0 = c == 2 ? 0 : 1;
    const int nx = c == 0 ? d.I + 2 : d.I, ny = c == 1 ? d.J + 2 : d.J, nz = c == 2 ? d.K + 2 : d.K;
    cudaMemcpy3DParms p;
    std::memset(&p, 0, sizeof p);
    p.srcPtr = make_cudaPitchedPtr(ctx->pred[c], (size_t)(d.I + 2) * sizeof(double), d.I + 2, d.J + 2);
    p.dstPtr = make_cudaPitchedPtr(pred, (size_t)(d.I + 2) * sizeof(double), d.I + 2, d.J + 2);
    p.srcPos = make_cudaPos((size_t)x0 * sizeof(double), y0, z0);
    p.dstPos = p.srcPos;
    p.extent = make_cudaExtent((size_t)nx * sizeof(double), ny, nz);
    p.kind = cudaMemcpyDeviceToHost;
    return cudaMemcpy3DAsync(&p, st);
}

double ms_between(std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

extern "C" int scf_mom_run(scf_mom_ctx *ctx, const scf_mom_opts *opts, scf_mom_stats *stats)
{
    if (!ctx || !opts) return SCF_ERR_BAD_ARG;
    ctx->err[0] = 0;
    if (!ctx->staged) {
        mom_err(ctx, "scf_mom_run before scf_mom_stage");
        return SCF_ERR_NO_SOLVE;
    }
    int rc = check_opts(ctx, *opts);
    if (rc != SCF_OK) return rc;
    MK(cudaSetDevice(ctx->device));
    scf_mom_stats s;
    std::memset(&s, 0, sizeof s);
    for (int c = 0; c < 3; ++c)
        if ((rc = check_numbering(ctx, c, s)) != SCF_OK) return rc;
    for (int c = 0; c < 3; ++c)
        if ((rc = run_component(ctx, c, *opts, s)) != SCF_OK) return rc;
    s.ms_total = s.ms_assemble + s.ms_solve + s.ms_tail;
    ctx->ran = true;
    if (stats) *stats = s;
    return converged_or_report(ctx, s);
}

extern "C" int scf_mom_fetch(scf_mom_ctx *ctx, double *pred_u, double *pred_v, double *pred_w, double *pu_dp,
                             double *pv_dp, double *pw_dp)
{
    if (!ctx) return SCF_ERR_BAD_ARG;
    if (!ctx->ran) {
        mom_err(ctx, "scf_mom_fetch before scf_mom_run");
        return SCF_ERR_NO_SOLVE;
    }
    MK(cudaSetDevice(ctx->device));
    double *preds[3] = {pred_u, pred_v, pred_w}, *dps[3] = {pu_dp, pv_dp, pw_dp};
    for (int c = 0; c < 3; ++c) MK(fetch_component(ctx, c, preds[c], dps[c], ctx->st));
    MK(cudaStreamSynchronize(ctx->st));
    return SCF_OK;
}

// The drop-in call, pipelined over the three components: a helper thread
// copies component c+1's inputs in (stream cin) while component c is
// assembled and solved, and a second one copies component c's results out
// (stream cout) while the next component runs.  Each component's tail
// touches only its own arrays, so it runs right after its solve; the
// results equal those of stage + run + fetch.
extern "C" int scf_predict_solves(scf_mom_ctx *ctx, const scf_mom_in in[3], const scf_mom_opts *opts,
                                  double *pred_u, double *pred_v, double *pred_w, double *pu_dp, double *pv_dp,
                                  double *pw_dp, scf_mom_stats *stats)
{
    if (!ctx || !in || !opts) return SCF_ERR_BAD_ARG;
    ctx->err[0] = 0;
    int rc = check_inputs(ctx, in);
    if (rc == SCF_OK) rc = check_opts(ctx, *opts);
    if (rc != SCF_OK) return rc;
    MK(cudaSetDevice(ctx->device));
    const auto t0 = std::chrono::steady_clock::now();
    double *preds[3] = {pred_u, pred_v, pred_w}, *dps[3] = {pu_dp, pv_dp, pw_dp};
    std::promise<cudaError_t> staged[3];
    std::promise<bool> done[3];
    std::future<cudaError_t> staged_f[3];
    std::future<bool> done_f[3];
    for (int c = 0; c < 3; ++c) {
        staged_f[c] = staged[c].get_future();
        done_f[c] = done[c].get_future();
    }
    std::chrono::steady_clock::time_point t_in_end = t0, t_out_end = t0;
    cudaError_t out_err = cudaSuccess;
    auto stage_all = [&] {
        cudaError_t e = cudaSetDevice(ctx->device);
        for (int c = 0; c < 3; ++c) {
            if (e == cudaSuccess)
                for (const Copy &cp : comp_copies(ctx, c, in[c])) {
                    // the first component's inputs are on the critical path
                    // (copy kernel, scf_stage.h); the others overlap the
                    // earlier components' solves and take the copy engine,
                    // which leaves the SMs to the solves
                    e = c == 0 ? stage_h2d(cp.dev, cp.host, cp.bytes, ctx->cin, 0, nullptr, nullptr)
                               : cudaMemcpyAsync(cp.dev, cp.host, cp.bytes, cudaMemcpyHostToDevice, ctx->cin);
                    if (e != cudaSuccess) break;
                }
            if (e == cudaSuccess) e = cudaEventRecord(ctx->staged_ev[c], ctx->cin);
            staged[c].set_value(e);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->cin);
        t_in_end = std::chrono::steady_clock::now();
    };
    auto fetch_all = [&] {
        cudaError_t e = cudaSetDevice(ctx->device);
        for (int c = 0; c < 3; ++c) {
            if (!done_f[c].get() || e != cudaSuccess) continue;
            e = cudaStreamWaitEvent(ctx->cout, ctx->done_ev[c], 0);
            if (e == cudaSuccess) e = fetch_component(ctx, c, preds[c], dps[c], ctx->cout);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->cout);
        out_err = e;
        t_out_end = std::chrono::steady_clock::now();
    };
    // the helper threads; an exception must not leave this C entry point
    std::thread stager, fetcher;
    try {
        stager = std::thread(stage_all);
        fetcher = std::thread(fetch_all);
    } catch (...) {
        if (stager.joinable()) stager.join();   // finishes on its own
        ctx->staged = ctx->ran = false;
        mom_err(ctx, "could not start the copy threads");
        return SCF_ERR_CUDA;
    }
    scf_mom_stats s;
    std::memset(&s, 0, sizeof s);
    int next = 0;   // components whose results were handed to the fetcher
    for (int c = 0; c < 3 && rc == SCF_OK; ++c) {
        const cudaError_t e = staged_f[c].get();
        if (e != cudaSuccess) {
            mom_err(ctx, "copy of component %d's inputs: %s", c, cudaGetErrorString(e));
            rc = SCF_ERR_CUDA;
            break;
        }
        if (cudaStreamWaitEvent(ctx->st, ctx->staged_ev[c], 0) != cudaSuccess) { rc = SCF_ERR_CUDA; break; }
        for (int f = 0; f < 6; ++f) ctx->comp[c].flag[f] = in[c].bc_flag[f];
        ctx->comp[c].extcell = in[c].extcell;
        if ((rc = check_numbering(ctx, c, s)) != SCF_OK) break;
        if ((rc = run_component(ctx, c, *opts, s)) != SCF_OK) break;
        if (cudaEventRecord(ctx->done_ev[c], ctx->st) != cudaSuccess) { rc = SCF_ERR_CUDA; break; }
        done[c].set_value(true);
        next = c + 1;
    }
    const auto t_dev_end = std::chrono::steady_clock::now();
    for (int c = next; c < 3; ++c) done[c].set_value(false);
    for (int c = 0; c < 3; ++c)   // a failed component: let the stager finish
        if (c >= next && staged_f[c].valid()) staged_f[c].wait();
    stager.join();
    fetcher.join();
    const auto t1 = std::chrono::steady_clock::now();
    ctx->staged = rc == SCF_OK;
    ctx->ran = rc == SCF_OK;
    if (rc == SCF_OK && out_err != cudaSuccess) {
        mom_err(ctx, "copy of the results: %s", cudaGetErrorString(out_err));
        rc = SCF_ERR_CUDA;
    }
    const Dims &d = ctx->d;
    long long h2d = 0, d2h = 0;
    for (int c = 0; c < 3; ++c) {
        for (const Copy &cp : comp_copies(ctx, c, in[c])) h2d += (long long)cp.bytes;
        if (dps[c]) d2h += (long long)d.ng * 8;
        if (preds[c])
            d2h += 8LL * (c == 0 ? d.I + 2 : d.I) * (c == 1 ? d.J + 2 : d.J) * (c == 2 ? d.K + 2 : d.K);
    }
    s.bytes_h2d = h2d;
    s.bytes_d2h = d2h;
    s.ms_h2d = ms_between(t0, t_in_end);
    s.ms_d2h = ms_between(t_dev_end, t_out_end > t_dev_end ? t_out_end : t_dev_end);
    s.ms_total = ms_between(t0, t1);
    if (stats) *stats = s;
    if (rc != SCF_OK) return rc;
    return converged_or_report(ctx, s);
}

extern "C" int scf_mom_device_fields(scf_mom_ctx *ctx, const double **pred_u, const double **pred_v,
                                     const double **pred_w, const double **pu_dp, const double **pv_dp,
                                     const double **pw_dp)
{
    if (!ctx) return SCF_ERR_BAD_ARG;
    if (!ctx->ran) return SCF_ERR_NO_SOLVE;
    if (pred_u) *pred_u = ctx->pred[0];
    if (pred_v) *pred_v = ctx->pred[1];
    if (pred_w) *pred_w = ctx->pred[2];
    if (pu_dp) *pu_dp = ctx->dp[0];
    if (pv_dp) *pv_dp = ctx->dp[1];
    if (pw_dp) *pw_dp = ctx->dp[2];
    return SCF_OK;
}

extern "C" int scf_mom_last_error(scf_mom_ctx *ctx, char *buf, size_t n)
{
    if (!ctx || !buf || n == 0) return SCF_ERR_BAD_ARG;
    std::snprintf(buf, n, "%s", ctx->err);
    return SCF_OK;
}
