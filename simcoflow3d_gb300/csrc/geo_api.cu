// geo_api.cu -- C ABI of the cut-cell geometry preprocessing
// (include/scf_geometry.h): device buffers of the four cell families, the
// copies in and out, and the launch sequence of GridPreprocess +
// DefineMomentumExchangeCell + NumberExternalCell x4.
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/scf_geometry.h"
#include "../../include/scf_projection.h"
#include "geo_kernels.h"
#include "scf_devmem.h"
#include "scf_stage.h"

struct scf_geo_ctx {
    Dims d;
    int device = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t evf[8] = {};   // around the four face kernels
    std::vector<void *> mem;
    GeoFam fam[4];
    bool has_moex[4] = {false, false, false, false};
    int *colbuf = nullptr;
    int *counters = nullptr;   // [0..3] family totals, [4] faces evaluated in full
    int ext_cell[4] = {-1, -1, -1, -1};
    bool staged = false, ran = false;
    char err[512] = {0};
};

namespace {

const int CUT[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

void geo_err(scf_geo_ctx *c, const char *fmt, ...)
{
    if (!c) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof(c->err), fmt, ap);
    va_end(ap);
}

#define GK(call)                                                                           \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            geo_err(ctx, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return e_ == cudaErrorMemoryAllocation ? SCF_ERR_OUT_OF_MEMORY : SCF_ERR_CUDA;  \
        }                                                                                  \
    } while (0)

template <typename P>
int galloc(scf_geo_ctx *ctx, P **ptr, size_t count)
{
    void *p = nullptr;
    const size_t bytes = count * sizeof(P) > 0 ? count * sizeof(P) : 16;
    cudaError_t e = scf_mem::dev_malloc(&p, bytes);
    if (e != cudaSuccess) {
        geo_err(ctx, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
        return SCF_ERR_OUT_OF_MEMORY;
    }
    ctx->mem.push_back(p);
    *ptr = (P *)p;
    return SCF_OK;
}

size_t posnu_count(const Dims &d, int f)
{
    return (size_t)(d.I - CUT[f][0]) * (d.J - CUT[f][1]) * (d.K - CUT[f][2]);
}

// One host<->device copy per array; the layouts are identical.
struct Item {
    void *dev;
    size_t bytes;
};

// Arrays copied in by stage (inputs and in/out arrays) and out by fetch
// (in/out and out arrays) for family f.
void items(scf_geo_ctx *ctx, int f, std::vector<Item> &in, std::vector<Item> &out)
{
    const Dims &d = ctx->d;
    const size_t n = d.n, ng = d.ng;
    GeoFam &t = ctx->fam[f];
    const size_t D = sizeof(double), I4 = sizeof(int);
    in = {{(void *)t.dx, n * D}, {(void *)t.dy, n * D}, {(void *)t.dz, n * D}, {(void *)t.phi, ng * D},
          {(void *)t.nx, ng * D}, {(void *)t.ny, ng * D}, {(void *)t.nz, ng * D}, {t.vof, ng * D},
          {t.vofl, ng * D}, {t.ct, n * I4}, {t.ee, ng * D}, {t.ne, ng * D}, {t.te, ng * D},
          {t.fce, 3 * ng * D}, {t.fcn, 3 * ng * D}, {t.fct, 3 * ng * D}, {t.cent, 3 * n * D},
          {t.wllh, n * D}, {t.delh, n * D}};
    out = {{t.vof, ng * D}, {t.vofl, ng * D}, {t.ct, n * I4}, {t.ee, ng * D}, {t.ne, ng * D},
           {t.te, ng * D}, {t.fce, 3 * ng * D}, {t.fcn, 3 * ng * D}, {t.fct, 3 * ng * D},
           {t.cent, 3 * n * D}, {t.wllh, n * D}, {t.delh, n * D}, {t.posnu, posnu_count(d, f) * I4}};
    if (ctx->has_moex[f]) {
        in.push_back({t.moex, n * I4});
        out.push_back({t.moex, n * I4});
    }
}

// Host pointers of a family in the order of items().
void host_ptrs(const scf_geo_cells *c, bool moex, std::vector<const void *> &in, std::vector<void *> &out)
{
    in = {c->dx, c->dy, c->dz, c->phi, c->nx, c->ny, c->nz, c->vof, c->vofl, c->cell_type, c->eearea,
          c->nearea, c->tearea, c->fce, c->fcn, c->fct, c->cell_cent, c->wllh, c->delh};
    out = {c->vof, c->vofl, c->cell_type, c->eearea, c->nearea, c->tearea, c->fce, c->fcn, c->fct,
           c->cell_cent, c->wllh, c->delh, c->posnu};
    if (moex) {
        in.push_back(c->moexcell);
        out.push_back(c->moexcell);
    }
}

int check_fams(scf_geo_ctx *ctx, const scf_geo_cells *const fams[4])
{
    for (int f = 0; f < 4; ++f) {
        const scf_geo_cells *c = fams[f];
        if (!c) { geo_err(ctx, "family %d is NULL", f); return SCF_ERR_BAD_ARG; }
        std::vector<const void *> in;
        std::vector<void *> out;
        host_ptrs(c, false, in, out);
        for (const void *p : in)
            if (!p) { geo_err(ctx, "family %d: an array pointer is NULL", f); return SCF_ERR_BAD_ARG; }
        if (!c->posnu) { geo_err(ctx, "family %d: posnu is NULL", f); return SCF_ERR_BAD_ARG; }
        if (f > 0 && !c->moexcell) {
            geo_err(ctx, "family %d: moexcell is NULL (DefineMomentumExchangeCell writes it)", f);
            return SCF_ERR_BAD_ARG;
        }
    }
    return SCF_OK;
}

int check_ctx(scf_geo_ctx *ctx)
{
    if (!ctx) return SCF_ERR_BAD_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) { geo_err(ctx, "cudaSetDevice: %s", cudaGetErrorString(e)); return SCF_ERR_CUDA; }
    return SCF_OK;
}

double ms_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" {

int scf_geo_create(scf_geo_ctx **out, int32_t imax, int32_t jmax, int32_t kmax, int32_t device)
{
    if (!out) return SCF_ERR_BAD_ARG;
    *out = nullptr;
    if (imax < 2 || jmax < 2 || kmax < 2) return SCF_ERR_BAD_ARG;
    const long long ng = (long long)(imax + 2) * (jmax + 2) * (kmax + 2);
    if (3 * ng >= (1ll << 31)) return SCF_ERR_BAD_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SCF_ERR_NO_DEVICE;
    if (device < 0 || device >= ndev) return SCF_ERR_BAD_ARG;
    scf_geo_ctx *ctx = new scf_geo_ctx();
    ctx->device = device;
    Dims &d = ctx->d;
    d.I = imax; d.J = jmax; d.K = kmax;
    d.gx = imax + 2; d.gy = jmax + 2; d.gz = kmax + 2;
    d.ng = (int)ng;
    d.n = imax * jmax * kmax;
    int rc = SCF_OK;
    auto fail = [&](int r) { scf_geo_destroy(ctx); return r; };
    if (cudaSetDevice(device) != cudaSuccess) return fail(SCF_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess) return fail(SCF_ERR_CUDA);
    if (cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess)
        return fail(SCF_ERR_CUDA);
    for (int q = 0; q < 8; ++q)
        if (cudaEventCreate(&ctx->evf[q]) != cudaSuccess) return fail(SCF_ERR_CUDA);
    const size_t n = d.n, g = d.ng;
    for (int f = 0; f < 4; ++f) {
        GeoFam &t = ctx->fam[f];
        double *dx, *dy, *dz, *phi, *nx, *ny, *nz;
        if ((rc = galloc(ctx, &dx, n)) || (rc = galloc(ctx, &dy, n)) || (rc = galloc(ctx, &dz, n)) ||
            (rc = galloc(ctx, &phi, g)) || (rc = galloc(ctx, &nx, g)) || (rc = galloc(ctx, &ny, g)) ||
            (rc = galloc(ctx, &nz, g)) || (rc = galloc(ctx, &t.vof, g)) || (rc = galloc(ctx, &t.vofl, g)) ||
            (rc = galloc(ctx, &t.ct, n)) || (rc = galloc(ctx, &t.ee, g)) || (rc = galloc(ctx, &t.ne, g)) ||
            (rc = galloc(ctx, &t.te, g)) || (rc = galloc(ctx, &t.fce, 3 * g)) || (rc = galloc(ctx, &t.fcn, 3 * g)) ||
            (rc = galloc(ctx, &t.fct, 3 * g)) || (rc = galloc(ctx, &t.cent, 3 * n)) ||
            (rc = galloc(ctx, &t.wllh, n)) || (rc = galloc(ctx, &t.delh, n)) || (rc = galloc(ctx, &t.moex, n)) ||
            (rc = galloc(ctx, &t.posnu, posnu_count(d, f))))
            return fail(rc);
        t.dx = dx; t.dy = dy; t.dz = dz; t.phi = phi; t.nx = nx; t.ny = ny; t.nz = nz;
        t.iu = CUT[f][0]; t.iv = CUT[f][1]; t.iw = CUT[f][2];
    }
    if ((rc = galloc(ctx, &ctx->colbuf, (size_t)imax * jmax)) || (rc = galloc(ctx, &ctx->counters, 8)))
        return fail(rc);
    *out = ctx;
    return SCF_OK;
}

int scf_geo_destroy(scf_geo_ctx *ctx)
{
    if (!ctx) return SCF_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    for (void *p : ctx->mem) scf_mem::dev_free(p);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    for (int q = 0; q < 8; ++q)
        if (ctx->evf[q]) cudaEventDestroy(ctx->evf[q]);
    if (ctx->st) cudaStreamDestroy(ctx->st);
    delete ctx;
    return SCF_OK;
}

int scf_geo_stage(scf_geo_ctx *ctx, const scf_geo_cells *p, const scf_geo_cells *u, const scf_geo_cells *v,
                  const scf_geo_cells *w)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    const scf_geo_cells *fams[4] = {p, u, v, w};
    if ((rc = check_fams(ctx, fams))) return rc;
    for (int f = 0; f < 4; ++f) {
        ctx->has_moex[f] = fams[f]->moexcell != nullptr;
        std::vector<Item> din, dout;
        items(ctx, f, din, dout);
        std::vector<const void *> hin;
        std::vector<void *> hout;
        host_ptrs(fams[f], ctx->has_moex[f], hin, hout);
        for (size_t q = 0; q < din.size(); ++q)
            GK(stage_h2d(din[q].dev, hin[q], din[q].bytes, ctx->st, 0, nullptr, nullptr));
    }
    GK(cudaStreamSynchronize(ctx->st));
    ctx->staged = true;
    ctx->ran = false;
    return SCF_OK;
}

int scf_geo_run(scf_geo_ctx *ctx, scf_geo_stats *stats)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!ctx->staged) { geo_err(ctx, "no inputs staged"); return SCF_ERR_NO_SOLVE; }
    const Dims &d = ctx->d;
    int launches = 0;
    GeoFam fam[4];
    for (int f = 0; f < 4; ++f) {
        fam[f] = ctx->fam[f];
        if (!ctx->has_moex[f]) fam[f].moex = nullptr;
    }
    GK(cudaMemsetAsync(ctx->counters, 0, 8 * sizeof(int), ctx->st));
    GK(cudaEventRecord(ctx->ev0, ctx->st));
    for (int f = 0; f < 4; ++f) launch_cell_geo(fam[f], d, ctx->counters + 4, ctx->st, &launches, ctx->evf + 2 * f);
    launch_grid_preprocess_tail(fam[0], fam[1], fam[2], fam[3], d, ctx->counters + 4, ctx->st, &launches);
    for (int f = 0; f < 4; ++f) launch_posnu(fam[f], d, ctx->colbuf, ctx->counters + f, ctx->st, &launches);
    GK(cudaGetLastError());
    GK(cudaEventRecord(ctx->ev1, ctx->st));
    int cnt[8];
    GK(cudaMemcpyAsync(cnt, ctx->counters, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->st));
    GK(cudaStreamSynchronize(ctx->st));
    for (int f = 0; f < 4; ++f) ctx->ext_cell[f] = cnt[f] - 1;
    float ms = 0.f, msf = 0.f;
    GK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    for (int f = 0; f < 4; ++f) {
        float m = 0.f;
        GK(cudaEventElapsedTime(&m, ctx->evf[2 * f], ctx->evf[2 * f + 1]));
        msf += m;
    }
    ctx->ran = true;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->gpu_launches = launches;
        stats->exact_faces = cnt[4];
        stats->ms_device = ms;
        stats->ms_total = ms;
        stats->ms_faces = msf;
        // per cell: dx, dy, dz, phi, nx, ny, nz read; EEArea, NEArea, TEArea,
        // FCE, FCN, FCT (3 each), Cell_Cent (3) and WlLh written (FP64 each)
        stats->bytes_faces = 4ll * (long long)d.n * 8 * (7 + 3 + 9 + 3 + 1);
    }
    return SCF_OK;
}

int scf_geo_fetch(scf_geo_ctx *ctx, scf_geo_cells *p, scf_geo_cells *u, scf_geo_cells *v, scf_geo_cells *w)
{
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!ctx->ran) { geo_err(ctx, "no run to fetch"); return SCF_ERR_NO_SOLVE; }
    scf_geo_cells *fams[4] = {p, u, v, w};
    const scf_geo_cells *cf[4] = {p, u, v, w};
    if ((rc = check_fams(ctx, cf))) return rc;
    for (int f = 0; f < 4; ++f) {
        if ((fams[f]->moexcell != nullptr) != ctx->has_moex[f]) {
            geo_err(ctx, "family %d: moexcell differs from the staged call", f);
            return SCF_ERR_BAD_ARG;
        }
        std::vector<Item> din, dout;
        items(ctx, f, din, dout);
        std::vector<const void *> hin;
        std::vector<void *> hout;
        host_ptrs(fams[f], ctx->has_moex[f], hin, hout);
        for (size_t q = 0; q < dout.size(); ++q)
            GK(stage_d2h(hout[q], dout[q].dev, dout[q].bytes, ctx->st, 0, nullptr, nullptr));
        fams[f]->ext_cell = ctx->ext_cell[f];
    }
    GK(cudaStreamSynchronize(ctx->st));
    return SCF_OK;
}

int scf_grid_preprocess(scf_geo_ctx *ctx, scf_geo_cells *p, scf_geo_cells *u, scf_geo_cells *v, scf_geo_cells *w,
                        scf_geo_stats *stats)
{
    const auto t0 = std::chrono::steady_clock::now();
    int rc = scf_geo_stage(ctx, p, u, v, w);
    if (rc) return rc;
    const double h2d = ms_since(t0);
    scf_geo_stats st;
    std::memset(&st, 0, sizeof(st));
    if ((rc = scf_geo_run(ctx, &st))) return rc;
    const auto t1 = std::chrono::steady_clock::now();
    if ((rc = scf_geo_fetch(ctx, p, u, v, w))) return rc;
    const double d2h = ms_since(t1);
    if (stats) {
        *stats = st;
        stats->ms_h2d = h2d;
        stats->ms_d2h = d2h;
        stats->ms_total = ms_since(t0);
        long long bi = 0, bo = 0;
        for (int f = 0; f < 4; ++f) {
            std::vector<Item> din, dout;
            items(ctx, f, din, dout);
            for (auto &x : din) bi += (long long)x.bytes;
            for (auto &x : dout) bo += (long long)x.bytes;
        }
        stats->bytes_h2d = bi;
        stats->bytes_d2h = bo;
    }
    return SCF_OK;
}

int scf_geo_last_error(scf_geo_ctx *ctx, char *buf, size_t n)
{
    if (!ctx || !buf || n == 0) return SCF_ERR_BAD_ARG;
    std::snprintf(buf, n, "%s", ctx->err);
    return SCF_OK;
}

}  // extern "C"
