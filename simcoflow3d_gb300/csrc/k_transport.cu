// k_transport.cu -- the CLSVOF interface transport on the device and its C
// ABI (include/scf_clsvof.h).
//
// One time step is six sub-steps; a sub-step is
//   3 x (k_reconstruct, k_sweep)   the split sweeps, each cell gathering its
//                                  own face fluxes (no scatter, no atomics)
//                                  with the divergence term fused in;
//   k_walls                        the wall planes and ghosts;
//   k_reconstruct (tail)           normals, liquid normals, centre distances;
//   k_band_reset, k_band_pairs,    the redistancing: the reset lists the
//   k_band_value                   interface cells; then one block per
//                                  listed cell computes its 9^3 band pairs,
//                                  one pair per thread, and sends each
//                                  distance with a 64-bit atomicMin
//                                  (non-negative doubles order like their
//                                  bits), so the result is the reference's
//                                  running minimum whatever the order.
// The VOF and level set ping-pong through three buffers (the sub-step's
// input, its first sweep's result, which the later sweeps' divergence terms
// read, and the second sweep's result); every sub-step ends in buffer 0.
// The sweeps write interior cells only: k_walls writes the ghost faces into
// all three buffers, and staging fills all three, so their ghosts agree.
// Kernels over cells run on 3-D grids (i along x, j and k as blockIdx.y/z),
// so no thread decodes its cell with integer division.
// Built with -fmad=false: the bodies round like the reference's Fortran.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/scf_clsvof.h"
#include "transport_body.cuh"
#include "scf_devmem.h"
#include "scf_stage.h"

using tr::Dims;
using tr::Geo;

struct scf_clsvof_ctx {
    Dims D{};
    int device = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[4] = {};
    std::vector<void *> mem;
    double *geo[6] = {};                 // x, y, z, dx, dy, dz
    double *vf[3] = {}, *ls[3] = {};     // ghosted ping-pong
    double *nx = nullptr, *ny = nullptr, *nz = nullptr, *dis = nullptr;
    double *nxl = nullptr, *nyl = nullptr, *nzl = nullptr;
    double *fn[3] = {};                  // fluid normals
    double *vel[3] = {};
    double *bc_vel[3] = {};              // W, S, B planes of u, v, w
    double *lvs_bc[6] = {}, *vof_bc[6] = {};
    unsigned long long *key = nullptr;
    uint8_t *fix = nullptr;
    uint32_t *band_list = nullptr;       // interface cells of the sub-step (interior indices)
    unsigned *nband = nullptr;           // how many
    double *vgeo[3][3] = {};             // U, V, W grid spacings (allocated on first use)
    double *vfld[3][5] = {};             // U, V, W: phiL, nxL, nyL, nzL, vofL
    int lvs_flag[6] = {}, vof_flag[6] = {};
    double lvs_const[6] = {}, vof_const[6] = {};
    double dt = 0.0;
    bool staged = false;
    bool timing = false;
    std::vector<cudaEvent_t> tev;        // 2 per launch of a step when timing
    std::vector<int> tkind;              // kernel kind of each timed launch
    char err[512] = {0};
};

namespace {

constexpr int NT = 256;   // threads per block of the linear kernels
constexpr int NX = 128;   // threads along i of the 3-D kernels

void tr_err(scf_clsvof_ctx *c, const char *fmt, ...)
{
    if (!c) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof(c->err), fmt, ap);
    va_end(ap);
}

#define TK(call)                                                                            \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            tr_err(ctx, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return e_ == cudaErrorMemoryAllocation ? SCF_ERR_OUT_OF_MEMORY : SCF_ERR_CUDA;   \
        }                                                                                   \
    } while (0)

int blocks_for(size_t n)
{
    const size_t b = (n + NT - 1) / NT;
    return (int)std::min<size_t>(std::max<size_t>(b, 1), (size_t)152 * 64);
}

Geo geo_of(const scf_clsvof_ctx *c)
{
    return Geo{c->geo[0], c->geo[1], c->geo[2], c->geo[3], c->geo[4], c->geo[5]};
}

// ---- kernels -------------------------------------------------------------

// Interface_Reconstruct over the interior; with `tail` also the liquid
// normals and the distance from the cell centre (Clsvof_Scheme 767-778).
__global__ void k_reconstruct(Dims D, Geo G, const double *__restrict__ vfl, const double *__restrict__ phi,
                              double *nx, double *ny, double *nz, double *dis, int tail, double *nxl, double *nyl,
                              double *nzl)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z + 1;
    if (i > D.I) return;
    double n1, n2, n3, d1;
    tr::reconstruct(D, G, vfl, phi, i, j, k, n1, n2, n3, d1);
    const size_t g = D.g(i, j, k), t = D.n(i, j, k);
    nx[g] = n1;
    ny[g] = n2;
    nz[g] = n3;
    if (tail) {
        nxl[g] = n1;
        nyl[g] = n2;
        nzl[g] = n3;
        d1 = (0.5 * G.dx[t] * fabs(n1) + 0.5 * G.dy[t] * fabs(n2) + 0.5 * G.dz[t] * fabs(n3)) - d1;
    }
    dis[g] = d1;
}

// One directional sweep over the interior cells.
__global__ void k_sweep(Dims D, Geo G, tr::SweepIn S, double *__restrict__ vf_out, double *__restrict__ ls_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z + 1;
    if (i > D.I) return;
    double a, b;
    tr::sweep_cell(D, G, S, i, j, k, a, b);
    const size_t t = D.g(i, j, k);
    vf_out[t] = a;
    ls_out[t] = b;
}

// BoundaryConditionLvsVof: blockIdx.y is the axis, x strides its planes.
__global__ void k_walls(Dims D, Geo G, tr::WallIn W)
{
    const int axis = blockIdx.y;
    const size_t np = D.plane_size(axis);
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < np; t += (size_t)gridDim.x * blockDim.x)
        tr::wall_point(D, G, W, axis, t);
}

// Resets the band keys and marks, and lists the interface cells (warp-
// aggregated appends; the list's order does not matter).
__global__ void k_band_reset(Dims D, const double *__restrict__ vfl, unsigned long long *key, uint8_t *fix,
                             uint32_t *list, unsigned *count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z + 1;
    const bool in = i <= D.I;
    bool src = false;
    if (in) {
        const size_t c = D.n(i, j, k);
        key[c] = (unsigned long long)tr::key_of(1.0e4);
        fix[c] = 0;
        src = tr::band_interface(vfl[D.g(i, j, k)]);
    }
    const unsigned mask = __ballot_sync(0xffffffffu, src);
    if (!mask) return;
    const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (src) list[base + __popc(mask & ((1u << lane) - 1u))] = (uint32_t)D.n(i, j, k);
}

// The band pairs of the listed interface cells: a block takes one cell at a
// time and its threads the cell's 729 offsets.
__global__ void __launch_bounds__(256, 2) k_band_pairs(Dims D, Geo G, const double *__restrict__ vfl,
                                                    const double *__restrict__ phi, const double *__restrict__ nx,
                                                    const double *__restrict__ ny, const double *__restrict__ nz,
                                                    const double *__restrict__ dis, const uint32_t *__restrict__ list,
                                                    const unsigned *__restrict__ count, unsigned long long *key,
                                                    uint8_t *fix)
{
    const unsigned n = *count;
    for (unsigned q = blockIdx.x; q < n; q += gridDim.x) {
        int i, j, k;
        tr::cell_of(D, list[q], i, j, k);
        for (int t = threadIdx.x; t < tr::BAND_CELLS; t += blockDim.x)
            tr::band_pair(D, G, vfl, phi, nx, ny, nz, dis, i, j, k, t, key, fix);
    }
}

__global__ void k_band_value(Dims D, Geo G, const double *__restrict__ vfl, const double *__restrict__ dis,
                             const unsigned long long *__restrict__ key, const uint8_t *__restrict__ fix,
                             double *phi)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z + 1;
    if (i > D.I) return;
    phi[D.g(i, j, k)] = tr::band_value(D, G, vfl, dis, i, j, k, key, fix);
}

// ComputeUVWLiquidField for one family over its ghosted grid: the cells of
// (0:I-1,0:J-1,0:K-1) take the direction averages, the interior cells the
// liquid fraction.
__global__ void k_uvw(Dims D, int fam, Geo G, const double *__restrict__ phil, const double *__restrict__ nxl,
                      const double *__restrict__ nyl, const double *__restrict__ nzl, const double *__restrict__ vofl,
                      const double *__restrict__ vdx, const double *__restrict__ vdy, const double *__restrict__ vdz,
                      double *o_phil, double *o_nxl, double *o_nyl, double *o_nzl, double *o_vofl)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
    if (i > D.I + 1) return;
    const double *pin[4] = {phil, nxl, nyl, nzl};
    const double *d = fam == 0 ? G.dx : fam == 1 ? G.dy : G.dz;
    const size_t t = D.g(i, j, k);
    if (i < D.I && j < D.J && k < D.K) {
        double av[4];
        tr::family_average(D, fam, d, pin, i, j, k, av);
        o_phil[t] = av[0];
        o_nxl[t] = av[1];
        o_nyl[t] = av[2];
        o_nzl[t] = av[3];
    }
    if (i >= 1 && i <= D.I && j >= 1 && j <= D.J && k >= 1 && k <= D.K)
        o_vofl[t] = tr::family_vofl(D, fam, G.dx, G.dy, G.dz, phil, nxl, nyl, nzl, vofl, vdx, vdy, vdz, i, j, k);
}

// ---- one time step ---------------------------------------------------------

int launch_check(scf_clsvof_ctx *ctx, const char *what)
{
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        tr_err(ctx, "%s launch: %s", what, cudaGetErrorString(e));
        return SCF_ERR_CUDA;
    }
    return SCF_OK;
}

// With timing on, an event pair around each launch, tagged with its kind
// (0 reconstruct, 1 sweep, 2 walls, 3 redistancing).
struct Timer {
    scf_clsvof_ctx *ctx;
    int n = 0;
    void before(int kind)
    {
        if (!ctx->timing || (size_t)(2 * n + 1) >= ctx->tev.size()) return;
        cudaEventRecord(ctx->tev[2 * n], ctx->st);
        ctx->tkind[n] = kind;
    }
    void after()
    {
        if (!ctx->timing || (size_t)(2 * n + 1) >= ctx->tev.size()) return;
        cudaEventRecord(ctx->tev[2 * n + 1], ctx->st);
        ++n;
    }
};

// Blocks of k_band_pairs: two per SM (the residency its registers allow),
// each looping over the listed cells.
constexpr int kBandBlocks = 152 * 2;

// Clsvof_Scheme (Clsvof.f90:355-798) on the staged state; counts launches.
int scheme_step(scf_clsvof_ctx *ctx, int &launches, Timer &T)
{
    const Dims D = ctx->D;
    const Geo G = geo_of(ctx);
    const double dtv = ctx->dt / (double)tr::NSUB;
    const dim3 gin((D.I + NX - 1) / NX, D.J, D.K);   // interior cells
    size_t pmax = std::max(D.plane_size(0), std::max(D.plane_size(1), D.plane_size(2)));
    int rc;
    for (int kk = 1; kk <= tr::NSUB; ++kk) {
        const int first = kk % 3 == 0 ? 0 : kk % 3 == 1 ? 1 : 2;
        int cur = 0;
        for (int s = 0; s < 3; ++s) {
            const int ax = (first + s) % 3, out = s == 0 ? 1 : s == 1 ? 2 : 0;
            T.before(0);
            k_reconstruct<<<gin, NX, 0, ctx->st>>>(D, G, ctx->vf[cur], ctx->ls[cur], ctx->nx, ctx->ny, ctx->nz,
                                                   ctx->dis, 0, nullptr, nullptr, nullptr);
            T.after();
            if ((rc = launch_check(ctx, "k_reconstruct")) != SCF_OK) return rc;
            tr::SweepIn S;
            S.vfl = ctx->vf[cur];
            S.phi = ctx->ls[cur];
            S.nx = ctx->nx;
            S.ny = ctx->ny;
            S.nz = ctx->nz;
            S.dis = ctx->dis;
            S.vel = ctx->vel[ax];
            S.bc_vel = ctx->bc_vel[ax];
            S.bc_lvs = ctx->lvs_bc[2 * ax];
            S.vf_first = ctx->vf[1];
            S.ls_first = ctx->ls[1];
            S.dtv = dtv;
            S.axis = ax;
            S.stage = s;
            T.before(1);
            k_sweep<<<gin, NX, 0, ctx->st>>>(D, G, S, ctx->vf[out], ctx->ls[out]);
            T.after();
            if ((rc = launch_check(ctx, "k_sweep")) != SCF_OK) return rc;
            launches += 2;
            cur = out;
        }
        tr::WallIn W;
        W.phil = ctx->ls[0];
        W.vofl = ctx->vf[0];
        for (int q = 0; q < 2; ++q) {
            W.phil_more[q] = ctx->ls[q + 1];
            W.vofl_more[q] = ctx->vf[q + 1];
        }
        W.nxl = ctx->nxl;
        W.nx = ctx->fn[0];
        W.ny = ctx->fn[1];
        W.nz = ctx->fn[2];
        for (int f = 0; f < 6; ++f) {
            W.lvs_bc[f] = ctx->lvs_bc[f];
            W.vof_bc[f] = ctx->vof_bc[f];
            W.lvs_flag[f] = ctx->lvs_flag[f];
            W.vof_flag[f] = ctx->vof_flag[f];
            W.lvs_const[f] = ctx->lvs_const[f];
            W.vof_const[f] = ctx->vof_const[f];
        }
        T.before(2);
        k_walls<<<dim3(blocks_for(pmax), 3), NT, 0, ctx->st>>>(D, G, W);
        T.after();
        if ((rc = launch_check(ctx, "k_walls")) != SCF_OK) return rc;
        T.before(0);
        k_reconstruct<<<gin, NX, 0, ctx->st>>>(D, G, ctx->vf[0], ctx->ls[0], ctx->nx, ctx->ny, ctx->nz, ctx->dis, 1,
                                               ctx->nxl, ctx->nyl, ctx->nzl);
        T.after();
        if ((rc = launch_check(ctx, "k_reconstruct")) != SCF_OK) return rc;
        T.before(3);
        if (cudaMemsetAsync(ctx->nband, 0, sizeof(unsigned), ctx->st) != cudaSuccess)
            return launch_check(ctx, "cudaMemsetAsync");
        k_band_reset<<<gin, NX, 0, ctx->st>>>(D, ctx->vf[0], ctx->key, ctx->fix, ctx->band_list, ctx->nband);
        T.after();
        if ((rc = launch_check(ctx, "k_band_reset")) != SCF_OK) return rc;
        T.before(3);
        k_band_pairs<<<kBandBlocks, 256, 0, ctx->st>>>(D, G, ctx->vf[0], ctx->ls[0], ctx->nx, ctx->ny, ctx->nz,
                                                       ctx->dis, ctx->band_list, ctx->nband, ctx->key, ctx->fix);
        T.after();
        if ((rc = launch_check(ctx, "k_band_pairs")) != SCF_OK) return rc;
        T.before(3);
        k_band_value<<<gin, NX, 0, ctx->st>>>(D, G, ctx->vf[0], ctx->dis, ctx->key, ctx->fix, ctx->ls[0]);
        T.after();
        if ((rc = launch_check(ctx, "k_band_value")) != SCF_OK) return rc;
        launches += 5;
    }
    return SCF_OK;
}

template <typename P>
int alloc(scf_clsvof_ctx *ctx, P **ptr, size_t count)
{
    void *p = nullptr;
    const size_t bytes = std::max<size_t>(count * sizeof(P), 16);
    const cudaError_t e = scf_mem::dev_malloc(&p, bytes);
    if (e != cudaSuccess) {
        tr_err(ctx, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
        return SCF_ERR_OUT_OF_MEMORY;
    }
    ctx->mem.push_back(p);
    *ptr = (P *)p;
    return cudaMemset(p, 0, bytes) == cudaSuccess ? SCF_OK : SCF_ERR_CUDA;
}

float elapsed(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

}  // namespace

extern "C" int scf_clsvof_create(scf_clsvof_ctx **out, int32_t imax, int32_t jmax, int32_t kmax, int32_t device)
{
    if (!out) return SCF_ERR_BAD_ARG;
    *out = nullptr;
    if (imax < 3 || jmax < 3 || kmax < 3 || imax > 65533 || jmax > 65533 || kmax > 65533) return SCF_ERR_BAD_ARG;
    // the redistancing lists interface cells by 32-bit interior index
    if ((unsigned long long)imax * (unsigned long long)jmax * (unsigned long long)kmax >= (1ull << 32))
        return SCF_ERR_BAD_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return SCF_ERR_NO_DEVICE;
    scf_clsvof_ctx *ctx = new scf_clsvof_ctx();
    ctx->device = device;
    ctx->D = Dims{imax, jmax, kmax};
    auto fail = [&](int rc) {
        scf_clsvof_destroy(ctx);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess) return fail(SCF_ERR_CUDA);
    for (auto &e : ctx->ev)
        if (cudaEventCreate(&e) != cudaSuccess) return fail(SCF_ERR_CUDA);
    const size_t nin = ctx->D.interior(), ng = ctx->D.ghosted();
    int rc;
#define TRY(ptr, count)                                         \
    if ((rc = alloc(ctx, &(ptr), (count))) != SCF_OK) return fail(rc);
    for (auto &p : ctx->geo) TRY(p, nin)
    for (int b = 0; b < 3; ++b) { TRY(ctx->vf[b], ng) TRY(ctx->ls[b], ng) }
    TRY(ctx->nx, ng) TRY(ctx->ny, ng) TRY(ctx->nz, ng) TRY(ctx->dis, ng)
    TRY(ctx->nxl, ng) TRY(ctx->nyl, ng) TRY(ctx->nzl, ng)
    for (auto &p : ctx->fn) TRY(p, ng)
    for (auto &p : ctx->vel) TRY(p, ng)
    for (int a = 0; a < 3; ++a) TRY(ctx->bc_vel[a], ctx->D.plane_size(a))
    for (int f = 0; f < 6; ++f) { TRY(ctx->lvs_bc[f], ctx->D.plane_size(f / 2)) TRY(ctx->vof_bc[f], ctx->D.plane_size(f / 2)) }
    TRY(ctx->key, nin) TRY(ctx->fix, nin) TRY(ctx->band_list, nin) TRY(ctx->nband, 1)
#undef TRY
    *out = ctx;
    return SCF_OK;
}

extern "C" int scf_clsvof_set_timing(scf_clsvof_ctx *ctx, int32_t on)
{
    if (!ctx) return SCF_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    const size_t need = 2 * (size_t)tr::NSUB * 11;   // two events per launch of a step
    while (on && ctx->tev.size() < need) {
        cudaEvent_t e = nullptr;
        TK(cudaEventCreate(&e));
        ctx->tev.push_back(e);
    }
    ctx->tkind.assign(need / 2, 0);
    ctx->timing = on != 0;
    return SCF_OK;
}

extern "C" int scf_clsvof_destroy(scf_clsvof_ctx *ctx)
{
    if (!ctx) return SCF_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    for (cudaEvent_t e : ctx->tev) cudaEventDestroy(e);
    for (void *p : ctx->mem) scf_mem::dev_free(p);
    for (auto &e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->st) cudaStreamDestroy(ctx->st);
    delete ctx;
    return SCF_OK;
}

extern "C" int scf_clsvof_stage(scf_clsvof_ctx *ctx, const scf_clsvof_in *in, const scf_clsvof_state *s)
{
    if (!ctx || !in || !s) return SCF_ERR_BAD_ARG;
    const double *need[] = {in->x, in->y, in->z, in->dx, in->dy, in->dz, in->u, in->v, in->w, in->nx, in->ny,
                            in->nz, in->bc_u_w, in->bc_v_s, in->bc_w_b, s->vofl, s->phil, s->nxl, s->nyl, s->nzl};
    for (const double *p : need)
        if (!p) {
            tr_err(ctx, "scf_clsvof_stage: a required array is null");
            return SCF_ERR_BAD_ARG;
        }
    for (int f = 0; f < 6; ++f)
        if (!s->lvs_bc[f]) {
            tr_err(ctx, "scf_clsvof_stage: lvs_bc[%d] is null", f);
            return SCF_ERR_BAD_ARG;
        }
    if (!(in->dt >= 0.0) || !std::isfinite(in->dt)) {
        tr_err(ctx, "scf_clsvof_stage: dt must be finite and >= 0");
        return SCF_ERR_BAD_ARG;
    }
    cudaSetDevice(ctx->device);
    const size_t nin = ctx->D.interior(), ng = ctx->D.ghosted();
    const size_t bi = nin * sizeof(double), bg = ng * sizeof(double);
    const double *geo[6] = {in->x, in->y, in->z, in->dx, in->dy, in->dz};
    for (int q = 0; q < 6; ++q) TK(stage_h2d(ctx->geo[q], geo[q], bi, ctx->st, 0, nullptr, nullptr));
    const double *vel[3] = {in->u, in->v, in->w}, *fn[3] = {in->nx, in->ny, in->nz};
    const double *bcv[3] = {in->bc_u_w, in->bc_v_s, in->bc_w_b};
    for (int a = 0; a < 3; ++a) {
        TK(stage_h2d(ctx->vel[a], vel[a], bg, ctx->st, 0, nullptr, nullptr));
        TK(stage_h2d(ctx->fn[a], fn[a], bg, ctx->st, 0, nullptr, nullptr));
        TK(stage_h2d(ctx->bc_vel[a], bcv[a], ctx->D.plane_size(a) * sizeof(double), ctx->st, 0, nullptr, nullptr));
    }
    TK(stage_h2d(ctx->vf[0], s->vofl, bg, ctx->st, 0, nullptr, nullptr));
    TK(stage_h2d(ctx->ls[0], s->phil, bg, ctx->st, 0, nullptr, nullptr));
    for (int b = 1; b < 3; ++b) {   // the ping-pong buffers' ghosts must match buffer 0's
        TK(cudaMemcpyAsync(ctx->vf[b], ctx->vf[0], bg, cudaMemcpyDeviceToDevice, ctx->st));
        TK(cudaMemcpyAsync(ctx->ls[b], ctx->ls[0], bg, cudaMemcpyDeviceToDevice, ctx->st));
    }
    TK(stage_h2d(ctx->nxl, s->nxl, bg, ctx->st, 0, nullptr, nullptr));
    TK(stage_h2d(ctx->nyl, s->nyl, bg, ctx->st, 0, nullptr, nullptr));
    TK(stage_h2d(ctx->nzl, s->nzl, bg, ctx->st, 0, nullptr, nullptr));
    for (int f = 0; f < 6; ++f)
        TK(cudaMemcpyAsync(ctx->lvs_bc[f], s->lvs_bc[f], ctx->D.plane_size(f / 2) * sizeof(double),
                           cudaMemcpyHostToDevice, ctx->st));
    for (int f = 0; f < 6; ++f) {
        ctx->lvs_flag[f] = in->lvs_flag[f];
        ctx->vof_flag[f] = in->vof_flag[f];
        ctx->lvs_const[f] = in->lvs_const[f];
        ctx->vof_const[f] = in->vof_const[f];
    }
    ctx->dt = in->dt;
    TK(cudaStreamSynchronize(ctx->st));
    ctx->staged = true;
    return SCF_OK;
}

extern "C" int scf_clsvof_run(scf_clsvof_ctx *ctx, int32_t steps, scf_clsvof_stats *stats)
{
    if (!ctx || steps < 0) return SCF_ERR_BAD_ARG;
    if (!ctx->staged) {
        tr_err(ctx, "scf_clsvof_run: nothing staged");
        return SCF_ERR_BAD_ARG;
    }
    cudaSetDevice(ctx->device);
    int launches = 0, rc;
    double ms_kind[4] = {0.0, 0.0, 0.0, 0.0};
    TK(cudaEventRecord(ctx->ev[0], ctx->st));
    for (int n = 0; n < steps; ++n) {
        Timer T{ctx};
        if ((rc = scheme_step(ctx, launches, T)) != SCF_OK) return rc;
        if (ctx->timing) {
            TK(cudaStreamSynchronize(ctx->st));
            for (int q = 0; q < T.n; ++q) ms_kind[ctx->tkind[q]] += elapsed(ctx->tev[2 * q], ctx->tev[2 * q + 1]);
        }
    }
    TK(cudaEventRecord(ctx->ev[1], ctx->st));
    TK(cudaStreamSynchronize(ctx->st));
    if (stats) {
        stats->ms_run = elapsed(ctx->ev[0], ctx->ev[1]);
        stats->steps = steps;
        stats->gpu_launches = launches;
        for (int q = 0; q < 4; ++q) stats->ms_kernels[q] = ms_kind[q];
    }
    return SCF_OK;
}

extern "C" int scf_clsvof_fetch(scf_clsvof_ctx *ctx, scf_clsvof_state *s, scf_clsvof_stats *stats)
{
    if (!ctx || !s) return SCF_ERR_BAD_ARG;
    if (!ctx->staged) {
        tr_err(ctx, "scf_clsvof_fetch: nothing staged");
        return SCF_ERR_BAD_ARG;
    }
    double *need[] = {s->vofl, s->phil, s->nxl, s->nyl, s->nzl};
    for (double *p : need)
        if (!p) return SCF_ERR_BAD_ARG;
    for (int f = 0; f < 6; ++f)
        if (!s->lvs_bc[f] || !s->vof_bc[f]) return SCF_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    const size_t bg = ctx->D.ghosted() * sizeof(double);
    TK(cudaEventRecord(ctx->ev[2], ctx->st));
    TK(stage_d2h(s->vofl, ctx->vf[0], bg, ctx->st, 0, nullptr, nullptr));
    TK(stage_d2h(s->phil, ctx->ls[0], bg, ctx->st, 0, nullptr, nullptr));
    TK(stage_d2h(s->nxl, ctx->nxl, bg, ctx->st, 0, nullptr, nullptr));
    TK(stage_d2h(s->nyl, ctx->nyl, bg, ctx->st, 0, nullptr, nullptr));
    TK(stage_d2h(s->nzl, ctx->nzl, bg, ctx->st, 0, nullptr, nullptr));
    int64_t planes = 0;
    for (int f = 0; f < 6; ++f) {
        const size_t pb = ctx->D.plane_size(f / 2) * sizeof(double);
        TK(stage_d2h(s->lvs_bc[f], ctx->lvs_bc[f], pb, ctx->st, 0, nullptr, nullptr));
        TK(stage_d2h(s->vof_bc[f], ctx->vof_bc[f], pb, ctx->st, 0, nullptr, nullptr));
        planes += 2 * (int64_t)pb;
    }
    TK(cudaEventRecord(ctx->ev[3], ctx->st));
    TK(cudaStreamSynchronize(ctx->st));
    if (stats) {
        stats->ms_d2h = elapsed(ctx->ev[2], ctx->ev[3]);
        stats->bytes_d2h = 5 * (int64_t)bg + planes;
    }
    return SCF_OK;
}

extern "C" int scf_clsvof_step(scf_clsvof_ctx *ctx, const scf_clsvof_in *in, scf_clsvof_state *s,
                               scf_clsvof_stats *stats)
{
    if (!ctx) return SCF_ERR_BAD_ARG;
    scf_clsvof_stats local{};
    scf_clsvof_stats *st = stats ? stats : &local;
    *st = scf_clsvof_stats{};
    cudaSetDevice(ctx->device);
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    TK(cudaEventCreate(&t0));
    TK(cudaEventCreate(&t1));
    int rc = SCF_OK;
    cudaEventRecord(t0, ctx->st);
    if ((rc = scf_clsvof_stage(ctx, in, s)) == SCF_OK) {
        cudaEventRecord(t1, ctx->st);
        cudaEventSynchronize(t1);
        st->ms_h2d = elapsed(t0, t1);
        const size_t nin = ctx->D.interior(), ng = ctx->D.ghosted();
        int64_t planes = 0;
        for (int a = 0; a < 3; ++a) planes += (int64_t)ctx->D.plane_size(a) * 3;   // bc_vel + two lvs planes
        st->bytes_h2d = (int64_t)(6 * nin + 11 * ng) * 8 + planes * 8;
        if ((rc = scf_clsvof_run(ctx, 1, st)) == SCF_OK) rc = scf_clsvof_fetch(ctx, s, st);
    }
    cudaEventRecord(t1, ctx->st);
    cudaEventSynchronize(t1);
    st->ms_total = elapsed(t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    return rc;
}

extern "C" int scf_clsvof_uvw_liquid_field(scf_clsvof_ctx *ctx, const scf_clsvof_vcell cells[3],
                                           scf_clsvof_stats *stats)
{
    if (!ctx || !cells) return SCF_ERR_BAD_ARG;
    if (!ctx->staged) {
        tr_err(ctx, "scf_clsvof_uvw_liquid_field: nothing staged");
        return SCF_ERR_BAD_ARG;
    }
    for (int f = 0; f < 3; ++f) {
        const scf_clsvof_vcell &c = cells[f];
        if (!c.dx || !c.dy || !c.dz || !c.phil || !c.nxl || !c.nyl || !c.nzl || !c.vofl) {
            tr_err(ctx, "scf_clsvof_uvw_liquid_field: a required array of family %d is null", f);
            return SCF_ERR_BAD_ARG;
        }
    }
    cudaSetDevice(ctx->device);
    const size_t nin = ctx->D.interior(), ng = ctx->D.ghosted();
    int rc;
    for (int f = 0; f < 3; ++f) {
        for (auto &p : ctx->vgeo[f])
            if (!p && (rc = alloc(ctx, &p, nin)) != SCF_OK) return rc;
        for (auto &p : ctx->vfld[f])
            if (!p && (rc = alloc(ctx, &p, ng)) != SCF_OK) return rc;
    }
    TK(cudaEventRecord(ctx->ev[0], ctx->st));
    for (int f = 0; f < 3; ++f) {
        const scf_clsvof_vcell &c = cells[f];
        const double *g[3] = {c.dx, c.dy, c.dz};
        double *h[5] = {c.phil, c.nxl, c.nyl, c.nzl, c.vofl};
        for (int q = 0; q < 3; ++q)
            TK(stage_h2d(ctx->vgeo[f][q], g[q], nin * sizeof(double), ctx->st, 0, nullptr, nullptr));
        for (int q = 0; q < 5; ++q)
            TK(stage_h2d(ctx->vfld[f][q], h[q], ng * sizeof(double), ctx->st, 0, nullptr, nullptr));
    }
    TK(cudaEventRecord(ctx->ev[1], ctx->st));
    const Geo G = geo_of(ctx);
    for (int f = 0; f < 3; ++f) {
        const dim3 gg((ctx->D.I + 2 + NX - 1) / NX, ctx->D.J + 2, ctx->D.K + 2);   // ghosted cells
        k_uvw<<<gg, NX, 0, ctx->st>>>(ctx->D, f, G, ctx->ls[0], ctx->nxl, ctx->nyl, ctx->nzl, ctx->vf[0],
                                                 ctx->vgeo[f][0], ctx->vgeo[f][1], ctx->vgeo[f][2], ctx->vfld[f][0],
                                                 ctx->vfld[f][1], ctx->vfld[f][2], ctx->vfld[f][3], ctx->vfld[f][4]);
        if ((rc = launch_check(ctx, "k_uvw")) != SCF_OK) return rc;
    }
    TK(cudaEventRecord(ctx->ev[2], ctx->st));
    for (int f = 0; f < 3; ++f) {
        const scf_clsvof_vcell &c = cells[f];
        double *h[5] = {c.phil, c.nxl, c.nyl, c.nzl, c.vofl};
        for (int q = 0; q < 5; ++q)
            TK(stage_d2h(h[q], ctx->vfld[f][q], ng * sizeof(double), ctx->st, 0, nullptr, nullptr));
    }
    TK(cudaEventRecord(ctx->ev[3], ctx->st));
    TK(cudaStreamSynchronize(ctx->st));
    if (stats) {
        *stats = scf_clsvof_stats{};
        stats->ms_h2d = elapsed(ctx->ev[0], ctx->ev[1]);
        stats->ms_run = elapsed(ctx->ev[1], ctx->ev[2]);
        stats->ms_d2h = elapsed(ctx->ev[2], ctx->ev[3]);
        stats->ms_total = elapsed(ctx->ev[0], ctx->ev[3]);
        stats->bytes_h2d = (int64_t)(3 * (3 * nin + 5 * ng)) * 8;
        stats->bytes_d2h = (int64_t)(15 * ng) * 8;
        stats->gpu_launches = 3;
    }
    return SCF_OK;
}

extern "C" int scf_clsvof_device_fields(scf_clsvof_ctx *ctx, double **vofl, double **phil)
{
    if (!ctx || !vofl || !phil) return SCF_ERR_BAD_ARG;
    *vofl = ctx->staged ? ctx->vf[0] : nullptr;
    *phil = ctx->staged ? ctx->ls[0] : nullptr;
    return SCF_OK;
}

extern "C" int scf_clsvof_last_error(scf_clsvof_ctx *ctx, char *buf, size_t n)
{
    if (!ctx || !buf || n == 0) return SCF_ERR_BAD_ARG;
    snprintf(buf, n, "%s", ctx->err);
    return SCF_OK;
}
