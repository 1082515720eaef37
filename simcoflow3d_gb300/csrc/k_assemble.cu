// k_assemble.cu -- face coefficients, pressure operator and right-hand side.
//
// Compiled with -fmad=false: every product and sum is rounded on its own, in
// the reference's evaluation order, so PoCoef, the operator and b are
// bit-identical to a strict IEEE evaluation of the Fortran expressions.
#include <cuda_pipeline.h>

#include "scf_kernels.h"

namespace {

// 1 = wet, 2 = dry, 0 = neither (ProjectionP.f90:170-174,212-221)
__device__ __forceinline__ int phase_of(double vofl, double vof, double phil, double epsi)
{
    const double hi = 1.0 - epsi;
    if ((vofl >= 0.5 && vof > hi) || (phil < 0.0 && vof <= hi && vof > epsi)) return 1;
    if ((vofl < 0.5 && vof > hi) || (phil >= 0.0 && vof <= hi && vof > epsi)) return 2;
    return 0;
}

// Direction table, faces W,S,B,E,N,T (PoCoef order).
__device__ __constant__ int c_di[6] = {-1, 0, 0, 1, 0, 0};
__device__ __constant__ int c_dj[6] = {0, -1, 0, 0, 1, 0};
__device__ __constant__ int c_dk[6] = {0, 0, -1, 0, 0, 1};

struct FaceGeo {
    const double *dp, *dg;
};

__device__ __forceinline__ FaceGeo face_geo(const AsmArgs &a, int f)
{
    FaceGeo g;
    const int axis = f % 3;
    g.dp = axis == 0 ? a.dpu : axis == 1 ? a.dpv : a.dpw;
    g.dg = axis == 0 ? a.udx : axis == 1 ? a.vdy : a.wdz;
    return g;
}

// Dp(im,jm,km)/DGrid with DGrid at (max(im,1),max(jm,1),max(km,1))
// (ProjectionP.f90:145-153).
__device__ __forceinline__ void face_terms(const AsmArgs &a, int f, int i, int j, int k, double &dp, double &dgrid)
{
    const Dims &d = a.d;
    const int minus = f < 3;
    const int im = i - (minus ? (c_di[f] != 0) : 0);
    const int jm = j - (minus ? (c_dj[f] != 0) : 0);
    const int km = k - (minus ? (c_dk[f] != 0) : 0);
    FaceGeo g = face_geo(a, f);
    dp = g.dp[gidx(d, im, jm, km)];
    dgrid = g.dg[nidx(d, im < 1 ? 1 : im, jm < 1 ? 1 : jm, km < 1 ? 1 : km)];
}

// The reference's coefficient expression Dp/DGrid*BetaP*BetaM/Beta.
__device__ __forceinline__ double coef_expr(double dp, double dgrid, double betap, double betam, double beta)
{
    double t = dp / dgrid;
    t = t * betap;
    t = t * betam;
    return t / beta;
}

__device__ __forceinline__ double lamda_of(const AsmArgs &a, int gc, int gn)
{
    const double pc = fabs(a.phil[gc]), pn = fabs(a.phil[gn]);
    return pc / ((pc + pn) + a.tol);
}

}  // namespace

// ---------------------------------------------------------------------------
// K1: Compute1DGFMCoefficient for the six faces (ProjectionP.f90:123-265).
//
// The reference's BetaW/BetaD are locals that keep their last assigned value:
// a wet (dry) cell whose neighbour is neither wet nor dry reuses the BetaW
// (BetaD) of the latest earlier cell, in its loop order (i outer, j, k
// innermost), that assigned it within the same face call.  Each thread
// marches one (i,j) column in k -- exactly a contiguous run of that loop
// order -- and carries the twelve (face, W/D) values in registers.  For
// parallelism a column is cut into segments of KSEG cells; segments are
// contiguous runs of the loop order too.  Cells with no earlier assignment
// inside their segment ("head" cells) are listed and resolved from
// per-segment and per-group summaries (k_pocoef_heads).
constexpr int KSEG = SCF_KSEG;

namespace {
__device__ __forceinline__ double beta_of(int pc, int pn, double lam, double betap, double betam)
{
    if (pc == 1) return pn == 2 ? lam * betam + (1.0 - lam) * betap : betam;
    return pn == 1 ? lam * betap + (1.0 - lam) * betam : betap;
}
}  // namespace

// Results are memoised on the bit patterns of their inputs: along a column
// the inputs of a face repeat in uniform regions, and an IEEE operation on
// identical inputs gives an identical result, so reusing it is exact.  This
// removes almost all FP64 divisions, whose throughput on this GPU is low.
struct CoefMemo {
    unsigned long long dp, dg, beta;
    double coef;
    bool valid;
};

// The FP64 work of a memo miss lives in functions that are never inlined:
// a call cannot be executed speculatively, while inline code in a short
// branch is often turned into unconditional arithmetic plus a select -- on
// this GPU that put every division and product back on every cell.
__device__ __noinline__ double coef_slow(double dp, double dg, double betap, double betam, double beta)
{
    return coef_expr(dp, dg, betap, betam, beta);
}

// GFM beta of a wet-dry face (ProjectionP.f90:155-156,176,218)
__device__ __noinline__ double beta_interface(double phic, double phin, double tol, int pc, double betap,
                                              double betam)
{
    const double x = fabs(phic), y = fabs(phin);
    const double lam = x / ((x + y) + tol);
    return pc == 1 ? lam * betam + (1.0 - lam) * betap : lam * betap + (1.0 - lam) * betam;
}

// The B face of cell k has the inputs of the T face of cell k-1 whenever both
// cells are in the same phase (Dp(k-1), DGrid(k-1) and the phase's beta):
// before the B face's own memo, it looks at the T face's memo, which still
// holds cell k-1's result when the B face of cell k is formed.
__device__ __forceinline__ bool memo_hit(const CoefMemo &m, double dp, double dg, double beta)
{
    return m.valid && (unsigned long long)__double_as_longlong(dp) == m.dp &&
           (unsigned long long)__double_as_longlong(dg) == m.dg &&
           (unsigned long long)__double_as_longlong(beta) == m.beta;
}

__device__ __forceinline__ double coef_memo(CoefMemo &m, double dp, double dg, double beta, double betap,
                                            double betam)
{
    const unsigned long long a = __double_as_longlong(dp), b = __double_as_longlong(dg),
                             c = __double_as_longlong(beta);
    if (!m.valid || a != m.dp || b != m.dg || c != m.beta) {
        m.dp = a; m.dg = b; m.beta = c; m.valid = true;
        m.coef = coef_slow(dp, dg, betap, betam, beta);
    }
    return m.coef;
}

// Phase of every ghosted cell (1 wet, 2 dry, 0 neither), once per call.
__global__ void __launch_bounds__(256) k_phase(AsmArgs a)
{
    const int ng = a.d.ng;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x)
        a.phase[g] = (unsigned char)phase_of(a.vofl[g], a.vof[g], a.phil[g], a.epsi);
}

// Inputs of the six faces of one cell: phases of the cell and of its
// neighbours W,S,B,E,N,T, and the Dp / DGrid pair of each face.
struct FaceIn {
    int ph[7];        // 0..5 neighbours in face order, 6 the cell
    double dp[6], dg[6];
};

// Loads of the cell (i,j,k) except the B face, whose inputs are those of the
// T face of (i,j,k-1) and are carried by the caller.
__device__ __forceinline__ void load_face_in(const AsmArgs &a, int i, int j, int k, int im, int jm, FaceIn &v)
{
    const Dims &d = a.d;
    const int sy = d.gx, sz = d.gx * d.gy;
    const int gc = gidx(d, i, j, k), nc = nidx(d, i, j, k);
    v.ph[6] = a.phase[gc];
    v.ph[0] = a.phase[gc - 1]; v.ph[1] = a.phase[gc - sy];
    v.ph[3] = a.phase[gc + 1]; v.ph[4] = a.phase[gc + sy]; v.ph[5] = a.phase[gc + sz];
    // Dp(im,jm,km) and DGrid(max(im,1),...) (ProjectionP.f90:145-153)
    v.dp[0] = a.dpu[gc - 1];  v.dg[0] = a.udx[nidx(d, im, j, k)];
    v.dp[1] = a.dpv[gc - sy]; v.dg[1] = a.vdy[nidx(d, i, jm, k)];
    v.dp[3] = a.dpu[gc];      v.dg[3] = a.udx[nc];
    v.dp[4] = a.dpv[gc];      v.dg[4] = a.vdy[nc];
    v.dp[5] = a.dpw[gc];      v.dg[5] = a.wdz[nc];
}

// Each thread marches one k segment of one (i,j) column.  The inputs of the
// next cell are loaded before the current one is processed (their latency
// overlaps its work), and the B face reuses the T-face inputs of the cell
// below.
__global__ void __launch_bounds__(128) k_pocoef(AsmArgs a)
{
    const Dims &d = a.d;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > d.I || j > d.J) return;
    const int nsk = (d.K + KSEG - 1) / KSEG, sk = blockIdx.z;
    const int col = (i - 1) * d.J + (j - 1);   // column index in loop order
    const int seg = col * nsk + sk;            // segment index in loop order
    const int kbeg = sk * KSEG + 1, kend = min(kbeg + KSEG - 1, d.K);
    const int sy = d.gx, sz = d.gx * d.gy;
    const int goff[6] = {-1, -sy, -sz, 1, sy, sz};
    double carryW[6], carryD[6];
    unsigned maskW = 0, maskD = 0;
    CoefMemo memo[6];
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        carryW[f] = 0.0; carryD[f] = 0.0;
        memo[f].valid = false; memo[f].dp = memo[f].dg = memo[f].beta = 0ull; memo[f].coef = 0.0;
    }
    const int im = i > 1 ? i - 1 : 1, jm = j > 1 ? j - 1 : 1;
    FaceIn cur, nxt;
    load_face_in(a, i, j, kbeg, im, jm, cur);
    {   // B face of the first cell: Dp(i,j,kbeg-1), DGrid(i,j,max(kbeg-1,1))
        const int gc = gidx(d, i, j, kbeg);
        cur.ph[2] = a.phase[gc - sz];
        cur.dp[2] = a.dpw[gc - sz];
        cur.dg[2] = a.wdz[nidx(d, i, j, kbeg > 1 ? kbeg - 1 : 1)];
    }
    for (int k = kbeg; k <= kend; ++k) {
        if (k < kend) load_face_in(a, i, j, k + 1, im, jm, nxt);
        const int gc = gidx(d, i, j, k), nc = nidx(d, i, j, k);
        const int pc = cur.ph[6];
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            double coef = 0.0;
            if (pc != 0) {
                int pn = cur.ph[f];
                const double dp = cur.dp[f], dg = cur.dg[f];
                double beta;
                bool have = true;
                if (pn == pc) {
                    beta = pc == 1 ? a.betam : a.betap;
                } else if (pn != 0) {
                    beta = beta_interface(a.phil[gc], a.phil[gc + goff[f]], a.tol, pc, a.betap, a.betam);
                } else if (pc == 1 ? (maskW >> f) & 1u : (maskD >> f) & 1u) {
                    beta = pc == 1 ? carryW[f] : carryD[f];
                    pn = -1;   // carried, not assigned
                } else {
                    have = false;
                    unsigned slot = atomicAdd(a.stale_count, 1u);
                    if (slot < a.stale_cap) {
                        const long long L = ((long long)col) * d.K + (k - 1);
                        a.stale_list[slot] = (L << 4) | ((long long)(2 * f + (pc == 2)));
                    } else {
                        atomicOr(a.flags, FLAG_STALE_OVERFLOW);
                    }
                }
                if (have) {
                    if (pn > 0) {
                        if (pc == 1) { carryW[f] = beta; maskW |= 1u << f; }
                        else { carryD[f] = beta; maskD |= 1u << f; }
                    }
                    coef = f == 2 && memo_hit(memo[5], dp, dg, beta)
                               ? memo[5].coef
                               : coef_memo(memo[f], dp, dg, beta, a.betap, a.betam);
                }
            }
            a.pocoef[nc + (long long)d.n * f] = coef;
        }
        if (k < kend) {
            nxt.ph[2] = pc; nxt.dp[2] = cur.dp[5]; nxt.dg[2] = cur.dg[5];
            cur = nxt;
        }
    }
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        a.col_val[(long long)seg * 12 + 2 * f] = carryW[f];
        a.col_val[(long long)seg * 12 + 2 * f + 1] = carryD[f];
    }
    unsigned m = 0;
#pragma unroll
    for (int f = 0; f < 6; ++f) m |= (((maskW >> f) & 1u) << (2 * f)) | (((maskD >> f) & 1u) << (2 * f + 1));
    a.col_mask[seg] = (unsigned short)m;
}

// Group summaries: the last assignment of each (face, W/D) stream within
// 64 consecutive segments.
__global__ void k_pocoef_groups(AsmArgs a, int ncol, int ngrp)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngrp) return;
    double v[12];
    unsigned m = 0;
#pragma unroll
    for (int s = 0; s < 12; ++s) v[s] = 0.0;
    const int c1 = min(ncol, (g + 1) * 64);
    for (int c = g * 64; c < c1; ++c) {
        const unsigned cm = a.col_mask[c];
        if (!cm) continue;
#pragma unroll
        for (int s = 0; s < 12; ++s)
            if (cm & (1u << s)) v[s] = a.col_val[(long long)c * 12 + s];
        m |= cm;
    }
#pragma unroll
    for (int s = 0; s < 12; ++s) a.grp_val[(long long)g * 12 + s] = v[s];
    a.grp_mask[g] = (unsigned short)m;
}

// Head cells: the carried value comes from the latest earlier segment (first
// within the cell's group, then whole groups) that assigned the stream.
__global__ void k_pocoef_heads(AsmArgs a, unsigned count)
{
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const Dims &d = a.d;
    const long long e = a.stale_list[t];
    const int s = (int)(e & 15);
    const int f = s >> 1;
    const long long L = e >> 4;
    const int col = (int)(L / d.K), k = (int)(L % d.K) + 1;
    const int i = col / d.J + 1, j = col % d.J + 1;
    const int nsk = (d.K + KSEG - 1) / KSEG;
    const int seg = col * nsk + (k - 1) / KSEG;
    const unsigned bit = 1u << s;
    double beta = a.stale_init;
    bool found = false;
    const int g = seg / 64;
    for (int c = seg - 1; c >= g * 64; --c)
        if (a.col_mask[c] & bit) { beta = a.col_val[(long long)c * 12 + s]; found = true; break; }
    if (!found)
        for (int q = g - 1; q >= 0; --q)
            if (a.grp_mask[q] & bit) { beta = a.grp_val[(long long)q * 12 + s]; break; }
    double dp, dg;
    face_terms(a, f, i, j, k, dp, dg);
    a.pocoef[nidx(d, i, j, k) + (long long)d.n * f] = coef_expr(dp, dg, a.betap, a.betam, beta);
}

// Boundary planes take the neighbouring plane (ProjectionP.f90:256-264).
__global__ void k_pocoef_boundary(AsmArgs a)
{
    const Dims &d = a.d;
    const int f = blockIdx.z;  // 0..5
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int axis = f % 3;
    const int na = axis == 0 ? d.J : d.I;
    const int nb = axis == 2 ? d.J : d.K;
    if (t >= na * nb) return;
    const int p = t % na + 1, q = t / na + 1;
    const bool minus = f < 3;
    double *pc = a.pocoef + (long long)d.n * f;
    if (axis == 0) {
        const int dst = minus ? 1 : d.I, src = minus ? 2 : d.I - 1;
        pc[nidx(d, dst, p, q)] = pc[nidx(d, src, p, q)];
    } else if (axis == 1) {
        const int dst = minus ? 1 : d.J, src = minus ? 2 : d.J - 1;
        pc[nidx(d, p, dst, q)] = pc[nidx(d, p, src, q)];
    } else {
        const int dst = minus ? 1 : d.K, src = minus ? 2 : d.K - 1;
        pc[nidx(d, p, q, dst)] = pc[nidx(d, p, q, src)];
    }
}

// ---------------------------------------------------------------------------
// K2: operator rows of SetPoissonMatrix (ProjectionP.f90:330-478) and the
// right-hand side of SetPoissonVectors (ProjectionP.f90:513-564).
// Per active cell: the exact diagonal, the couplings towards E/N/T from the
// cell's own row, the diagonal part without a coupling (Dirichlet faces and
// faces to solid cells, used to coarsen), and b.  Solid cells: identity.
namespace {
__device__ __forceinline__ bool finite_bits(double x)
{
    return ((unsigned long long)__double_as_longlong(x) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull;
}
__device__ __forceinline__ unsigned long long bits(double x) { return (unsigned long long)__double_as_longlong(x); }

// ((p*area)*d1)*d2, the face term of SetPoissonMatrix, memoised on its inputs.
// The memo also keeps the partial product (p*ar)*d1: along a column only d2
// (the cell's dz for the x and y faces) often changes in its last bits, and
// then one multiplication finishes the term, in the expression's own order.
struct TermMemo {
    unsigned long long p, ar, d1, d2;
    double pd1, t;
    bool valid;
};
__device__ __noinline__ double prod3(double p, double ar, double d1) { return p * ar * d1; }
__device__ __noinline__ double mul_slow(double a, double b) { return a * b; }
__device__ __forceinline__ double term_memo(TermMemo &m, double p, double ar, double d1, double d2)
{
    const bool head = m.valid && bits(p) == m.p && bits(ar) == m.ar && bits(d1) == m.d1;
    if (!head) {
        m.p = bits(p); m.ar = bits(ar); m.d1 = bits(d1); m.valid = true;
        m.pd1 = prod3(p, ar, d1);
        m.d2 = bits(d2);
        m.t = mul_slow(m.pd1, d2);
    } else if (bits(d2) != m.d2) {
        m.d2 = bits(d2);
        m.t = mul_slow(m.pd1, d2);
    }
    return m.t;
}
// The diagonal of a row: the six own-side terms minus those of Neumann
// boundary faces (bit f of nb set) (ProjectionP.f90:378-430).
__device__ __noinline__ double row_diag(double t1, double t2, double t3, double t4, double t5, double t6, int nb)
{
    double v = t1 + t2 + t3 + t4 + t5 + t6;
    if (nb & 1) v = v - t1;
    if (nb & 2) v = v - t2;
    if (nb & 4) v = v - t3;
    if (nb & 8) v = v - t4;
    if (nb & 16) v = v - t5;
    if (nb & 32) v = v - t6;
    return v;
}
// 0 + the terms of the faces in mask m, in face order (ProjectionP.f90:378-430)
__device__ __noinline__ double extra_sum(double t1, double t2, double t3, double t4, double t5, double t6, int m)
{
    double v = 0.0;
    if (m & 1) v += t1;
    if (m & 2) v += t2;
    if (m & 4) v += t3;
    if (m & 8) v += t4;
    if (m & 16) v += t5;
    if (m & 32) v += t6;
    return v;
}
__device__ __noinline__ double recip_slow(double v) { return v > 0.0 ? 1.0 / v : 0.0; }
// -dy*dz, dx*dz, dx*dy of the rhs (ProjectionP.f90:521-526)
__device__ __noinline__ double3 spacing_products(double dx, double dy, double dz)
{
    return make_double3(-dy * dz, dx * dz, dx * dy);
}
// (vof - vofO)*dx*dy*dz/dt (ProjectionP.f90:527)
__device__ __noinline__ double vof_term(double vf, double vo, double dx, double dy, double dz, double dt)
{
    return (vf - vo) * dx * dy * dz / dt;
}
// a*u with a == 1.0 short-cut (exact: 1.0*u == u)
__device__ __forceinline__ double amul(double ar, double u)
{
    return bits(ar) == 0x3ff0000000000000ull ? u : mul_slow(ar, u);
}
}  // namespace

// Staged inputs of one cell of k_operator: FP64 values and int32 values,
// one smem column per thread (struct of arrays: consecutive threads hit
// consecutive banks).
enum OpVal { V_DX, V_DY, V_DZ, V_P1, V_P2, V_P3, V_P4, V_P5, V_P6, V_EW, V_EE, V_NS, V_NN, V_TB, V_TT,
             V_UW, V_UE, V_VS, V_VN, V_WB, V_WT, V_VF, V_VO, V_COUNT };
enum OpInt { I_CT, I_POS, I_PW, I_PE, I_PS, I_PN, I_PB, I_PT, I_COUNT };
constexpr int OP_THREADS = 128;
constexpr size_t OP_SMEM = 2 * (sizeof(double) * V_COUNT + sizeof(int) * I_COUNT) * OP_THREADS;

// Asynchronous copies (cp.async) of cell (i,j,k)'s inputs into stage `st`:
// the loads of the next cell are in flight while the current one is
// computed, without holding registers.  Neighbour PosNu entries that the
// cell does not use read the cell's own entry (always in range).
__device__ __forceinline__ void op_issue(const AsmArgs &a, double *sd, int *si, int tid, int i, int j, int k)
{
    const Dims &d = a.d;
    const int sy = d.gx, sz = d.gx * d.gy;
    const int g = gidx(d, i, j, k), n = nidx(d, i, j, k);
    const long long N = d.n;
    const double *src[V_COUNT] = {a.pdx + n, a.pdy + n, a.pdz + n, a.pocoef + n, a.pocoef + n + N,
                                  a.pocoef + n + 2 * N, a.pocoef + n + 3 * N, a.pocoef + n + 4 * N,
                                  a.pocoef + n + 5 * N, a.ee + g - 1, a.ee + g, a.ne + g - sy, a.ne + g,
                                  a.te + g - sz, a.te + g, a.us + g - 1, a.us + g, a.vs + g - sy, a.vs + g,
                                  a.ws + g - sz, a.ws + g, a.vof + g, a.vofo + g};
#pragma unroll
    for (int v = 0; v < V_COUNT; ++v) __pipeline_memcpy_async(sd + v * OP_THREADS + tid, src[v], sizeof(double));
    const int IJ = d.I * d.J;
    const int *isrc[I_COUNT] = {a.ct + n, a.pos + n, a.pos + (i > 1 ? n - 1 : n), a.pos + (i < d.I ? n + 1 : n),
                                a.pos + (j > 1 ? n - d.I : n), a.pos + (j < d.J ? n + d.I : n),
                                a.pos + (k > 1 ? n - IJ : n), a.pos + (k < d.K ? n + IJ : n)};
#pragma unroll
    for (int v = 0; v < I_COUNT; ++v) __pipeline_memcpy_async(si + v * OP_THREADS + tid, isrc[v], sizeof(int));
    __pipeline_commit();
}

// Matrix rows, FP32 copies and right-hand side of each cell (a block is
// 32 x 4 columns, each thread marches one KSEG segment along k).  The
// inputs of cell k+1 are copied into shared memory while cell k is
// computed (two stages).
template <bool MIXED>
__global__ void __launch_bounds__(OP_THREADS, 3) k_operator(AsmArgs a, OpArgs o)
{
    extern __shared__ __align__(16) unsigned char op_smem[];
    double *sd0 = (double *)op_smem;
    int *si0 = (int *)(sd0 + 2 * V_COUNT * OP_THREADS);
    const Dims &d = a.d;
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > d.I || j > d.J) return;
    const int kbeg = blockIdx.z * KSEG + 1, kend = min(kbeg + KSEG - 1, d.K);
    const int *fl = a.flag;
    TermMemo tm[6];
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        tm[f].valid = false; tm[f].p = tm[f].ar = tm[f].d1 = tm[f].d2 = 0ull; tm[f].pd1 = tm[f].t = 0.0;
    }
    // memo of the row (diag and dependants) on the six terms and the
    // Neumann-face mask
    unsigned long long rt[6] = {0, 0, 0, 0, 0, 0};
    int rnb = -1;
    double dg = 0.0, dinv = 0.0;
    float d32 = 0.f;
    // memo of the spacing products of the rhs
    unsigned long long pdx = 0, pdy = 0, pdz = 0;
    double dydz = 0.0, dxdz = 0.0, dxdy = 0.0;
    bool pvalid = false;
    op_issue(a, sd0, si0, tid, i, j, kbeg);
    unsigned char ph_next = a.phase[gidx(d, i, j, kbeg)];
    for (int k = kbeg; k <= kend; ++k) {
        const int st = (k - kbeg) & 1;
        const double *sd = sd0 + st * V_COUNT * OP_THREADS;
        const int *si = si0 + st * I_COUNT * OP_THREADS;
        const unsigned char ph = ph_next;
        if (k < kend) {
            op_issue(a, sd0 + (st ^ 1) * V_COUNT * OP_THREADS, si0 + (st ^ 1) * I_COUNT * OP_THREADS, tid, i, j, k + 1);
            ph_next = a.phase[gidx(d, i, j, k + 1)];
            __pipeline_wait_prior(1);
        } else {
            __pipeline_wait_prior(0);
        }
#define SV(v) sd[(v) * OP_THREADS + tid]
#define SI(v) si[(v) * OP_THREADS + tid]
        const int g = gidx(d, i, j, k);
        const int ct = SI(I_CT), pos = SI(I_POS);
        if ((pos == -1) != (ct == 2) || pos > a.ext_cell || pos < -1) atomicOr(a.flags, FLAG_BAD_POSNU);
        if (ct == 2) {   // solid: identity-free row, marked by diag = -1 (x stays 0 there)
            o.diag[g] = -1.0; o.dinv[g] = 0.0; o.cE[g] = 0.0; o.cN[g] = 0.0; o.cT[g] = 0.0;
            o.extra[g] = 0.0; o.b[g] = 0.0; o.active[g] = 0;
            if (MIXED) {
                o.diag32[g] = -1.0f; o.cE32[g] = 0.0f; o.cN32[g] = 0.0f; o.cT32[g] = 0.0f;
                o.diag_lo[g] = 0.0f; o.cE_lo[g] = 0.0f; o.cN_lo[g] = 0.0f; o.cT_lo[g] = 0.0f;
                o.extra32[g] = 0.0f;
            }
            continue;
        }
        const double dx = SV(V_DX), dy = SV(V_DY), dz = SV(V_DZ);
        const double p1 = SV(V_P1), p2 = SV(V_P2), p3 = SV(V_P3);
        const double p4 = SV(V_P4), p5 = SV(V_P5), p6 = SV(V_P6);
        const double eW = SV(V_EW), eE = SV(V_EE);
        const double nS = SV(V_NS), nN = SV(V_NN);
        const double tB = SV(V_TB), tT = SV(V_TT);
        const double t1 = term_memo(tm[0], p1, eW, dy, dz), t2 = term_memo(tm[1], p2, nS, dx, dz);
        // the B term of cell k is the T term of cell k-1 when its inputs are
        // (same coefficient, the same TEArea entry, and dx, dy of a tensor
        // grid): tm[5] still holds cell k-1's T term here
        const double t3 = (tm[5].valid && bits(p3) == tm[5].p && bits(tB) == tm[5].ar && bits(dx) == tm[5].d1 &&
                           bits(dy) == tm[5].d2)
                              ? tm[5].t
                              : term_memo(tm[2], p3, tB, dx, dy);
        const double t4 = term_memo(tm[3], p4, eE, dy, dz);
        const double t5 = term_memo(tm[4], p5, nN, dx, dz), t6 = term_memo(tm[5], p6, tT, dx, dy);
        const bool bnd = i == 1 || j == 1 || k == 1 || i == d.I || j == d.J || k == d.K;
        const int nb = (fl[0] == 1 && i == 1 ? 1 : 0) | (fl[2] == 1 && j == 1 ? 2 : 0) |
                       (fl[4] == 1 && k == 1 ? 4 : 0) | (fl[1] == 1 && i == d.I ? 8 : 0) |
                       (fl[3] == 1 && j == d.J ? 16 : 0) | (fl[5] == 1 && k == d.K ? 32 : 0);
        if (nb != rnb || bits(t1) != rt[0] || bits(t2) != rt[1] || bits(t3) != rt[2] || bits(t4) != rt[3] ||
            bits(t5) != rt[4] || bits(t6) != rt[5]) {
            dg = row_diag(t1, t2, t3, t4, t5, t6, nb);
            if (!MIXED) dinv = recip_slow(dg);
            if (MIXED) d32 = scf_to_f32(dg);
            rnb = nb;
            rt[0] = bits(t1); rt[1] = bits(t2); rt[2] = bits(t3); rt[3] = bits(t4); rt[4] = bits(t5); rt[5] = bits(t6);
        }
        // faces whose term goes to the extra diagonal part: Dirichlet
        // boundary faces and faces to solid cells (bit f, order W,S,B,E,N,T)
        double cE = 0.0, cN = 0.0, cT = 0.0;
        int xm = 0;
        if (i == 1) { if (fl[0] == 0) xm |= 1; } else if (SI(I_PW) == -1) xm |= 1;
        if (j == 1) { if (fl[2] == 0) xm |= 2; } else if (SI(I_PS) == -1) xm |= 2;
        if (k == 1) { if (fl[4] == 0) xm |= 4; } else if (SI(I_PB) == -1) xm |= 4;
        if (i == d.I) { if (fl[1] == 0) xm |= 8; } else if (SI(I_PE) == -1) xm |= 8; else cE = t4;
        if (j == d.J) { if (fl[3] == 0) xm |= 16; } else if (SI(I_PN) == -1) xm |= 16; else cN = t5;
        if (k == d.K) { if (fl[5] == 0) xm |= 32; } else if (SI(I_PT) == -1) xm |= 32; else cT = t6;
        const double ex = xm ? extra_sum(t1, t2, t3, t4, t5, t6, xm) : 0.0;

        // right-hand side (ProjectionP.f90:521-546), same rounding as the
        // Fortran expression: -dy*dz*(A) - dx*dz*(B) - dx*dy*(C)
        if (!pvalid || bits(dx) != pdx || bits(dy) != pdy || bits(dz) != pdz) {
            pdx = bits(dx); pdy = bits(dy); pdz = bits(dz); pvalid = true;
            const double3 sp = spacing_products(dx, dy, dz);
            dydz = sp.x; dxdz = sp.y; dxdy = sp.z;
        }
        const double A = amul(eE, SV(V_UE)) - amul(eW, SV(V_UW));
        const double B = amul(nN, SV(V_VN)) - amul(nS, SV(V_VS));
        const double Cc = amul(tT, SV(V_WT)) - amul(tB, SV(V_WB));
        double r = dydz * A - dxdz * B - dxdy * Cc;
        const double vf = SV(V_VF), vo = SV(V_VO);
#undef SV
#undef SI
        if (bits(vf) == bits(vo) && finite_bits(vf)) {
            // (vof - vofO)*dx*dy*dz/dt is +0 exactly, and r + 0.0 is r except
            // that -0 becomes +0
            if (bits(r) == 0x8000000000000000ull) r = 0.0;
        } else {
            r = r + vof_term(vf, vo, dx, dy, dz, a.dt);
        }
        if (bnd) {
            if (fl[0] == 0 && i == 1) r = r + p1 * a.bvar[0][(j - 1) + d.J * (k - 1)];
            if (fl[1] == 0 && i == d.I) r = r + p4 * a.bvar[1][(j - 1) + d.J * (k - 1)];
            if (fl[2] == 0 && j == 1) r = r + p2 * a.bvar[2][(i - 1) + d.I * (k - 1)];
            if (fl[3] == 0 && j == d.J) r = r + p5 * a.bvar[3][(i - 1) + d.I * (k - 1)];
            if (fl[4] == 0 && k == 1) r = r + p3 * a.bvar[4][(i - 1) + d.I * (j - 1)];
            if (fl[5] == 0 && k == d.K) r = r + p6 * a.bvar[5][(i - 1) + d.I * (j - 1)];
        }
        if (!finite_bits(dg)) atomicOr(a.flags, FLAG_NONFINITE);
        else if ((long long)bits(dg) <= 0) atomicOr(a.flags, FLAG_BAD_DIAG);   // dg <= 0 (finite)
        if (!finite_bits(r) || !finite_bits(cE) || !finite_bits(cN) || !finite_bits(cT) || !finite_bits(ex))
            atomicOr(a.flags, FLAG_NONFINITE);
        if (ph == 0) atomicOr(a.flags, FLAG_NEITHER_ACTIVE);

        o.diag[g] = dg;
        if (!MIXED) o.dinv[g] = dinv;
        o.cE[g] = cE; o.cN[g] = cN; o.cT[g] = cT;
        o.extra[g] = ex;
        o.b[g] = r;
        o.active[g] = 1;
        if (MIXED) {
            o.diag32[g] = d32;
            o.diag_lo[g] = scf_lo_part(dg, d32);
            const float e32 = scf_to_f32(cE), n32 = scf_to_f32(cN), t32 = scf_to_f32(cT);
            o.cE32[g] = e32; o.cN32[g] = n32; o.cT32[g] = t32;
            o.cE_lo[g] = scf_lo_part(cE, e32);
            o.cN_lo[g] = scf_lo_part(cN, n32);
            o.cT_lo[g] = scf_lo_part(cT, t32);
            o.extra32[g] = scf_to_f32(ex);
        }
    }
}

// ---------------------------------------------------------------------------
// host launchers
int launch_assemble(const AsmArgs &a, const OpArgs &o, bool mixed, const double *rho, double rho_ref,
                    cudaStream_t st, unsigned *stale_count_host, int *launches)
{
    const Dims &d = a.d;
    cudaMemsetAsync(a.stale_count, 0, sizeof(unsigned), st);
    if (rho) {
        k_phase<<<2 * 152 * 8, 256, 0, st>>>(a);
        launch_pocoef_rho(a, rho, rho_ref, st, launches);
        *launches += 1;
        *stale_count_host = 0;
    } else {
        dim3 b(32, 4), g((d.I + 31) / 32, (d.J + 3) / 4, (d.K + KSEG - 1) / KSEG);
        k_phase<<<2 * 152 * 8, 256, 0, st>>>(a);
        k_pocoef<<<g, b, 0, st>>>(a);
        *launches += 2;
        cudaMemcpyAsync(stale_count_host, a.stale_count, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
    }
    unsigned cnt = *stale_count_host;
    if (cnt > a.stale_cap) cnt = a.stale_cap;
    if (cnt) {
        const int ncol = d.I * d.J * ((d.K + KSEG - 1) / KSEG), ngrp = (ncol + 63) / 64;
        k_pocoef_groups<<<(ngrp + 127) / 128, 128, 0, st>>>(a, ncol, ngrp);
        k_pocoef_heads<<<(cnt + 127) / 128, 128, 0, st>>>(a, cnt);
        *launches += 2;
    }
    {
        int m = d.J * d.K;
        if (d.I * d.K > m) m = d.I * d.K;
        if (d.I * d.J > m) m = d.I * d.J;
        dim3 g((m + 255) / 256, 1, 6);
        k_pocoef_boundary<<<g, 256, 0, st>>>(a);
        *launches += 1;
    }
    dim3 ob(32, 4), og((d.I + 31) / 32, (d.J + 3) / 4, (d.K + KSEG - 1) / KSEG);
    // the staged inputs need more than the default 48 KB of dynamic shared
    // memory (set per device, so on every call)
    cudaFuncSetAttribute(k_operator<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OP_SMEM);
    cudaFuncSetAttribute(k_operator<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OP_SMEM);
    if (mixed)
        k_operator<true><<<og, ob, OP_SMEM, st>>>(a, o);
    else
        k_operator<false><<<og, ob, OP_SMEM, st>>>(a, o);
    *launches += 1;
    return (int)cudaGetLastError();
}
