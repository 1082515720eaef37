// gmg.cpp -- CPU multigrid-preconditioned CG for the SIMCOFlow pressure system.
//
// TEST INFRASTRUCTURE ONLY (oracle and timed CPU baseline; never linked into
// the product).  It restates, on the host cores, the solver design of the CUDA
// library so that parity of the device solution can be checked against an
// independent FP64 implementation and so that the benchmark has a CPU path of
// the same algorithm family as the reference's HYPRE PCG + BoomerAMG
// (src/ProjectionP.f90:267-299) to time.
//
// Operator: the 7-point system of SetPoissonMatrix (ProjectionP.f90:301-482)
// in structured form -- per active cell the reference's exact diagonal and
// the couplings to the E/N/T neighbours taken from the cell's own row.  Solid
// cells (Cell_Type == 2, PosNu == -1) are identity rows.
//
// Hierarchy: 2x2x2 cell agglomeration; a coarse face conductance is the
// series combination, along the face normal, of the summed fine conductances
// of the two half-cells and of the coarse face itself; the coarse diagonal is
// the sum of its face conductances plus half the children's Dirichlet terms.
// Smoother: Chebyshev polynomial of the Jacobi-preconditioned operator on
// [lmax/ratio, lmax], lmax = 2 (Gershgorin bound); the Jacobi blocks are single
// cells or (line_seg > 0) segments of line_seg cells along k.  Coarsest level: dense
// Cholesky in FP64 (rank-one regularised when the system is all-Neumann).
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#include <type_traits>
#ifdef _OPENMP
#include <omp.h>
#endif
extern "C" {
#include "../include/scf_projection.h"
}

namespace {

struct Level {
    int n[3];
    size_t sy, sz, tot;   // padded strides
    std::vector<double> diag, cE, cN, cT, extra;  // FP64 master copy
    std::vector<uint8_t> active;
    std::vector<double> dinv;
};

inline size_t pidx(const Level &L, int i, int j, int k) { return (size_t)i + L.sy * (size_t)j + L.sz * (size_t)k; }

void alloc_level(Level &L, int n0, int n1, int n2)
{
    L.n[0] = n0; L.n[1] = n1; L.n[2] = n2;
    L.sy = (size_t)(n0 + 2);
    L.sz = L.sy * (size_t)(n1 + 2);
    L.tot = L.sz * (size_t)(n2 + 2);
    L.diag.assign(L.tot, 0.0); L.cE.assign(L.tot, 0.0); L.cN.assign(L.tot, 0.0); L.cT.assign(L.tot, 0.0);
    L.extra.assign(L.tot, 0.0); L.active.assign(L.tot, 0); L.dinv.assign(L.tot, 0.0);
}

// Coarse conductance between two coarse cells along one axis.
static int g_coarse_mode = -1;
static double g_overcorr = 1.0;
inline double series(double gface, double gl, bool hasl, double gr, bool hasr)
{
    if (g_coarse_mode < 0) {
        const char *e = getenv("SCF_PROTO_COARSE");
        g_coarse_mode = e ? atoi(e) : 2;
        const char *o = getenv("SCF_PROTO_OVERCORR");
        g_overcorr = o ? atof(o) : 1.0;
    }
    if (g_coarse_mode == 1) return gface;
    if (g_coarse_mode == 2) return 0.5 * gface;
    if (!(gface > 0.0)) return 0.0;
    double r = 1.0 / gface;
    if (hasl && gl > 0.0) r += 0.5 / gl;
    if (hasr && gr > 0.0) r += 0.5 / gr;
    return 1.0 / r;
}

void coarsen(const Level &F, Level &C)
{
    int m0 = (F.n[0] + 1) / 2, m1 = (F.n[1] + 1) / 2, m2 = (F.n[2] + 1) / 2;
    if (F.n[0] <= 2) m0 = F.n[0];
    if (F.n[1] <= 2) m1 = F.n[1];
    if (F.n[2] <= 2) m2 = F.n[2];
    alloc_level(C, m0, m1, m2);
    const int f0 = F.n[0] > 2 ? 2 : 1, f1 = F.n[1] > 2 ? 2 : 1, f2 = F.n[2] > 2 ? 2 : 1;
#pragma omp parallel for collapse(2) schedule(static)
    for (int K = 1; K <= m2; ++K)
        for (int J = 1; J <= m1; ++J)
            for (int I = 1; I <= m0; ++I) {
                size_t ci = pidx(C, I, J, K);
                // children range (1-based fine indices)
                int i0 = (I - 1) * f0 + 1, j0 = (J - 1) * f1 + 1, k0 = (K - 1) * f2 + 1;
                int i1 = std::min(i0 + f0 - 1, F.n[0]), j1 = std::min(j0 + f1 - 1, F.n[1]), k1 = std::min(k0 + f2 - 1, F.n[2]);
                bool act = false;
                double ext = 0.0;
                for (int k = k0; k <= k1; ++k)
                    for (int j = j0; j <= j1; ++j)
                        for (int i = i0; i <= i1; ++i) {
                            size_t fi = pidx(F, i, j, k);
                            act = act || F.active[fi];
                            ext += F.extra[fi];
                        }
                C.active[ci] = act;
                C.extra[ci] = 0.5 * ext;
                // x-face towards I+1: fine face between i1 and i1+1
                auto sumE = [&](int ii) {
                    double s = 0.0;
                    for (int k = k0; k <= k1; ++k)
                        for (int j = j0; j <= j1; ++j) s += F.cE[pidx(F, ii, j, k)];
                    return s;
                };
                auto sumN = [&](int jj) {
                    double s = 0.0;
                    for (int k = k0; k <= k1; ++k)
                        for (int i = i0; i <= i1; ++i) s += F.cN[pidx(F, i, jj, k)];
                    return s;
                };
                auto sumT = [&](int kk) {
                    double s = 0.0;
                    for (int j = j0; j <= j1; ++j)
                        for (int i = i0; i <= i1; ++i) s += F.cT[pidx(F, i, j, kk)];
                    return s;
                };
                if (I < m0) {
                    double gf = sumE(i1);
                    bool hl = i1 > i0, hr = i1 + 2 <= std::min(i1 + f0, F.n[0]);
                    double gl = hl ? sumE(i0) : 0.0;
                    double gr = hr ? sumE(i1 + 1) : 0.0;
                    C.cE[ci] = series(gf, gl, hl, gr, hr);
                }
                if (J < m1) {
                    double gf = sumN(j1);
                    bool hl = j1 > j0, hr = j1 + 2 <= std::min(j1 + f1, F.n[1]);
                    double gl = hl ? sumN(j0) : 0.0;
                    double gr = hr ? sumN(j1 + 1) : 0.0;
                    C.cN[ci] = series(gf, gl, hl, gr, hr);
                }
                if (K < m2) {
                    double gf = sumT(k1);
                    bool hl = k1 > k0, hr = k1 + 2 <= std::min(k1 + f2, F.n[2]);
                    double gl = hl ? sumT(k0) : 0.0;
                    double gr = hr ? sumT(k1 + 1) : 0.0;
                    C.cT[ci] = series(gf, gl, hl, gr, hr);
                }
            }
#pragma omp parallel for collapse(2) schedule(static)
    for (int K = 1; K <= m2; ++K)
        for (int J = 1; J <= m1; ++J)
            for (int I = 1; I <= m0; ++I) {
                size_t c = pidx(C, I, J, K);
                if (!C.active[c]) { C.diag[c] = 1.0; C.dinv[c] = 0.0; continue; }
                double d = C.cE[c] + C.cE[c - 1] + C.cN[c] + C.cN[c - C.sy] + C.cT[c] + C.cT[c - C.sz] + C.extra[c];
                C.diag[c] = d;
                C.dinv[c] = d > 0.0 ? 1.0 / d : 0.0;
            }
}

template <typename T>
struct LevelT {
    std::vector<T> diag, cE, cN, cT, dinv, x, b, r, d;
};

template <typename T>
void load_level(const Level &L, LevelT<T> &M)
{
    M.diag.assign(L.diag.begin(), L.diag.end());
    M.cE.assign(L.cE.begin(), L.cE.end());
    M.cN.assign(L.cN.begin(), L.cN.end());
    M.cT.assign(L.cT.begin(), L.cT.end());
    M.dinv.assign(L.dinv.begin(), L.dinv.end());
    M.x.assign(L.tot, T(0)); M.b.assign(L.tot, T(0)); M.r.assign(L.tot, T(0)); M.d.assign(L.tot, T(0));
}

// y = A x (active cells; inactive rows identity)
template <typename T>
inline T apply_at(const Level &L, const LevelT<T> &M, const T *x, size_t c)
{
    return M.diag[c] * x[c] - (M.cE[c] * x[c + 1] + M.cE[c - 1] * x[c - 1] + M.cN[c] * x[c + L.sy] +
                               M.cN[c - L.sy] * x[c - L.sy] + M.cT[c] * x[c + L.sz] + M.cT[c - L.sz] * x[c - L.sz]);
}

#define FOR_CELLS(L)                                  \
    _Pragma("omp parallel for collapse(2) schedule(static)") \
    for (int k = 1; k <= (L).n[2]; ++k)               \
        for (int j = 1; j <= (L).n[1]; ++j)           \
            for (int i = 1; i <= (L).n[0]; ++i)

struct Params {
    int degree = 2;
    double lmax = 2.0, ratio = 6.0;
    int line_seg = 0;   // 0: point Jacobi; n > 0: z-line Jacobi on segments of n cells
};

// out = T^{-1} in on the active cells, T the block diagonal of A whose
// blocks are the segments of `seg` cells along k of each (i, j) column
// (diagonal and T couplings inside a segment), by the Thomas algorithm.
template <typename T>
void line_solve(const Level &L, const LevelT<T> &M, const std::vector<T> &in, std::vector<T> &out, int seg)
{
    const int K = L.n[2];
#pragma omp parallel for collapse(2) schedule(static)
    for (int j = 1; j <= L.n[1]; ++j)
        for (int i = 1; i <= L.n[0]; ++i) {
            std::vector<double> cp(K + 2, 0.0), dp(K + 2, 0.0);
            for (int k = 1; k <= K; ++k) {
                const size_t c = pidx(L, i, j, k);
                if (!L.active[c]) { cp[k] = 0.0; dp[k] = 0.0; continue; }
                const bool first = (k - 1) % seg == 0, last = k % seg == 0;
                const double a = (k > 1 && !first) ? -(double)M.cT[c - L.sz] : 0.0;
                const double cc = (k < K && !last) ? -(double)M.cT[c] : 0.0;
                const double den = (double)M.diag[c] - a * cp[k - 1];
                cp[k] = cc / den;
                dp[k] = ((double)in[c] - a * dp[k - 1]) / den;
            }
            double nxt = 0.0;
            for (int k = K; k >= 1; --k) {
                const size_t c = pidx(L, i, j, k);
                if (k % seg == 0) nxt = 0.0;
                const double v = L.active[c] ? dp[k] - cp[k] * nxt : 0.0;
                out[c] = (T)v;
                nxt = v;
            }
        }
}

// Chebyshev smoothing with the z-line blocks
template <typename T>
void chebyshev_line(const Level &L, LevelT<T> &M, int deg, bool zero_init, const Params &P)
{
    const double lmax = P.lmax, lmin = P.lmax / P.ratio;
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin), sigma = theta / delta;
    double rho = 1.0 / sigma;
    std::vector<T> z(L.tot, T(0));
    {
        T *x = M.x.data();
        FOR_CELLS(L) {
            size_t c = pidx(L, i, j, k);
            M.r[c] = zero_init ? M.b[c] : M.b[c] - apply_at(L, M, x, c);
        }
        line_solve(L, M, M.r, z, P.line_seg);
        FOR_CELLS(L) {
            size_t c = pidx(L, i, j, k);
            M.d[c] = (T)(z[c] / theta);
            M.x[c] = (zero_init ? T(0) : M.x[c]) + M.d[c];
        }
    }
    for (int s = 1; s < deg; ++s) {
        double rho_new = 1.0 / (2.0 * sigma - rho);
        double c1 = rho_new * rho, c2 = 2.0 * rho_new / delta;
        rho = rho_new;
        T *x = M.x.data();
        FOR_CELLS(L) {
            size_t c = pidx(L, i, j, k);
            M.r[c] = M.b[c] - apply_at(L, M, x, c);
        }
        line_solve(L, M, M.r, z, P.line_seg);
        FOR_CELLS(L) {
            size_t c = pidx(L, i, j, k);
            M.d[c] = (T)(c1 * M.d[c] + c2 * z[c]);
            M.x[c] += M.d[c];
        }
    }
}

// Chebyshev smoothing of A x = b, `deg` steps, starting from x (zero if zero_init)
template <typename T>
void chebyshev(const Level &L, LevelT<T> &M, int deg, bool zero_init, const Params &P)
{
    if (P.line_seg > 0) { chebyshev_line(L, M, deg, zero_init, P); return; }
    const double lmax = P.lmax, lmin = P.lmax / P.ratio;
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin), sigma = theta / delta;
    double rho = 1.0 / sigma;
    // step 0: d = D^{-1} r / theta ; x += d
    {
        T *x = M.x.data();
        FOR_CELLS(L) {
            size_t c = pidx(L, i, j, k);
            T r = zero_init ? M.b[c] : M.b[c] - apply_at(L, M, x, c);
            M.d[c] = (T)(M.dinv[c] * r / theta);
        }
        FOR_CELLS(L) {
            size_t c = pidx(L, i, j, k);
            M.x[c] = (zero_init ? T(0) : M.x[c]) + M.d[c];
        }
    }
    for (int s = 1; s < deg; ++s) {
        double rho_new = 1.0 / (2.0 * sigma - rho);
        double c1 = rho_new * rho, c2 = 2.0 * rho_new / delta;
        rho = rho_new;
        T *x = M.x.data();
        FOR_CELLS(L) {
            size_t c = pidx(L, i, j, k);
            T r = M.b[c] - apply_at(L, M, x, c);
            M.r[c] = (T)(c1 * M.d[c] + c2 * M.dinv[c] * r);
        }
        FOR_CELLS(L) {
            size_t c = pidx(L, i, j, k);
            M.d[c] = M.r[c];
            M.x[c] += M.d[c];
        }
    }
}

struct Coarse {
    int n;
    std::vector<double> chol;  // dense lower-triangular factor
    std::vector<int> map;      // dense index -> padded index
};

void coarse_factor(const Level &L, Coarse &C, bool singular)
{
    std::vector<int> map;
    for (int k = 1; k <= L.n[2]; ++k)
        for (int j = 1; j <= L.n[1]; ++j)
            for (int i = 1; i <= L.n[0]; ++i) map.push_back((int)pidx(L, i, j, k));
    int n = (int)map.size();
    std::vector<int> inv(L.tot, -1);
    for (int a = 0; a < n; ++a) inv[map[a]] = a;
    std::vector<double> A((size_t)n * n, 0.0);
    double dsum = 0.0;
    int nact = 0;
    for (int a = 0; a < n; ++a) {
        size_t c = map[a];
        A[(size_t)a * n + a] = L.diag[c];
        if (L.active[c]) { dsum += L.diag[c]; nact++; }
        const size_t nb[6] = {c + 1, c - 1, c + L.sy, c - L.sy, c + L.sz, c - L.sz};
        const double w[6] = {L.cE[c], L.cE[c - 1], L.cN[c], L.cN[c - L.sy], L.cT[c], L.cT[c - L.sz]};
        for (int q = 0; q < 6; ++q)
            if (inv[nb[q]] >= 0 && w[q] != 0.0) A[(size_t)a * n + inv[nb[q]]] -= w[q];
    }
    if (singular && nact > 0) {
        double s = dsum / nact / nact;
        for (int a = 0; a < n; ++a)
            for (int b = 0; b < n; ++b)
                if (L.active[map[a]] && L.active[map[b]]) A[(size_t)a * n + b] += s;
    }
    // Cholesky (lower), guarded
    for (int j = 0; j < n; ++j) {
        double s = A[(size_t)j * n + j];
        for (int p = 0; p < j; ++p) s -= A[(size_t)j * n + p] * A[(size_t)j * n + p];
        double d = s > 0.0 ? std::sqrt(s) : 0.0;
        A[(size_t)j * n + j] = d;
        for (int i = j + 1; i < n; ++i) {
            double t = A[(size_t)i * n + j];
            for (int p = 0; p < j; ++p) t -= A[(size_t)i * n + p] * A[(size_t)j * n + p];
            A[(size_t)i * n + j] = d > 0.0 ? t / d : 0.0;
        }
    }
    C.n = n;
    C.chol = A;
    C.map = map;
}

template <typename T>
void coarse_solve(const Level &L, const Coarse &C, LevelT<T> &M, bool singular)
{
    int n = C.n;
    std::vector<double> y(n);
    double mean = 0.0;
    int nact = 0;
    for (int a = 0; a < n; ++a) {
        y[a] = (double)M.b[C.map[a]];
        if (L.active[C.map[a]]) { mean += y[a]; nact++; }
    }
    if (singular && nact) {
        mean /= nact;
        for (int a = 0; a < n; ++a)
            if (L.active[C.map[a]]) y[a] -= mean;
    }
    for (int i = 0; i < n; ++i) {
        double s = y[i];
        for (int p = 0; p < i; ++p) s -= C.chol[(size_t)i * n + p] * y[p];
        double d = C.chol[(size_t)i * n + i];
        y[i] = d > 0.0 ? s / d : 0.0;
    }
    for (int i = n - 1; i >= 0; --i) {
        double s = y[i];
        for (int p = i + 1; p < n; ++p) s -= C.chol[(size_t)p * n + i] * y[p];
        double d = C.chol[(size_t)i * n + i];
        y[i] = d > 0.0 ? s / d : 0.0;
    }
    for (int a = 0; a < n; ++a) M.x[C.map[a]] = (T)(L.active[C.map[a]] ? y[a] : 0.0);
}

template <typename T>
struct Hier {
    std::vector<Level> *lv;
    std::vector<LevelT<T>> m;
    Coarse coarse;
    bool singular;
    Params P;
};

template <typename T>
void vcycle(Hier<T> &H, int l)
{
    std::vector<Level> &lv = *H.lv;
    const Level &L = lv[l];
    LevelT<T> &M = H.m[l];
    if (l == (int)lv.size() - 1) {
        coarse_solve(L, H.coarse, M, H.singular);
        return;
    }
    chebyshev(L, M, H.P.degree, true, H.P);
    // residual, restrict (sum of children)
    const Level &C = lv[l + 1];
    LevelT<T> &MC = H.m[l + 1];
    {
        T *x = M.x.data();
        FOR_CELLS(L) {
            size_t c = pidx(L, i, j, k);
            M.r[c] = M.b[c] - apply_at(L, M, x, c);
        }
    }
    const int f0 = L.n[0] > 2 ? 2 : 1, f1 = L.n[1] > 2 ? 2 : 1, f2 = L.n[2] > 2 ? 2 : 1;
    std::fill(MC.b.begin(), MC.b.end(), T(0));
    FOR_CELLS(C) {
        size_t cc = pidx(C, i, j, k);
        int i0 = (i - 1) * f0 + 1, j0 = (j - 1) * f1 + 1, k0 = (k - 1) * f2 + 1;
        double s = 0.0;
        for (int kk = k0; kk <= std::min(k0 + f2 - 1, L.n[2]); ++kk)
            for (int jj = j0; jj <= std::min(j0 + f1 - 1, L.n[1]); ++jj)
                for (int ii = i0; ii <= std::min(i0 + f0 - 1, L.n[0]); ++ii) s += (double)M.r[pidx(L, ii, jj, kk)];
        MC.b[cc] = C.active[cc] ? (T)s : T(0);
    }
    vcycle(H, l + 1);
    // prolong (piecewise constant) and correct
    FOR_CELLS(L) {
        size_t c = pidx(L, i, j, k);
        int I = (i - 1) / f0 + 1, J = (j - 1) / f1 + 1, K = (k - 1) / f2 + 1;
        if (L.active[c]) M.x[c] += (T)(g_overcorr * MC.x[pidx(C, I, J, K)]);
    }
    chebyshev(L, M, H.P.degree, false, H.P);
}

double dot_active(const Level &L, const std::vector<double> &a, const std::vector<double> &b)
{
    double s = 0.0;
#pragma omp parallel for collapse(2) reduction(+ : s) schedule(static)
    for (int k = 1; k <= L.n[2]; ++k)
        for (int j = 1; j <= L.n[1]; ++j)
            for (int i = 1; i <= L.n[0]; ++i) {
                size_t c = pidx(L, i, j, k);
                if (L.active[c]) s += a[c] * b[c];
            }
    return s;
}

void project_mean(const Level &L, std::vector<double> &a)
{
    double s = 0.0;
    long cnt = 0;
    for (int k = 1; k <= L.n[2]; ++k)
        for (int j = 1; j <= L.n[1]; ++j)
            for (int i = 1; i <= L.n[0]; ++i) {
                size_t c = pidx(L, i, j, k);
                if (L.active[c]) { s += a[c]; cnt++; }
            }
    if (!cnt) return;
    s /= cnt;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k <= L.n[2]; ++k)
        for (int j = 1; j <= L.n[1]; ++j)
            for (int i = 1; i <= L.n[0]; ++i) {
                size_t c = pidx(L, i, j, k);
                if (L.active[c]) a[c] -= s;
            }
}

void project_mean_f(const Level &L, std::vector<float> &a)
{
    double s = 0.0;
    long cnt = 0;
    for (size_t c = 0; c < L.tot; ++c)
        if (L.active[c]) { s += a[c]; cnt++; }
    if (!cnt) return;
    float m = (float)(s / cnt);
    for (size_t c = 0; c < L.tot; ++c)
        if (L.active[c]) a[c] -= m;
}

}  // namespace

// ---------------------------------------------------------------------------
// Level-0 operator from the reference's formulas.  Outputs (padded (I+2)^3):
// diag (the exact SetPoissonMatrix diagonal), couplings from the cell's own
// row, Dirichlet/solid-face diagonal terms, active mask, and the rhs b.
static void build_level0(int I, int J, int K, const scf_poisson_in *in, const double *pocoef, const double *rhs_posnu,
                         Level &L, std::vector<double> &b)
{
    alloc_level(L, I, J, K);
    b.assign(L.tot, 0.0);
    const int32_t *pos = in->pcell_posnu, *ct = in->pcell_cell_type;
    const double *EE = in->pcell_eearea, *NE = in->pcell_nearea, *TE = in->pcell_tearea;
    auto NIx = [&](int i, int j, int k) { return (size_t)(i - 1) + (size_t)I * ((size_t)(j - 1) + (size_t)J * (k - 1)); };
    auto GIx = [&](int i, int j, int k) { return (size_t)i + (size_t)(I + 2) * ((size_t)j + (size_t)(J + 2) * k); };
    const size_t NN = (size_t)I * J * K;
    const int *fl = in->bcp_flag;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k <= K; ++k)
        for (int j = 1; j <= J; ++j)
            for (int i = 1; i <= I; ++i) {
                size_t n = NIx(i, j, k), c = pidx(L, i, j, k);
                if (ct[n] == 2) { L.diag[c] = 1.0; L.active[c] = 0; continue; }
                L.active[c] = 1;
                double dx = in->pgrid_dx[n], dy = in->pgrid_dy[n], dz = in->pgrid_dz[n];
                double t1 = pocoef[n] * EE[GIx(i - 1, j, k)] * dy * dz;
                double t2 = pocoef[n + NN] * NE[GIx(i, j - 1, k)] * dx * dz;
                double t3 = pocoef[n + 2 * NN] * TE[GIx(i, j, k - 1)] * dx * dy;
                double t4 = pocoef[n + 3 * NN] * EE[GIx(i, j, k)] * dy * dz;
                double t5 = pocoef[n + 4 * NN] * NE[GIx(i, j, k)] * dx * dz;
                double t6 = pocoef[n + 5 * NN] * TE[GIx(i, j, k)] * dx * dy;
                double d = t1 + t2 + t3 + t4 + t5 + t6;
                if (fl[0] == 1 && i == 1) d = d - t1;
                if (fl[2] == 1 && j == 1) d = d - t2;
                if (fl[4] == 1 && k == 1) d = d - t3;
                if (fl[1] == 1 && i == I) d = d - t4;
                if (fl[3] == 1 && j == J) d = d - t5;
                if (fl[5] == 1 && k == K) d = d - t6;
                L.diag[c] = d;
                double ex = 0.0;
                if (i == 1) { if (fl[0] == 0) ex += t1; } else if (pos[NIx(i - 1, j, k)] == -1) ex += t1;
                if (j == 1) { if (fl[2] == 0) ex += t2; } else if (pos[NIx(i, j - 1, k)] == -1) ex += t2;
                if (k == 1) { if (fl[4] == 0) ex += t3; } else if (pos[NIx(i, j, k - 1)] == -1) ex += t3;
                if (i == I) { if (fl[1] == 0) ex += t4; } else if (pos[NIx(i + 1, j, k)] == -1) ex += t4; else L.cE[c] = t4;
                if (j == J) { if (fl[3] == 0) ex += t5; } else if (pos[NIx(i, j + 1, k)] == -1) ex += t5; else L.cN[c] = t5;
                if (k == K) { if (fl[5] == 0) ex += t6; } else if (pos[NIx(i, j, k + 1)] == -1) ex += t6; else L.cT[c] = t6;
                L.extra[c] = ex;
                b[c] = rhs_posnu[pos[n]];
            }
#pragma omp parallel for schedule(static)
    for (size_t c = 0; c < L.tot; ++c) L.dinv[c] = (L.active[c] && L.diag[c] > 0.0) ? 1.0 / L.diag[c] : 0.0;
}

extern "C" {

typedef struct {
    int precision;     // 0 fp64, 1 mixed
    double rel_tol;
    int max_iter;
    int max_rounds;
    double inner_rtol;
    int degree;
    double ratio;
    int coarse_max;
    int line_seg;      // 0: point-Jacobi Chebyshev; n: z-line Jacobi on n-cell segments
    // outputs
    int iterations;
    int rounds;
    int levels;
    double rel_residual;
    double rhs_norm;
} oracle_gmg_params;

// Solve the structured system; x_posnu (length ExtCell+1) receives the
// solution in PosNu order.  Returns 0 if converged, 2 otherwise.
int oracle_gmg_solve(int I, int J, int K, const scf_poisson_in *in, const double *pocoef, const double *rhs_posnu,
                     double *x_posnu, oracle_gmg_params *prm)
{
    std::vector<Level> lv(1);
    std::vector<double> b;
    build_level0(I, J, K, in, pocoef, rhs_posnu, lv[0], b);
    bool singular = true;
    for (int q = 0; q < 6; ++q)
        if (in->bcp_flag[q] == 0) singular = false;
    while ((size_t)lv.back().n[0] * lv.back().n[1] * lv.back().n[2] > (size_t)prm->coarse_max &&
           (lv.back().n[0] > 2 || lv.back().n[1] > 2 || lv.back().n[2] > 2)) {
        lv.emplace_back();
        coarsen(lv[lv.size() - 2], lv.back());
    }
    prm->levels = (int)lv.size();
    const Level &L0 = lv[0];
    if (singular) project_mean(L0, b);
    double bn = std::sqrt(dot_active(L0, b, b));
    prm->rhs_norm = bn;
    std::vector<double> x(L0.tot, 0.0), r(b), z(L0.tot, 0.0), p(L0.tot, 0.0), q(L0.tot, 0.0);
    Params P;
    P.degree = prm->degree;
    P.line_seg = prm->line_seg;
    P.ratio = prm->ratio;
    int its = 0, rounds = 0;
    double relres = bn > 0 ? 1.0 : 0.0;
    // FP64 operator on level 0 for residuals
    LevelT<double> M0;
    load_level(L0, M0);
    auto residual64 = [&]() {
        double *xp = x.data();
        FOR_CELLS(L0) {
            size_t c = pidx(L0, i, j, k);
            r[c] = L0.active[c] ? b[c] - apply_at(L0, M0, xp, c) : 0.0;
        }
        if (singular) project_mean(L0, r);
        return std::sqrt(dot_active(L0, r, r));
    };
    if (bn == 0.0) goto done;
    {
        // FP64 CG.  The V-cycle preconditioner runs in FP64 (precision 0) or
        // FP32 (precision 1: FP32 storage and arithmetic, FP64 coarsest solve).
        Hier<double> H64;
        Hier<float> H32;
        const bool mixed = prm->precision != 0;
        if (!mixed) {
            H64.lv = &lv; H64.m.resize(lv.size());
            for (size_t l = 0; l < lv.size(); ++l) load_level(lv[l], H64.m[l]);
            coarse_factor(lv.back(), H64.coarse, singular);
            H64.singular = singular; H64.P = P;
        } else {
            H32.lv = &lv; H32.m.resize(lv.size());
            for (size_t l = 0; l < lv.size(); ++l) load_level(lv[l], H32.m[l]);
            coarse_factor(lv.back(), H32.coarse, singular);
            H32.singular = singular; H32.P = P;
        }
        rounds = 1;
        auto precond = [&]() {
            if (!mixed) {
                LevelT<double> &M = H64.m[0];
                for (size_t c = 0; c < L0.tot; ++c) M.b[c] = r[c];
                vcycle(H64, 0);
                for (size_t c = 0; c < L0.tot; ++c) z[c] = L0.active[c] ? M.x[c] : 0.0;
            } else {
                LevelT<float> &M = H32.m[0];
                for (size_t c = 0; c < L0.tot; ++c) M.b[c] = (float)r[c];
                vcycle(H32, 0);
                for (size_t c = 0; c < L0.tot; ++c) z[c] = L0.active[c] ? (double)M.x[c] : 0.0;
            }
        };
        precond();
        p = z;
        double rz = dot_active(L0, r, z);
        while (its < prm->max_iter) {
            its++;
            double *pp = p.data();
            FOR_CELLS(L0) {
                size_t c = pidx(L0, i, j, k);
                q[c] = L0.active[c] ? apply_at(L0, M0, pp, c) : 0.0;
            }
            double alpha = rz / dot_active(L0, p, q);
            for (size_t c = 0; c < L0.tot; ++c) {
                x[c] += alpha * p[c];
                r[c] -= alpha * q[c];
            }
            if (singular) project_mean(L0, r);
            double rn = std::sqrt(dot_active(L0, r, r));
            relres = rn / bn;
            if (relres <= prm->rel_tol) break;
            precond();
            double rz2 = dot_active(L0, r, z);
            double beta = rz2 / rz;
            rz = rz2;
            for (size_t c = 0; c < L0.tot; ++c) p[c] = z[c] + beta * p[c];
        }
    }
done:
    if (singular) project_mean(L0, x);
    {
        double rn = residual64();
        relres = bn > 0 ? rn / bn : 0.0;
    }
    for (int k = 1; k <= K; ++k)
        for (int j = 1; j <= J; ++j)
            for (int i = 1; i <= I; ++i) {
                size_t n = (size_t)(i - 1) + (size_t)I * ((size_t)(j - 1) + (size_t)J * (k - 1));
                if (in->pcell_posnu[n] >= 0) x_posnu[in->pcell_posnu[n]] = x[pidx(L0, i, j, k)];
            }
    prm->iterations = its;
    prm->rounds = rounds;
    prm->rel_residual = relres;
    return relres <= prm->rel_tol ? 0 : 2;
}

// One V-cycle of the hierarchy built from (in, pocoef): z = M r.  r and z
// are ghosted FP64 arrays ((I+2)(J+2)(K+2), the level-0 padded layout); r is
// read on the active cells only, z is 0 elsewhere.  prm->precision selects
// the FP64 (0) or FP32 (1) V-cycle; prm->degree, ratio and coarse_max as in
// oracle_gmg_solve.  This is the reference of the device V-cycle's parity
// test.
int oracle_gmg_vcycle(int I, int J, int K, const scf_poisson_in *in, const double *pocoef, const double *r,
                      double *z, oracle_gmg_params *prm)
{
    std::vector<Level> lv(1);
    std::vector<double> b;
    std::vector<double> zero_rhs((size_t)in->pcell_extcell + 1, 0.0);
    build_level0(I, J, K, in, pocoef, zero_rhs.data(), lv[0], b);
    bool singular = true;
    for (int q = 0; q < 6; ++q)
        if (in->bcp_flag[q] == 0) singular = false;
    while ((size_t)lv.back().n[0] * lv.back().n[1] * lv.back().n[2] > (size_t)prm->coarse_max &&
           (lv.back().n[0] > 2 || lv.back().n[1] > 2 || lv.back().n[2] > 2)) {
        lv.emplace_back();
        coarsen(lv[lv.size() - 2], lv.back());
    }
    prm->levels = (int)lv.size();
    Params P;
    P.degree = prm->degree;
    P.line_seg = prm->line_seg;
    P.ratio = prm->ratio;
    const Level &L0 = lv[0];
    auto run = [&](auto &H) {
        H.lv = &lv;
        H.m.resize(lv.size());
        for (size_t l = 0; l < lv.size(); ++l) load_level(lv[l], H.m[l]);
        coarse_factor(lv.back(), H.coarse, singular);
        H.singular = singular;
        H.P = P;
        auto &M = H.m[0];
        using TT = typename std::remove_reference<decltype(M.x[0])>::type;
        for (size_t c = 0; c < L0.tot; ++c) M.b[c] = L0.active[c] ? (TT)r[c] : TT(0);
        vcycle(H, 0);
        for (size_t c = 0; c < L0.tot; ++c) z[c] = L0.active[c] ? (double)M.x[c] : 0.0;
    };
    if (prm->precision == 0) {
        Hier<double> H;
        run(H);
    } else {
        Hier<float> H;
        run(H);
    }
    return 0;
}

}  // extern "C"
