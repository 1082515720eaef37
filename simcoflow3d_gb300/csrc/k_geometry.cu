// k_geometry.cu -- cut-cell geometry preprocessing on the GPU: DefineCell,
// CellGeoCal, GridPreprocess, DefineMomentumExchangeCell and
// NumberExternalCell (src/CutCell.f90).
//
// Compiled with -fmad=false: every product and sum rounds on its own, in the
// reference's order, so the results are bit-identical to the Fortran
// expressions.  FP64 issues at 2 lanes per clock per SM on this GPU, so the
// face polygon of FaceGeoCal is only evaluated for faces the solid surface
// actually cuts: an exponent test on the integer pipe proves that all four
// corners of a face lie on one side (open or closed), and an open face's
// result depends only on its two edge lengths (a per-thread memo).
#include "geo_kernels.h"

namespace {

__device__ __forceinline__ unsigned long long bits(double x) { return (unsigned long long)__double_as_longlong(x); }
// -x (IEEE negation: the sign bit), on the 32-bit halves so that the
// compiler does not turn it back into an FP64 instruction
__device__ __forceinline__ double neg(double x)
{
    return __hiloint2double(__double2hiint(x) ^ (int)0x80000000, __double2loint(x));
}
constexpr unsigned long long ONE = 0x3ff0000000000000ull;
constexpr double EPSI = 1.0e-3;    // CutCell.f90:11
constexpr double TOL = 1.0e-20;    // CutCell.f90:396

struct Face {
    double a, c1, c2;   // open fraction and centroid; the third component is d3
};

// FaceGeoCal (CutCell.f90:883-981), evaluated in full.
__device__ __noinline__ Face face_exact(double d1, double d2, double n1, double n2, double n3, double d3, double phi)
{
    const double d11 = d1 / 2.0, d22 = d2 / 2.0;
    double x[7], y[7];
    int m = 0;
    const double p1 = d11 * n1 - d22 * n2 + d3 * n3 + phi;
    const double p2 = -(d11 * n1) - d22 * n2 + d3 * n3 + phi;
    const double p3 = -(d11 * n1) + d22 * n2 + d3 * n3 + phi;
    const double p4 = d11 * n1 + d22 * n2 + d3 * n3 + phi;
#pragma unroll
    for (int q = 0; q < 7; ++q) { x[q] = 0.0; y[q] = 0.0; }
    // a line clips a rectangle to five vertices at most; six only if the
    // rounded corner values alternate in sign, which the arrays still hold
    if (p1 > 0.0) { x[m] = d11; y[m] = -d22; ++m; }
    if (p1 * p2 < 0.0) { x[m] = (d22 * n2 - d3 * n3 - phi) / n1; y[m] = -d22; ++m; }
    if (p2 > 0.0) { x[m] = -d11; y[m] = -d22; ++m; }
    if (p2 * p3 < 0.0) { x[m] = -d11; y[m] = (d11 * n1 - d3 * n3 - phi) / n2; ++m; }
    if (p3 > 0.0) { x[m] = -d11; y[m] = d22; ++m; }
    if (p3 * p4 < 0.0) { x[m] = (-(d22 * n2) - d3 * n3 - phi) / n1; y[m] = d22; ++m; }
    if (p4 > 0.0) { x[m] = d11; y[m] = d22; ++m; }
    if (p4 * p1 < 0.0) { x[m] = d11; y[m] = (-(d11 * n1) - d3 * n3 - phi) / n2; ++m; }
    x[m] = x[0];
    y[m] = y[0];
    double vol = 0.0;
    for (int q = 0; q < m; ++q) vol = vol + 0.5 * (x[q] * y[q + 1] - x[q + 1] * y[q]);
    Face f;
    f.a = fabs(vol / (d1 * d2));
    f.c1 = 0.0;
    f.c2 = 0.0;
    if (f.a > 0.0) {
        const double s = 1.0 / 6.0 / vol;
        for (int q = 0; q < m; ++q) {
            const double cr = x[q] * y[q + 1] - x[q + 1] * y[q];
            f.c1 = f.c1 + s * (x[q] + x[q + 1]) * cr;
            f.c2 = f.c2 + s * (y[q] + y[q + 1]) * cr;
        }
    }
    return f;
}

// x / 2 for normal x with a biased exponent above 1 (the exponent field
// minus one); other values take the FP64 division.  Both are exact.
__device__ __noinline__ double half_slow(double x) { return x / 2.0; }
__device__ __forceinline__ double half(double x)
{
    const unsigned long long b = bits(x), e = (b >> 52) & 0x7ff;
    return (e > 1 && e < 0x7ff) ? __longlong_as_double((long long)(b - (1ull << 52))) : half_slow(x);
}

// |x| truncated to FP32 on the integer pipe (|x|(1 - 2^-23) < result <= |x|);
// ok is cleared for values outside FP32's normal range (zero is exact).
// (Works on the 32-bit halves: a 64-bit mask of the sign bit is recognised
// as fabs and issued on the FP64 pipe.)
__device__ __forceinline__ float abs_f32_trunc(double x, bool &ok)
{
    const unsigned hi = (unsigned)__double2hiint(x) & 0x7fffffffu, lo = (unsigned)__double2loint(x);
    if ((hi | lo) == 0u) return 0.0f;
    const int e = (int)(hi >> 20) - 1023 + 127;
    if (e < 1 || e > 254) { ok = false; return 0.0f; }
    return __uint_as_float(((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
}

// 1: every corner of the face is open (n.x + phi > 0), -1: every corner is
// closed, 0: undecided (evaluate in full).  The four corner values are
// phi +- d11 n1 +- d22 n2 + d3 n3, so |phi| > |d11 n1| + |d22 n2| + |d3 n3|
// gives all of them phi's sign.  The test runs in FP32 on truncated
// magnitudes with a relative margin of 1e-4, far above the truncation
// (2^-23 per value), the FP32 rounding and the FP64 rounding of the four
// sums; anything outside FP32's range is undecided.
__device__ __forceinline__ int face_class(double d1, double d2, double n1, double n2, double n3, double d3,
                                          double phi)
{
    bool ok = true;
    const float a1 = abs_f32_trunc(d1, ok) * 0.5f * abs_f32_trunc(n1, ok);
    const float a2 = abs_f32_trunc(d2, ok) * 0.5f * abs_f32_trunc(n2, ok);
    const float a3 = abs_f32_trunc(d3, ok) * abs_f32_trunc(n3, ok);
    const float p = abs_f32_trunc(phi, ok);
    if (!ok || !(p > (a1 + a2 + a3) * 1.0001f) || !(p > 1.0e-30f)) return 0;
    return __double2hiint(phi) < 0 ? -1 : 1;
}

// An open face: its result depends on d1, d2 only (the corners of the
// rectangle); d3 passes through as the third centroid component.
struct FullMemo {
    unsigned long long d1, d2;
    Face f;
};

__device__ __noinline__ Face face_full(double d1, double d2) { return face_exact(d1, d2, 0.0, 0.0, 0.0, 0.0, 1.0); }

__device__ __forceinline__ Face face_eval(FullMemo &mm, double d1, double d2, double n1, double n2, double n3,
                                          double d3, double phi, int &exact)
{
    const int c = face_class(d1, d2, n1, n2, n3, d3, phi);
    if (c > 0) {
        if (bits(d1) != mm.d1 || bits(d2) != mm.d2) {
            mm.d1 = bits(d1); mm.d2 = bits(d2);
            mm.f = face_full(d1, d2);
        }
        return mm.f;
    }
    if (c < 0) {
        Face f;
        f.a = 0.0; f.c1 = 0.0; f.c2 = 0.0;
        return f;
    }
    ++exact;
    return face_exact(d1, d2, n1, n2, n3, d3, phi);
}

// Shared face of CellGeoCal (CutCell.f90:474-531): the area average of the
// two sides' open fractions w (this cell) and e (the neighbour), and the
// area-weighted centroid components (xa, ya) and (xb, yb).
struct Shared {
    double avg, fa, fb;
};
// The FP64 work of share() is out of line: inline, the compiler evaluates
// short branches unconditionally and selects, which put the products and
// divisions on every face.
__device__ __noinline__ Shared share_slow(double w, double e, double xa, double ya, double xb, double yb)
{
    Shared s;
    const double na = xa * w + ya * e, nb = xb * w + yb * e;
    const double den = w + e + TOL;
    s.avg = (w * w + e * e) / den;
    s.fa = na / den;
    s.fb = nb / den;
    return s;
}
// both sides open: den = 1 + 1 + 1e-20 = 2, avg = 2/2 = 1 and x*1 = x
__device__ __noinline__ Shared share_open(double xa, double ya, double xb, double yb)
{
    Shared s;
    s.avg = 1.0;
    s.fa = (xa + ya) / 2.0;
    s.fb = (xb + yb) / 2.0;
    return s;
}
__device__ __forceinline__ Shared share(double w, double e, double xa, double ya, double xb, double yb)
{
    Shared s;
    const bool zc = (bits(xa) | bits(ya) | bits(xb) | bits(yb)) == 0ull;   // all four centroid components +0
    if (zc && ((bits(w) == ONE && bits(e) == ONE) || (bits(w) | bits(e)) == 0ull)) {
        // both sides open: (1 + 1)/(1 + 1 + 1e-20) = 1 and (+0 + +0)/2 = +0;
        // both closed: (0 + 0)/1e-20 = +0 and (+0*0 + +0*0)/1e-20 = +0
        s.avg = bits(w) == ONE ? 1.0 : 0.0;
        s.fa = 0.0;
        s.fb = 0.0;
        return s;
    }
    if (bits(w) == ONE && bits(e) == ONE) return share_open(xa, ya, xb, yb);
    return share_slow(w, e, xa, ya, xb, yb);
}

// sqrt(a^2 + b^2 + c^2) of CutCell.f90:455-462
__device__ __noinline__ double wllh_slow(double ee, double we, double ne, double se, double te, double be, double dx,
                                         double dy, double dz)
{
    const double a = (ee - we) * dy * dz, b = (ne - se) * dx * dz, c = (te - be) * dx * dy;
    return sqrt(a * a + b * b + c * c);
}

__device__ __noinline__ double div_slow(double a, double b) { return a / b; }

// ---------------------------------------------------------------------------
// DefineCell (CutCell.f90:329-365) on the interior; on the ghost shell the
// face apertures take CellGeoCal's initial 1 (CutCell.f90:398-400).
__global__ void __launch_bounds__(256) k_geo_define(GeoFam t, Dims d)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < d.ng; g += gridDim.x * blockDim.x) {
        const int i = g % d.gx, j = (g / d.gx) % d.gy, k = g / (d.gx * d.gy);
        if (i == 0 || j == 0 || k == 0 || i == d.I + 1 || j == d.J + 1 || k == d.K + 1) {
            t.ee[g] = 1.0; t.ne[g] = 1.0; t.te[g] = 1.0;
            continue;
        }
        const int n = nidx(d, i, j, k);
        double vof = t.vof[g], vofl = t.vofl[g];
        int ct = t.ct[n];
        if (vof >= 1.0 - EPSI) {
            ct = 0;
            if (bits(vof) != ONE) vofl = div_slow(vofl, vof);   // x / 1.0 = x
            vof = 1.0;
        }
        if (vof <= EPSI) { ct = 2; vof = 0.0; vofl = 0.0; }
        if (vof >= EPSI && vof <= 1.0 - EPSI) ct = 1;
        t.vof[g] = vof; t.vofl[g] = vofl; t.ct[n] = ct;
    }
}

// Inputs of one FaceGeoCal call.
struct FaceIn {
    double d1, d2, n1, n2, n3, d3, phi;
};

// Faces whose corners are all open or all closed are resolved here; the
// rest (cut faces) are put on the block's queue (slot >= 0) for a dense
// evaluation, or evaluated in place when the queue is full (slot -1, -2
// meaning resolved).
__device__ __forceinline__ Face face_resolve(FullMemo &mm, const FaceIn &in, FaceIn *q_in, int *q_count, int cap,
                                             int &slot, int &exact)
{
    Face f;
    f.a = 0.0; f.c1 = 0.0; f.c2 = 0.0;
    slot = -2;
    const int c = face_class(in.d1, in.d2, in.n1, in.n2, in.n3, in.d3, in.phi);
    if (c > 0) {
        if (bits(in.d1) != mm.d1 || bits(in.d2) != mm.d2) {
            mm.d1 = bits(in.d1); mm.d2 = bits(in.d2);
            mm.f = face_full(in.d1, in.d2);
        }
        return mm.f;
    }
    if (c < 0) return f;
    ++exact;
    const int q = atomicAdd(q_count, 1);
    if (q < cap) {
        q_in[q] = in;
        slot = q;
        return f;
    }
    return face_exact(in.d1, in.d2, in.n1, in.n2, in.n3, in.d3, in.phi);
}

// CellGeoCal's face loop and shared-face averaging (CutCell.f90:402-531).
// A block is 32 x 4 columns; each thread marches a GEO_KSEG-cell segment of
// its (i,j) column.  For cell (i,j,k) it needs its six faces (WlLh takes
// them all) and finishes the three faces it shares with its lower
// neighbours: the W face with the E face of (i-1,j,k), the S face with the N
// face of (i,j-1,k) (both evaluated here again) and the B face with the T
// face of (i,j,k-1) (carried from the previous cell of the march).  Faces on
// the upper boundary keep their own value.  Every aperture and face centre
// is written by exactly one thread.
//
// Faces the solid surface cuts are rare and scattered: evaluated where they
// occur, a warp would run the whole polygon (four FP64 divisions) for one
// lane.  Each k step therefore queues them in shared memory, the block
// evaluates the queue with one face per thread, and the threads pick their
// results up.  The queue is double-buffered by k parity and reset by thread
// 0 after its evaluation; a k step in which no thread queued anything takes
// one barrier only.
constexpr int GEO_QCAP = 256;

__global__ void __launch_bounds__(128) k_geo_faces(GeoFam t, Dims d, int *exact_count)
{
    __shared__ FaceIn q_in[2][GEO_QCAP];
    __shared__ Face q_out[2][GEO_QCAP];
    __shared__ int q_count[2];
    const int tid = threadIdx.x + 32 * threadIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const bool live = i <= d.I && j <= d.J;
    const int kbeg = blockIdx.z * GEO_KSEG + 1, kend = min(kbeg + GEO_KSEG - 1, d.K);
    const long long NG = d.ng, NN = d.n;
    if (tid < 2) q_count[tid] = 0;
    __syncthreads();
    // an open face's result depends on its edges (d1, d2) only, so the faces
    // of one orientation share a memo: T/B (dx, dy), E/W (dy, dz), N/S (dz, dx)
    FullMemo mXY, mYZ, mZX;
    mXY.d1 = mXY.d2 = ~0ull; mXY.f.a = mXY.f.c1 = mXY.f.c2 = 0.0;
    mYZ = mXY;
    mZX = mXY;
    int exact = 0;
    Face prevT;
    double prevhz = 0.0;
    prevT.a = prevT.c1 = prevT.c2 = 0.0;
    for (int k = kbeg; k <= kend; ++k) {
        const int b = (k - kbeg) & 1;
        // faces 0..5: T, B, E, W, N, S of this cell; 6: E of (i-1,j,k);
        // 7: N of (i,j-1,k); 8: T of (i,j,k-1) at the segment start
        Face F[9];
        int slot[9];
        double hx = 0.0, hy = 0.0, hz = 0.0, hxw = 0.0, hys = 0.0, hzb = prevhz;
        int g = 0, n = 0;
        double dx = 0.0, dy = 0.0, dz = 0.0;
#pragma unroll
        for (int f = 0; f < 9; ++f) { slot[f] = -2; F[f].a = F[f].c1 = F[f].c2 = 0.0; }
        int queued = 0;
        if (live) {
            g = gidx(d, i, j, k); n = nidx(d, i, j, k);
            dx = t.dx[n]; dy = t.dy[n]; dz = t.dz[n];
            const double nx = t.nx[g], ny = t.ny[g], nz = t.nz[g], phi = t.phi[g];
            hx = half(dx); hy = half(dy); hz = half(dz);
            FaceIn in;
            in.n1 = nx; in.n2 = ny; in.n3 = nz; in.phi = phi; in.d1 = dx; in.d2 = dy;
            in.d3 = hz;      F[0] = face_resolve(mXY, in, q_in[b], &q_count[b], GEO_QCAP, slot[0], exact);
            in.d3 = neg(hz); F[1] = face_resolve(mXY, in, q_in[b], &q_count[b], GEO_QCAP, slot[1], exact);
            in.n1 = ny; in.n2 = nz; in.n3 = nx; in.d1 = dy; in.d2 = dz;
            in.d3 = hx;      F[2] = face_resolve(mYZ, in, q_in[b], &q_count[b], GEO_QCAP, slot[2], exact);
            in.d3 = neg(hx); F[3] = face_resolve(mYZ, in, q_in[b], &q_count[b], GEO_QCAP, slot[3], exact);
            in.n1 = nz; in.n2 = nx; in.n3 = ny; in.d1 = dz; in.d2 = dx;
            in.d3 = hy;      F[4] = face_resolve(mZX, in, q_in[b], &q_count[b], GEO_QCAP, slot[4], exact);
            in.d3 = neg(hy); F[5] = face_resolve(mZX, in, q_in[b], &q_count[b], GEO_QCAP, slot[5], exact);
            if (i > 1) {
                const int gw = g - 1, nw = n - 1;
                hxw = half(t.dx[nw]);
                in.d1 = t.dy[nw]; in.d2 = t.dz[nw]; in.n1 = t.ny[gw]; in.n2 = t.nz[gw]; in.n3 = t.nx[gw];
                in.d3 = hxw; in.phi = t.phi[gw];
                F[6] = face_resolve(mYZ, in, q_in[b], &q_count[b], GEO_QCAP, slot[6], exact);
            }
            if (j > 1) {
                const int gs = g - d.gx, ns = n - d.I;
                hys = half(t.dy[ns]);
                in.d1 = t.dz[ns]; in.d2 = t.dx[ns]; in.n1 = t.nz[gs]; in.n2 = t.nx[gs]; in.n3 = t.ny[gs];
                in.d3 = hys; in.phi = t.phi[gs];
                F[7] = face_resolve(mZX, in, q_in[b], &q_count[b], GEO_QCAP, slot[7], exact);
            }
            if (k > 1 && k == kbeg) {
                const int gb = g - d.gx * d.gy, nb = n - d.I * d.J;
                hzb = half(t.dz[nb]);
                in.d1 = t.dx[nb]; in.d2 = t.dy[nb]; in.n1 = t.nx[gb]; in.n2 = t.ny[gb]; in.n3 = t.nz[gb];
                in.d3 = hzb; in.phi = t.phi[gb];
                F[8] = face_resolve(mXY, in, q_in[b], &q_count[b], GEO_QCAP, slot[8], exact);
            }
#pragma unroll
            for (int f = 0; f < 9; ++f) queued |= slot[f] >= 0;
        }
        if (__syncthreads_count(queued)) {
            const int nq = min(q_count[b], GEO_QCAP);
            for (int q = tid; q < nq; q += 128) {
                const FaceIn &in = q_in[b][q];
                q_out[b][q] = face_exact(in.d1, in.d2, in.n1, in.n2, in.n3, in.d3, in.phi);
            }
            __syncthreads();
            if (tid == 0) q_count[b] = 0;
#pragma unroll
            for (int f = 0; f < 9; ++f)
                if (slot[f] >= 0) F[f] = q_out[b][slot[f]];
        }
        if (!live) continue;
        if (!(k > 1 && k == kbeg)) F[8] = prevT;
        const Face &T = F[0], &B = F[1], &E = F[2], &Wf = F[3], &N = F[4], &S = F[5];
        t.cent[n] = 0.0; t.cent[n + NN] = 0.0; t.cent[n + 2 * NN] = 0.0;
        const bool fin = ((bits(E.a) >> 52) & 0x7ff) != 0x7ff && ((bits(N.a) >> 52) & 0x7ff) != 0x7ff &&
                         ((bits(T.a) >> 52) & 0x7ff) != 0x7ff;
        if (fin && bits(E.a) == bits(Wf.a) && bits(N.a) == bits(S.a) && bits(T.a) == bits(B.a))
            t.wllh[n] = 0.0;   // (x - x) = +0 in every term, sqrt(+0) = +0
        else
            t.wllh[n] = wllh_slow(E.a, Wf.a, N.a, S.a, T.a, B.a, dx, dy, dz);
        // W face (i-1 | i): CeW = (-dx/2, W.c1, W.c2), CeE(i-1) = (dx'/2, E'.c1, E'.c2)
        if (i > 1) {
            const int gw = g - 1;
            const Shared sh = share(Wf.a, F[6].a, Wf.c1, F[6].c1, Wf.c2, F[6].c2);
            t.fce[gw + NG] = sh.fa;
            t.fce[gw + 2 * NG] = sh.fb;
            t.fce[gw] = hxw;
            t.ee[gw] = sh.avg;
        }
        if (i == d.I) t.ee[g] = E.a;
        // S face (j-1 | j): CeS = (S.c2, -dy/2, S.c1), CeN(j-1) = (N'.c2, dy'/2, N'.c1)
        if (j > 1) {
            const int gs = g - d.gx;
            const Shared sh = share(S.a, F[7].a, S.c2, F[7].c2, S.c1, F[7].c1);
            t.fcn[gs] = sh.fa;
            t.fcn[gs + 2 * NG] = sh.fb;
            t.fcn[gs + NG] = hys;
            t.ne[gs] = sh.avg;
        }
        if (j == d.J) t.ne[g] = N.a;
        // B face (k-1 | k): CeB = (B.c1, B.c2, -dz/2), CeT(k-1) = (T'.c1, T'.c2, dz'/2);
        // the second component weights CeB(...,1), as the reference does
        if (k > 1) {
            const int gb = g - d.gx * d.gy;
            const Shared sh = share(B.a, F[8].a, B.c1, F[8].c1, B.c1, F[8].c2);
            t.fct[gb] = sh.fa;
            t.fct[gb + NG] = sh.fb;
            t.fct[gb + 2 * NG] = hzb;
            t.te[gb] = sh.avg;
        }
        if (k == d.K) t.te[g] = T.a;
        prevT = T;
        prevhz = hz;
    }
    if (exact) atomicAdd(exact_count, exact);
}

// Cells whose six apertures are all below 1e-2 become solid where MoExCell
// is not allocated (CutCell.f90:533-546).
__global__ void __launch_bounds__(256) k_geo_maxface(GeoFam t, Dims d)
{
    INTERIOR_LOOP(d) {
        if (i < 2 || j < 2 || k < 2) continue;
        const int g = gidx(d, i, j, k);
        const double m = fmax(fmax(fmax(t.ee[g - 1], t.ee[g]), fmax(t.ne[g - d.gx], t.ne[g])),
                              fmax(t.te[g - d.gx * d.gy], t.te[g]));
        if (m < 1.0e-2) t.ct[nidx(d, i, j, k)] = 2;
    }
}

// Faces of solid cells are closed (CutCell.f90:548-578), as a gather over
// faces: aperture (i|i+1) is 0 if either side is an interior solid cell.
// The cut-cell rule of the reference is implied by this one.
__global__ void __launch_bounds__(256) k_geo_close(GeoFam t, Dims d)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < d.ng; g += gridDim.x * blockDim.x) {
        const int i = g % d.gx, j = (g / d.gx) % d.gy, k = g / (d.gx * d.gy);
        if (i > d.I || j > d.J || k > d.K) continue;
        const bool in_j = j >= 1, in_k = k >= 1, in_i = i >= 1;
        auto solid = [&](int a, int b, int c) {
            return a >= 1 && a <= d.I && b >= 1 && b <= d.J && c >= 1 && c <= d.K && t.ct[nidx(d, a, b, c)] == 2;
        };
        if (in_j && in_k && (solid(i, j, k) || solid(i + 1, j, k))) t.ee[g] = 0.0;
        if (in_i && in_k && (solid(i, j, k) || solid(i, j + 1, k))) t.ne[g] = 0.0;
        if (in_i && in_j && (solid(i, j, k) || solid(i, j, k + 1))) t.te[g] = 0.0;
    }
}

// One step of the boundary-plane copies of the face centres
// (CutCell.f90:580-632).  The reference's statements per array are
//   FCE: (0,:,:) <- (1,:,:); (I,:,:) <- (I-1,:,:); (:,0,:) <- (:,1,:); (:,:,0) <- (:,:,1)
//   FCN: (0,:,:) <- (1,:,:); (:,0,:) <- (:,1,:); (:,J,:) <- (:,J-1,:); (:,:,0) <- (:,:,1)
//   FCT: (0,:,:) <- (1,:,:); (:,0,:) <- (:,1,:); (:,:,0) <- (:,:,1); (:,:,K) <- (:,:,K-1)
// step s applies statement s of all three arrays (they are independent).
__device__ __forceinline__ void plane_copy(double *a, const Dims &d, long long NG, int axis, int dst, int src,
                                           int p)
{
    // p enumerates the (extent1 x extent2 x 3) entries of the plane
    int e1, e2;
    if (axis == 0) { e1 = d.gy; e2 = d.gz; } else if (axis == 1) { e1 = d.gx; e2 = d.gz; } else { e1 = d.gx; e2 = d.gy; }
    if (p >= e1 * e2 * 3) return;
    const int c = p / (e1 * e2), r = p % (e1 * e2), u = r % e1, v = r / e1;
    int gd, gs;
    if (axis == 0) { gd = gidx(d, dst, u, v); gs = gidx(d, src, u, v); }
    else if (axis == 1) { gd = gidx(d, u, dst, v); gs = gidx(d, u, src, v); }
    else { gd = gidx(d, u, v, dst); gs = gidx(d, u, v, src); }
    a[gd + c * NG] = a[gs + c * NG];
}

__global__ void __launch_bounds__(256) k_geo_fc_planes(GeoFam t, Dims d, int step)
{
    const long long NG = d.ng;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    switch (step) {
    case 0:
        plane_copy(t.fce, d, NG, 0, 0, 1, p); plane_copy(t.fcn, d, NG, 0, 0, 1, p); plane_copy(t.fct, d, NG, 0, 0, 1, p);
        break;
    case 1:
        plane_copy(t.fce, d, NG, 0, d.I, d.I - 1, p); plane_copy(t.fcn, d, NG, 1, 0, 1, p);
        plane_copy(t.fct, d, NG, 1, 0, 1, p);
        break;
    case 2:
        plane_copy(t.fce, d, NG, 1, 0, 1, p); plane_copy(t.fcn, d, NG, 1, d.J, d.J - 1, p);
        plane_copy(t.fct, d, NG, 2, 0, 1, p);
        break;
    default:
        plane_copy(t.fce, d, NG, 2, 0, 1, p); plane_copy(t.fcn, d, NG, 2, 0, 1, p);
        plane_copy(t.fct, d, NG, 2, d.K, d.K - 1, p);
        break;
    }
}

// Full cells with a closed face (CutCell.f90:634-661).
__global__ void __launch_bounds__(256) k_geo_wallcells(GeoFam t, Dims d)
{
    INTERIOR_LOOP(d) {
        if (i < 2 || j < 2 || k < 2) continue;
        const int g = gidx(d, i, j, k), n = nidx(d, i, j, k);
        const double vof = t.vof[g];
        if (bits(vof) != ONE && !(fabs(vof - 1.0) < EPSI)) continue;
        const bool ew = bits(t.ee[g - 1] ) << 1 == 0 || bits(t.ee[g]) << 1 == 0;
        const bool ns = bits(t.ne[g - d.gx]) << 1 == 0 || bits(t.ne[g]) << 1 == 0;
        const bool tb = bits(t.te[g - d.gx * d.gy]) << 1 == 0 || bits(t.te[g]) << 1 == 0;
        if (!(ew || ns || tb)) continue;
        const double dx = t.dx[n], dy = t.dy[n], dz = t.dz[n];
        if (ew) { t.wllh[n] = dy * dz; t.delh[n] = dx / 2.0; }
        if (ns) { t.wllh[n] = dx * dz; t.delh[n] = dy / 2.0; }
        if (tb) { t.wllh[n] = dx * dy; t.delh[n] = dz / 2.0; }
    }
}

// Face centres of velocity cells on stretched grids (CutCell.f90:92-163).
__global__ void __launch_bounds__(256) k_geo_stretch(GeoFam P, GeoFam U, GeoFam V, GeoFam W, Dims d)
{
    const long long NG = d.ng;
    INTERIOR_LOOP(d) {
        const int g = gidx(d, i, j, k), n = nidx(d, i, j, k);
        if (i < d.I) {
            const int n1 = nidx(d, i + 1, j, k);
            if (U.ct[n] != 1 && U.ct[n1] != 1 && bits(U.dx[n]) != bits(U.dx[n1]) &&
                fabs(U.dx[n] - U.dx[n1]) > 1.0e-10) {
                U.fce[g] = 0.5 * P.dx[n1]; U.fcn[g] = 0.0; U.fct[g] = 0.0;
            }
        } else {
            U.fcn[g] = 0.0; U.fct[g] = 0.0;
        }
        if (j < d.J) {
            const int n1 = nidx(d, i, j + 1, k);
            if (V.ct[n] != 1 && V.ct[n1] != 1 && bits(V.dy[n]) != bits(V.dy[n1]) &&
                fabs(V.dy[n] - V.dy[n1]) > 1.0e-10) {
                V.fcn[g + NG] = 0.5 * P.dy[n1]; V.fce[g + NG] = 0.0; V.fct[g + NG] = 0.0;
            }
        } else {
            V.fce[g + NG] = 0.0; V.fct[g + NG] = 0.0;
        }
        if (k < d.K) {
            const int n1 = nidx(d, i, j, k + 1);
            if (W.ct[n] != 1 && W.ct[n1] != 1 && bits(W.dz[n]) != bits(W.dz[n1]) &&
                fabs(W.dz[n] - W.dz[n1]) > 1.0e-10) {
                W.fct[g + 2 * NG] = 0.5 * P.dz[n1]; W.fce[g + 2 * NG] = 0.0; W.fcn[g + 2 * NG] = 0.0;
            }
        } else {
            W.fce[g + 2 * NG] = 0.0; W.fcn[g + 2 * NG] = 0.0;
        }
    }
}

// Velocity-cell apertures and face centres from the pressure cells
// (CutCell.f90:165-227).
__global__ void __launch_bounds__(256) k_geo_from_p(GeoFam P, GeoFam U, GeoFam V, GeoFam W, Dims d, int *exact_count)
{
    const long long NG = d.ng, NN = d.n;
    int exact = 0;
    INTERIOR_LOOP(d) {
        const int g = gidx(d, i, j, k), n = nidx(d, i, j, k);
        const double dx = P.dx[n], dy = P.dy[n], dz = P.dz[n];
        P.cent[n] = 0.0; P.cent[n + NN] = 0.0; P.cent[n + 2 * NN] = 0.0;
        const double vof = P.vof[g];
        const int ge = g - 1, gn = g - d.gx, gt = g - d.gx * d.gy;
        if (vof < 1.0 && vof > 0.0) {
            const double nx = P.nx[g], ny = P.ny[g], nz = P.nz[g], phi = P.phi[g];
            FullMemo mm;
            mm.d1 = mm.d2 = ~0ull; mm.f.a = mm.f.c1 = mm.f.c2 = 0.0;
            Face f = face_eval(mm, dy, dz, ny, nz, nx, 0.0, phi, exact);
            U.ee[ge] = f.a;
            U.fce[ge] = 0.0 + dx / 2.0; U.fce[ge + NG] = f.c1; U.fce[ge + 2 * NG] = f.c2;
            mm.d1 = mm.d2 = ~0ull;
            f = face_eval(mm, dz, dx, nz, nx, ny, 0.0, phi, exact);
            V.ne[gn] = f.a;
            V.fcn[gn + NG] = 0.0 + dy / 2.0; V.fcn[gn] = f.c2; V.fcn[gn + 2 * NG] = f.c1;
            mm.d1 = mm.d2 = ~0ull;
            f = face_eval(mm, dx, dy, nx, ny, nz, 0.0, phi, exact);
            W.te[gt] = f.a;
            W.fct[gt + 2 * NG] = 0.0 + dz / 2.0; W.fct[gt] = f.c1; W.fct[gt + NG] = f.c2;
        } else if (vof > 0.5) {
            U.fce[ge] = dx / 2.0; U.fce[ge + NG] = 0.0; U.fce[ge + 2 * NG] = 0.0; U.ee[ge] = 1.0;
            V.fcn[gn + NG] = dy / 2.0; V.fcn[gn] = 0.0; V.fcn[gn + 2 * NG] = 0.0; V.ne[gn] = 1.0;
            W.fct[gt + 2 * NG] = dz / 2.0; W.fct[gt] = 0.0; W.fct[gt + NG] = 0.0; W.te[gt] = 1.0;
        } else {
            U.ee[ge] = 0.0; U.fce[ge] = 0.0; U.fce[ge + NG] = 0.0; U.fce[ge + 2 * NG] = 0.0;
            V.ne[gn] = 0.0; V.fcn[gn] = 0.0; V.fcn[gn + NG] = 0.0; V.fcn[gn + 2 * NG] = 0.0;
            W.te[gt] = 0.0; W.fct[gt] = 0.0; W.fct[gt + NG] = 0.0; W.fct[gt + 2 * NG] = 0.0;
        }
    }
    if (exact) atomicAdd(exact_count, exact);
}

// Pressure-cell apertures and face centres, velocity-cell centres, from the
// velocity cells (CutCell.f90:229-323).
__global__ void __launch_bounds__(256) k_geo_from_uvw(GeoFam P, GeoFam U, GeoFam V, GeoFam W, Dims d,
                                                      int *exact_count)
{
    const long long NG = d.ng, NN = d.n;
    int exact = 0;
    INTERIOR_LOOP(d) {
        const int g = gidx(d, i, j, k), n = nidx(d, i, j, k);
        FullMemo mm;
        if (U.vof[g] < 1.0 && U.vof[g] > 0.0) {
            mm.d1 = mm.d2 = ~0ull; mm.f.a = mm.f.c1 = mm.f.c2 = 0.0;
            const Face f = face_eval(mm, U.dy[n], U.dz[n], U.ny[g], U.nz[g], U.nx[g], 0.0, U.phi[g], exact);
            P.fce[g] = 0.0 + P.dx[n] / 2.0; P.fce[g + NG] = f.c1; P.fce[g + 2 * NG] = f.c2;
            U.cent[n] = 0.0; U.cent[n + NN] = f.c1; U.cent[n + 2 * NN] = f.c2;
        } else if (U.vof[g] > 0.5) {
            P.ee[g] = 1.0;
            P.fce[g] = P.dx[n] / 2.0; P.fce[g + NG] = 0.0; P.fce[g + 2 * NG] = 0.0;
            U.cent[n] = 0.0; U.cent[n + NN] = 0.0; U.cent[n + 2 * NN] = 0.0;
        } else {
            P.ee[g] = 0.0;
            P.fce[g] = 0.0; P.fce[g + NG] = 0.0; P.fce[g + 2 * NG] = 0.0;
            U.cent[n] = 0.0; U.cent[n + NN] = 0.0; U.cent[n + 2 * NN] = 0.0;
        }
        if (V.vof[g] < 1.0 && V.vof[g] > 0.0) {
            mm.d1 = mm.d2 = ~0ull;
            const Face f = face_eval(mm, V.dz[n], V.dx[n], V.nz[g], V.nx[g], V.ny[g], 0.0, V.phi[g], exact);
            P.fcn[g] = f.c2; P.fcn[g + 2 * NG] = f.c1; P.fcn[g + NG] = 0.0 + P.dy[n] / 2.0;
            V.cent[n] = f.c2; V.cent[n + NN] = 0.0; V.cent[n + 2 * NN] = f.c1;
        } else if (V.vof[g] > 0.5) {
            P.ne[g] = 1.0;
            P.fcn[g] = 0.0; P.fcn[g + 2 * NG] = 0.0; P.fcn[g + NG] = P.dy[n] / 2.0;
            V.cent[n] = 0.0; V.cent[n + NN] = 0.0; V.cent[n + 2 * NN] = 0.0;
        } else {
            P.ne[g] = 0.0;
            P.fcn[g] = 0.0; P.fcn[g + NG] = 0.0; P.fcn[g + 2 * NG] = 0.0;
            V.cent[n] = 0.0; V.cent[n + NN] = 0.0; V.cent[n + 2 * NN] = 0.0;
        }
        if (W.vof[g] < 1.0 && W.vof[g] > 0.0) {
            mm.d1 = mm.d2 = ~0ull;
            const Face f = face_eval(mm, W.dx[n], W.dy[n], W.nx[g], W.ny[g], W.nz[g], 0.0, W.phi[g], exact);
            P.fct[g] = f.c1; P.fct[g + NG] = f.c2; P.fct[g + 2 * NG] = 0.0 + P.dz[n] / 2.0;
            W.cent[n] = f.c1; W.cent[n + NN] = f.c2; W.cent[n + 2 * NN] = 0.0;
        } else if (W.vof[g] > 0.5) {
            P.te[g] = 1.0;
            P.fct[g] = 0.0; P.fct[g + NG] = 0.0; P.fct[g + 2 * NG] = P.dz[n] / 2.0;
            W.cent[n] = 0.0; W.cent[n + NN] = 0.0; W.cent[n + 2 * NN] = 0.0;
        } else {
            P.te[g] = 0.0;
            P.fct[g] = 0.0; P.fct[g + NG] = 0.0; P.fct[g + 2 * NG] = 0.0;
            W.cent[n] = 0.0; W.cent[n + NN] = 0.0; W.cent[n + 2 * NN] = 0.0;
        }
    }
    if (exact) atomicAdd(exact_count, exact);
}

// DefineMomentumExchangeCell (CutCell.f90:673-749)
__global__ void __launch_bounds__(256) k_geo_moex(GeoFam P, GeoFam U, GeoFam V, GeoFam W, Dims d)
{
    INTERIOR_LOOP(d) {
        const int n = nidx(d, i, j, k);
        const bool ps = P.ct[n] == 2;
        if (U.ct[n] == 1 && (ps || (i < d.I && P.ct[nidx(d, i + 1, j, k)] == 2))) U.moex[n] = 1;
        if (V.ct[n] == 1 && (ps || (j < d.J && P.ct[nidx(d, i, j + 1, k)] == 2))) V.moex[n] = 1;
        if (W.ct[n] == 1 && (ps || (k < d.K && P.ct[nidx(d, i, j, k + 1)] == 2))) W.moex[n] = 1;
    }
}

// NumberExternalCell (CutCell.f90:753-786).  The numbering runs over
// (i, j, k) with k fastest; an (i,j) column is a contiguous run of it.
// Pass 1: active cells per column; pass 2 (one block): exclusive prefix over
// the columns in (i, j) order; pass 3: each column numbers its cells.
__global__ void __launch_bounds__(256) k_posnu_count(GeoFam t, Dims d, int *colcount)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int ni = d.I - t.iu, nj = d.J - t.iv, nk = d.K - t.iw;
    if (i > ni || j > nj) return;
    int c = 0;
    for (int k = 1; k <= nk; ++k) c += t.ct[nidx(d, i, j, k)] != 2;
    colcount[(i - 1) * nj + (j - 1)] = c;
}

__global__ void __launch_bounds__(1024) k_posnu_scan(int *colcount, int ncol, int *total)
{
    __shared__ int part[1024];
    const int t = threadIdx.x;
    const int per = (ncol + 1023) / 1024;
    const int a = min(ncol, t * per), b = min(ncol, a + per);
    int s = 0;
    for (int q = a; q < b; ++q) s += colcount[q];
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {   // inclusive Hillis-Steele scan
        const int v = t >= off ? part[t - off] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = t > 0 ? part[t - 1] : 0;
    for (int q = a; q < b; ++q) {
        const int c = colcount[q];
        colcount[q] = run;
        run += c;
    }
    if (t == 1023) *total = part[1023];
}

__global__ void __launch_bounds__(256) k_posnu_write(GeoFam t, Dims d, const int *colstart)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int ni = d.I - t.iu, nj = d.J - t.iv, nk = d.K - t.iw;
    if (i > ni || j > nj) return;
    int p = colstart[(i - 1) * nj + (j - 1)];
    for (int k = 1; k <= nk; ++k) {
        const long long q = (long long)(i - 1) + (long long)ni * ((j - 1) + (long long)nj * (k - 1));
        t.posnu[q] = t.ct[nidx(d, i, j, k)] != 2 ? p++ : -1;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// host launchers
static int grid_for(int n, int per_block) { return std::min((n + per_block - 1) / per_block, 152 * 16); }

void launch_cell_geo(const GeoFam &t, const Dims &d, int *exact_count, cudaStream_t st, int *launches,
                     cudaEvent_t *ev)
{
    k_geo_define<<<grid_for(d.ng, 256), 256, 0, st>>>(t, d);
    dim3 b(32, 4), g((d.I + 31) / 32, (d.J + 3) / 4, (d.K + GEO_KSEG - 1) / GEO_KSEG);
    if (ev) cudaEventRecord(ev[0], st);
    k_geo_faces<<<g, b, 0, st>>>(t, d, exact_count);
    if (ev) cudaEventRecord(ev[1], st);
    *launches += 2;
    if (!t.moex) {
        k_geo_maxface<<<grid_for(d.n, 256), 256, 0, st>>>(t, d);
        *launches += 1;
    }
    k_geo_close<<<grid_for(d.ng, 256), 256, 0, st>>>(t, d);
    *launches += 1;
    const int plane = std::max(d.gy * d.gz, std::max(d.gx * d.gz, d.gx * d.gy)) * 3;
    for (int s = 0; s < 4; ++s) k_geo_fc_planes<<<(plane + 255) / 256, 256, 0, st>>>(t, d, s);
    k_geo_wallcells<<<grid_for(d.n, 256), 256, 0, st>>>(t, d);
    *launches += 5;
}

void launch_grid_preprocess_tail(const GeoFam &P, const GeoFam &U, const GeoFam &V, const GeoFam &W, const Dims &d,
                                 int *exact_count, cudaStream_t st, int *launches)
{
    k_geo_stretch<<<grid_for(d.n, 256), 256, 0, st>>>(P, U, V, W, d);
    k_geo_from_p<<<grid_for(d.n, 256), 256, 0, st>>>(P, U, V, W, d, exact_count);
    k_geo_from_uvw<<<grid_for(d.n, 256), 256, 0, st>>>(P, U, V, W, d, exact_count);
    k_geo_moex<<<grid_for(d.n, 256), 256, 0, st>>>(P, U, V, W, d);
    *launches += 4;
}

void launch_posnu(const GeoFam &t, const Dims &d, int *colbuf, int *total, cudaStream_t st, int *launches)
{
    const int ni = d.I - t.iu, nj = d.J - t.iv;
    dim3 b(64, 4), g((ni + 63) / 64, (nj + 3) / 4);
    k_posnu_count<<<g, b, 0, st>>>(t, d, colbuf);
    k_posnu_scan<<<1, 1024, 0, st>>>(colbuf, ni * nj, total);
    k_posnu_write<<<g, b, 0, st>>>(t, d, colbuf);
    *launches += 3;
}
