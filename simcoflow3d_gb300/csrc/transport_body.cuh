// transport_body.cuh -- the per-cell work of the CLSVOF interface transport
// (src/Clsvof.f90: Clsvof_Scheme 355-798 and the routines it calls), written
// once for the device kernels of k_transport.cu and, compiled by a host C++
// compiler, for the tests that run the same bodies on the CPU.
//
// Layout (column-major, i fastest): "ghosted" (0:I+1,0:J+1,0:K+1), "interior"
// (1:I,1:J,1:K), wall planes (J,K) for x, (I,K) for y, (I,J) for z.  Every
// body is a function of one cell (or one wall-plane point), so a kernel is a
// bounds test and one call.
//
// Expressions keep the reference's operation order; the kernels are built
// with -fmad=false and the host build with -ffp-contract=off, so sqrt,
// division and the products round alike on both, and x**3 and x**(1/3) are
// computed correctly rounded on both (cube, cbrt_like), so the device
// reproduces the host bit for bit.
#pragma once

#include <math.h>
#include <stddef.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define TR_HD __host__ __device__ inline
#else
#define TR_HD inline
#endif

#if defined(TR_HOST_CHECK)
#include <stdio.h>
#include <stdlib.h>
#define TR_CHECK(cond, what)                                                            \
    do {                                                                                \
        if (!(cond)) {                                                                  \
            fprintf(stderr, "transport index out of range: %s (%s:%d)\n", what, __FILE__, __LINE__); \
            abort();                                                                    \
        }                                                                               \
    } while (0)
#else
#define TR_CHECK(cond, what) ((void)0)
#endif

namespace tr {

constexpr double VOFEPS = 1.0e-14;   // Clsvof.f90:32
constexpr double ETA = 0.075;        // Clsvof.f90:32
constexpr double TOLPAR = 1.0e-14;   // Clsvof.f90:35
constexpr int BAND = 4;              // band_width, Clsvof.f90:31
constexpr int NSUB = 6;              // nv, Clsvof.f90:31

struct Dims {
    int I, J, K;
    TR_HD size_t g(int i, int j, int k) const
    {
        TR_CHECK(i >= 0 && i <= I + 1 && j >= 0 && j <= J + 1 && k >= 0 && k <= K + 1, "ghosted");
        return (size_t)i + (size_t)(I + 2) * ((size_t)j + (size_t)(J + 2) * (size_t)k);
    }
    TR_HD size_t n(int i, int j, int k) const
    {
        TR_CHECK(i >= 1 && i <= I && j >= 1 && j <= J && k >= 1 && k <= K, "interior");
        return (size_t)(i - 1) + (size_t)I * ((size_t)(j - 1) + (size_t)J * (size_t)(k - 1));
    }
    TR_HD size_t interior() const { return (size_t)I * J * K; }
    TR_HD size_t ghosted() const { return (size_t)(I + 2) * (J + 2) * (K + 2); }
    TR_HD int len(int axis) const { return axis == 0 ? I : axis == 1 ? J : K; }
    // the first dimension of a wall plane normal to `axis`
    TR_HD int plane_lead(int axis) const { return axis == 0 ? J : I; }
    TR_HD size_t plane_size(int axis) const
    {
        return axis == 0 ? (size_t)J * K : axis == 1 ? (size_t)I * K : (size_t)I * J;
    }
};

struct Geo {   // cell centres and spacings, interior
    const double *x, *y, *z, *dx, *dy, *dz;
};

TR_HD double sgn(double a) { return copysign(1.0, a); }

TR_HD uint64_t bits_of(double v)
{
    union { double d; uint64_t u; } c;
    c.d = v;
    return c.u;
}
TR_HD double from_bits(uint64_t u)
{
    union { double d; uint64_t u; } c;
    c.u = u;
    return c.d;
}

// x / d.  When d is a normal power of two its reciprocal is exact and
// x * (1/d) is the same correctly rounded quotient, without an FP64
// division (about ten instructions on GB300's narrow FP64 pipes).  Uniform
// grids with power-of-two spacings, and divisions by 2 or by 1, take it.
TR_HD double divd(double x, double d)
{
    const uint64_t b = bits_of(d);
    const uint64_t e = (b >> 52) & 0x7FFull;
    if ((b & 0xFFFFFFFFFFFFFull) == 0 && e >= 1 && e <= 2045)
        return x * from_bits((b & 0x8000000000000000ull) | ((2046ull - e) << 52));
    return x / d;
}

// x**3.d0, rounded once: x*x split exactly by an FMA, times x split again,
// one rounding of the sum (Dekker's product; correct but for ties finer
// than 2^-100).  gfortran calls the math library's pow, which comes within a
// hair of this but in glibc lands on the wrong side of a near-tie for about
// 0.08% of arguments; the correctly rounded value is what every build of the
// reference approximates, and host and device compute it alike.
TR_HD double cube(double x)
{
    const double p = x * x;
    const double e1 = fma(x, x, -p);   // x*x = p + e1 exactly
    const double c = p * x;
    const double e2 = fma(p, x, -c);   // p*x = c + e2 exactly
    return c + fma(e1, x, e2);
}

// x**(1.d0/3.d0) = x**a, a = fl(1/3) = 1/3 - 2^-54/3, rounded once: the
// cube root c refined by one Newton step on the residual x - c^3 (exact
// products by FMA), times x**(-2^-54/3) = 1 - (2^-54/3) ln x (the next term
// is below 2^-90).  Whatever ulp the starting cbrt or log carry, the sum
// rounds to the same double on host and device.
TR_HD double cbrt_like(double x)
{
    if (!(x > 0.0) || isinf(x)) return pow(x, 1.0 / 3.0);
    const double c = cbrt(x);
    const double c2h = c * c, c2l = fma(c, c, -c2h);
    const double c3h = c2h * c, c3l = fma(c2h, c, -c3h) + c2l * c;
    const double d = ((x - c3h) - c3l) / (3.0 * c2h);
    const double g = -(0x1p-54 / 3.0) * log(x);
    return c + (d + c * g);
}

TR_HD double max3(double a, double b, double c)
{
    const double m = a > b ? a : b;
    return m > c ? m : c;
}
TR_HD double min3(double a, double b, double c)
{
    const double m = a < b ? a : b;
    return m < c ? m : c;
}

// Volume_Fraction_Calc (Clsvof.f90:1475-1550): the liquid volume of the
// box cut at distance s from its corner along the normal.
TR_HD double volume_fraction(double dx, double dy, double dz, double nxx, double nyy, double nzz, double s)
{
    const double nx1 = fabs(nxx), ny1 = fabs(nyy), nz1 = fabs(nzz);
    const double dx1 = max3(nx1 * dx, ny1 * dy, nz1 * dz);
    const double dz1 = min3(nx1 * dx, ny1 * dy, nz1 * dz);
    const double dy1 = nx1 * dx + ny1 * dy + nz1 * dz - dx1 - dz1;
    const double sm = dx1 + dy1 + dz1;
    const double sc = s < sm - s ? s : sm - s;
    if (s <= 0.0) return 0.0;
    if (s >= sm) return 1.0 * dx * dy * dz;
    double fc;
    if (sc <= dz1) {
        fc = cube(sc) / (6.0 * dx1 * dy1 * dz1);
    } else if (sc <= dy1) {
        fc = (sc * sc - dz1 * sc + dz1 * dz1 / 3.0) / (2.0 * dx1 * dy1);
    } else if (dx1 >= dy1 + dz1) {
        if (sc >= dy1 + dz1) {
            fc = (2.0 * sc - dy1 - dz1) / (2.0 * dx1);
        } else {
            fc = cube(sc) - cube(sc - dz1) - cube(sc - dy1);
            fc = fc / (6.0 * dx1 * dy1 * dz1);
        }
    } else {
        if (sc > dx1) fc = cube(sc) - cube(sc - dz1) - cube(sc - dy1) - cube(sc - dx1);
        else fc = cube(sc) - cube(sc - dz1) - cube(sc - dy1);
        fc = fc / (6.0 * dx1 * dy1 * dz1);
    }
    if (s <= 0.5 * sm) return fc * dx * dy * dz;
    return (1.0 - fc) * dx * dy * dz;
}

// Newton_Raphson (1462-1473), at most 200 steps (the reference has no cap).
TR_HD double newton(double a3, double a2, double a1, double a0, double sc)
{
    double delvar = 1.0e6;
    for (int it = 0; it < 200 && fabs(delvar) > 1.0e-6 * fabs(sc); ++it) {
        delvar = (a3 * cube(sc) + a2 * (sc * sc) + a1 * sc + a0) / (3.0 * a3 * (sc * sc) + 2.0 * a2 * sc + a1);
        sc = sc - delvar;
    }
    return sc;
}

// Cubic_Equation_Solve (1380-1398).
TR_HD double cubic(double fc, double dx1, double dy1, double dz1, double sc, bool case2)
{
    if (case2)
        return newton(1.0, -3.0 * (dy1 + dz1), 3.0 * (dy1 * dy1 + dz1 * dz1),
                      6.0 * fc * dx1 * dy1 * dz1 - (cube(dy1) + cube(dz1)), sc);
    return newton(2.0, -3.0 * (dx1 + dy1 + dz1), 3.0 * (dx1 * dx1 + dy1 * dy1 + dz1 * dz1),
                  6.0 * fc * dx1 * dy1 * dz1 - (cube(dx1) + cube(dy1) + cube(dz1)), sc);
}

// Find_Distance (1311-1378) with Final_Distance (1400-1408).
TR_HD double find_distance(double dx, double dy, double dz, double nxx, double nyy, double nzz, double f)
{
    const double nx1 = fabs(nxx), ny1 = fabs(nyy), nz1 = fabs(nzz);
    const double dx1 = max3(nx1 * dx, ny1 * dy, nz1 * dz);
    double dz1 = min3(nx1 * dx, ny1 * dy, nz1 * dz);
    if (fabs(dz1) < TOLPAR) dz1 = 0.0;
    double dy1 = nx1 * dx + ny1 * dy + nz1 * dz - dx1 - dz1;
    if (fabs(dy1) < TOLPAR) dy1 = 0.0;
    const double fc = f < 1.0 - f ? f : 1.0 - f;
    const double sm = dx1 + dy1 + dz1;
    const bool lower = f <= 0.5;
    double sc = 6.0 * fc * dx1 * dy1 * dz1;
    sc = sgn(sc) * cbrt_like(fabs(sc));
    if (sc < dz1) return lower ? sc : sm - sc;
    sc = 0.5 * dz1 + sqrt(2.0 * fc * dx1 * dy1 - dz1 * dz1 / 12.0);
    if (sc < dy1) return lower ? sc : sm - sc;
    sc = fc * dx1 + (dy1 + dz1) / 2.0;
    if (dx1 >= dy1 + dz1) {
        if (sc < dy1 + dz1) sc = cubic(fc, dx1, dy1, dz1, sc, true);
    } else if (sc >= dx1) {
        sc = cubic(fc, dx1, dy1, dz1, sc, false);
        if (sc < dx1) sc = cubic(fc, dx1, dy1, dz1, sc, true);
    } else {
        sc = cubic(fc, dx1, dy1, dz1, sc, true);
    }
    return lower ? sc : sm - sc;
}

// Isinterface (801-815): partly filled, or next to the opposite phase.  A
// bulk cell -- exactly +0 or 1 with its six neighbours holding the same
// bits -- fails every test below, so it is answered with integer compares
// and no FP64 work.
TR_HD bool is_interface(const Dims &D, const double *vfl, int i, int j, int k)
{
    const double v = vfl[D.g(i, j, k)];
    const uint64_t b = bits_of(v);
    if ((b == 0 || b == 0x3FF0000000000000ull) && bits_of(vfl[D.g(i - 1, j, k)]) == b &&
        bits_of(vfl[D.g(i + 1, j, k)]) == b && bits_of(vfl[D.g(i, j - 1, k)]) == b &&
        bits_of(vfl[D.g(i, j + 1, k)]) == b && bits_of(vfl[D.g(i, j, k - 1)]) == b &&
        bits_of(vfl[D.g(i, j, k + 1)]) == b)
        return false;
    const double jump = 1.0 - 2.1 * VOFEPS;
    bool flag = v > VOFEPS && v < 1.0 - VOFEPS;
    if (fabs(vfl[D.g(i - 1, j, k)] - v) >= jump) flag = true;
    if (fabs(vfl[D.g(i + 1, j, k)] - v) >= jump) flag = true;
    if (fabs(vfl[D.g(i, j - 1, k)] - v) >= jump) flag = true;
    if (fabs(vfl[D.g(i, j + 1, k)] - v) >= jump) flag = true;
    if (fabs(vfl[D.g(i, j, k - 1)] - v) >= jump) flag = true;
    if (fabs(vfl[D.g(i, j, k + 1)] - v) >= jump) flag = true;
    return flag;
}

// |grad phi| - 1 of a difference triple, the test Normal_Vector_Irre uses.
TR_HD double off_unit(double vx, double vy, double vz) { return fabs(1.0 - sqrt(vx * vx + vy * vy + vz * vz)); }

TR_HD int side_of(double qm, double qp)
{
    return (qm < ETA && qp >= ETA) ? -1 : (qm >= ETA && qp < ETA) ? 1 : 0;
}

// Normal_Vector_Irre (2361-2456) for 1 < i < I, 1 < j < J, 1 < k < K: per
// axis a one-sided difference towards the side whose neighbour's gradient
// is within ETA of unit length when the other's is not, else the central
// one.  The neighbours' tangential differences are taken where the
// reference takes them (the x test's minus side at i-1 with the j and k
// differences, and so on).
TR_HD void normal_irre(const Dims &D, const Geo &G, const double *phi, int i, int j, int k, double &nxx,
                       double &nyy, double &nzz)
{
    auto P = [&](int a, int b, int c) { return phi[D.g(a, b, c)]; };
    auto X = [&](int a, int b, int c) { return G.x[D.n(a, b, c)]; };
    auto Y = [&](int a, int b, int c) { return G.y[D.n(a, b, c)]; };
    auto Z = [&](int a, int b, int c) { return G.z[D.n(a, b, c)]; };
    auto Q = [](double num, double den) { return divd(num, den); };
    double vx, vy, vz, qm, qp;
    vx = i >= 3 ? Q(P(i, j, k) - P(i - 2, j, k), X(i, j, k) - X(i - 2, j, k))
                : Q(P(i, j, k) - P(i - 1, j, k), X(i, j, k) - X(i - 1, j, k));
    vy = Q(P(i - 1, j + 1, k) - P(i - 1, j - 1, k), Y(i - 1, j + 1, k) - Y(i - 1, j - 1, k));
    vz = Q(P(i - 1, j, k + 1) - P(i - 1, j, k - 1), Z(i - 1, j, k + 1) - Z(i - 1, j, k - 1));
    qm = off_unit(vx, vy, vz);
    vx = i <= D.I - 2 ? Q(P(i + 2, j, k) - P(i, j, k), X(i + 2, j, k) - X(i, j, k))
                      : Q(P(i + 1, j, k) - P(i, j, k), X(i + 1, j, k) - X(i, j, k));
    vy = Q(P(i + 1, j + 1, k) - P(i + 1, j - 1, k), Y(i + 1, j + 1, k) - Y(i + 1, j - 1, k));
    vz = Q(P(i + 1, j, k + 1) - P(i + 1, j, k - 1), Z(i + 1, j, k + 1) - Z(i + 1, j, k - 1));
    qp = off_unit(vx, vy, vz);
    const int sx = side_of(qm, qp);
    vy = j >= 3 ? Q(P(i, j, k) - P(i, j - 2, k), Y(i, j, k) - Y(i, j - 2, k))
                : Q(P(i, j, k) - P(i, j - 1, k), Y(i, j, k) - Y(i, j - 1, k));
    vx = Q(P(i + 1, j - 1, k) - P(i - 1, j - 1, k), X(i + 1, j - 1, k) - X(i - 1, j - 1, k));
    vz = Q(P(i, j - 1, k + 1) - P(i, j - 1, k - 1), Z(i, j - 1, k + 1) - Z(i, j - 1, k - 1));
    qm = off_unit(vx, vy, vz);
    vx = Q(P(i + 1, j + 1, k) - P(i - 1, j + 1, k), X(i + 1, j + 1, k) - X(i - 1, j + 1, k));
    vy = j <= D.J - 2 ? Q(P(i, j + 2, k) - P(i, j, k), Y(i, j + 2, k) - Y(i, j, k))
                      : Q(P(i, j + 1, k) - P(i, j, k), Y(i, j + 1, k) - Y(i, j, k));
    vz = Q(P(i, j + 1, k + 1) - P(i, j + 1, k - 1), Z(i, j + 1, k + 1) - Z(i, j + 1, k - 1));
    qp = off_unit(vx, vy, vz);
    const int sy = side_of(qm, qp);
    vx = Q(P(i + 1, j, k - 1) - P(i - 1, j, k - 1), X(i + 1, j, k - 1) - X(i - 1, j, k - 1));
    vy = Q(P(i, j + 1, k - 1) - P(i, j - 1, k - 1), Y(i, j + 1, k - 1) - Y(i, j - 1, k - 1));
    vz = k >= 3 ? Q(P(i, j, k) - P(i, j, k - 2), Z(i, j, k) - Z(i, j, k - 2))
                : Q(P(i, j, k) - P(i, j, k - 1), Z(i, j, k) - Z(i, j, k - 1));
    qm = off_unit(vx, vy, vz);
    vx = Q(P(i + 1, j, k + 1) - P(i - 1, j, k + 1), X(i + 1, j, k + 1) - X(i - 1, j, k + 1));
    vy = Q(P(i, j + 1, k + 1) - P(i, j - 1, k + 1), Y(i, j + 1, k + 1) - Y(i, j - 1, k + 1));
    vz = k <= D.K - 2 ? Q(P(i, j, k + 2) - P(i, j, k), Z(i, j, k + 2) - Z(i, j, k))
                      : Q(P(i, j, k + 1) - P(i, j, k), Z(i, j, k + 1) - Z(i, j, k));
    qp = off_unit(vx, vy, vz);
    const int sz = side_of(qm, qp);
    nxx = sx == -1 ? Q(P(i, j, k) - P(i - 1, j, k), X(i, j, k) - X(i - 1, j, k))
        : sx == 1  ? Q(P(i + 1, j, k) - P(i, j, k), X(i + 1, j, k) - X(i, j, k))
                   : Q(P(i + 1, j, k) - P(i - 1, j, k), X(i + 1, j, k) - X(i - 1, j, k));
    nyy = sy == -1 ? Q(P(i, j, k) - P(i, j - 1, k), Y(i, j, k) - Y(i, j - 1, k))
        : sy == 1  ? Q(P(i, j + 1, k) - P(i, j, k), Y(i, j + 1, k) - Y(i, j, k))
                   : Q(P(i, j + 1, k) - P(i, j - 1, k), Y(i, j + 1, k) - Y(i, j - 1, k));
    nzz = sz == -1 ? Q(P(i, j, k) - P(i, j, k - 1), Z(i, j, k) - Z(i, j, k - 1))
        : sz == 1  ? Q(P(i, j, k + 1) - P(i, j, k), Z(i, j, k + 1) - Z(i, j, k))
                   : Q(P(i, j, k + 1) - P(i, j, k - 1), Z(i, j, k + 1) - Z(i, j, k - 1));
}

// Interface_Reconstruct (1216-1309) of one cell: the unit normal and the
// corner distance of an interface cell, zeros elsewhere.  Cells on the
// walls take clamped central differences; a vanishing gradient gives +z.
TR_HD void reconstruct(const Dims &D, const Geo &G, const double *vfl, const double *phi, int i, int j, int k,
                       double &n1, double &n2, double &n3, double &d1)
{
    n1 = n2 = n3 = d1 = 0.0;
    if (!is_interface(D, vfl, i, j, k)) return;
    if (i > 1 && i < D.I && j > 1 && j < D.J && k > 1 && k < D.K) {
        normal_irre(D, G, phi, i, j, k, n1, n2, n3);
    } else {
        const int ip = i + 1 < D.I ? i + 1 : D.I, im = i - 1 > 1 ? i - 1 : 1;
        const int jp = j + 1 < D.J ? j + 1 : D.J, jm = j - 1 > 1 ? j - 1 : 1;
        const int kp = k + 1 < D.K ? k + 1 : D.K, km = k - 1 > 1 ? k - 1 : 1;
        n1 = divd(phi[D.g(ip, j, k)] - phi[D.g(im, j, k)], G.x[D.n(ip, j, k)] - G.x[D.n(im, j, k)]);
        n2 = divd(phi[D.g(i, jp, k)] - phi[D.g(i, jm, k)], G.y[D.n(i, jp, k)] - G.y[D.n(i, jm, k)]);
        n3 = divd(phi[D.g(i, j, kp)] - phi[D.g(i, j, km)], G.z[D.n(i, j, kp)] - G.z[D.n(i, j, km)]);
    }
    const double temp = sqrt(n1 * n1 + n2 * n2 + n3 * n3);
    if (temp < 1.0e-14) {
        n1 = 0.0; n2 = 0.0; n3 = 1.0;
    } else {
        n1 = n1 / temp; n2 = n2 / temp; n3 = n3 / temp;
    }
    const size_t c = D.n(i, j, k);
    d1 = find_distance(G.dx[c], G.dy[c], G.dz[c], n1, n2, n3, vfl[D.g(i, j, k)]);
}

// East/West/North/South/Top/Bottom_Flux (1553-1688): the liquid crossing
// one face in one sub-step, per unit face area, from the upstream cell.
TR_HD double face_flux(int axis, int side, double nxx, double nyy, double nzz, double diss, double volf, double dx,
                       double dy, double dz, double wdt)
{
    if (wdt == 0.0) return 0.0;
    const double nn = axis == 0 ? nxx : axis == 1 ? nyy : nzz;
    const bool thin = side > 0 ? nn <= 0.0 : nn >= 0.0;
    double flux;
    if (axis == 0) {
        flux = thin ? volume_fraction(wdt, dy, dz, nxx, nyy, nzz, diss) / (wdt * dy * dz)
                    : (volf * dx * dy * dz - volume_fraction(dx - wdt, dy, dz, nxx, nyy, nzz, diss)) / (wdt * dy * dz);
    } else if (axis == 1) {
        flux = thin ? volume_fraction(dx, wdt, dz, nxx, nyy, nzz, diss) / (dx * wdt * dz)
                    : (volf * dx * dy * dz - volume_fraction(dx, dy - wdt, dz, nxx, nyy, nzz, diss)) / (dx * wdt * dz);
    } else {
        flux = thin ? volume_fraction(dx, dy, wdt, nxx, nyy, nzz, diss) / (dx * dy * wdt)
                    : (volf * dx * dy * dz - volume_fraction(dx, dy, dz - wdt, nxx, nyy, nzz, diss)) / (dx * dy * wdt);
    }
    return flux * wdt;
}

// The fields one directional sweep reads.
struct SweepIn {
    const double *vfl, *phi;                 // ghosted, before the sweep
    const double *nx, *ny, *nz, *dis;        // ghosted normals, interior corner distances
    const double *vel;                       // the axis' face velocity, ghosted
    const double *bc_vel, *bc_lvs;           // the low wall plane of the axis
    const double *vf_first, *ls_first;       // the sub-step's first sweep result (later sweeps)
    double dtv;
    int axis, stage;                         // stage 0, 1, 2 within the sub-step
};

// A cell of the line along `axis` through (a, b): x lines are (j, k),
// y lines (i, k), z lines (i, j).
TR_HD size_t line_g(const Dims &D, int axis, int m, int a, int b)
{
    return axis == 0 ? D.g(m, a, b) : axis == 1 ? D.g(a, m, b) : D.g(a, b, m);
}
TR_HD size_t line_n(const Dims &D, int axis, int m, int a, int b)
{
    return axis == 0 ? D.n(m, a, b) : axis == 1 ? D.n(a, m, b) : D.n(a, b, m);
}

// The VOF flux through the face between cells q and q+1 of a line
// (X_Sweep 835-860 and its y, z forms): a full or empty upstream cell
// sends vfl*u*dt, a partial one its geometric cut.  z tests w >= 0 where x
// and y test > 0.
TR_HD double vof_face(const Dims &D, const Geo &G, const SweepIn &S, int q, int a, int b)
{
    const double w = S.vel[line_g(D, S.axis, q, a, b)];
    const bool down = S.axis == 2 ? w >= 0.0 : w > 0.0;
    const int up = down ? q : q + 1;
    const size_t gu = line_g(D, S.axis, up, a, b), nu = line_n(D, S.axis, up, a, b);
    const double v = S.vfl[gu];
    if (v >= 1.0 - VOFEPS || v <= VOFEPS) return v * w * S.dtv;
    if (down) return face_flux(S.axis, +1, S.nx[gu], S.ny[gu], S.nz[gu], S.dis[gu], v, G.dx[nu], G.dy[nu], G.dz[nu],
                               w * S.dtv);
    return -face_flux(S.axis, -1, S.nx[gu], S.ny[gu], S.nz[gu], S.dis[gu], v, G.dx[nu], G.dy[nu], G.dz[nu], -w * S.dtv);
}

// The level-set flux u*phi_face*dt through the face on the high side of
// cell q, phi_face extrapolated half a step upstream; q = 1 and q = n take
// the reference's boundary forms (x's backward difference /2*dx(2), z's
// plus sign, z's last face scaled by dy).
TR_HD double ls_face(const Dims &D, const Geo &G, const SweepIn &S, const double *d, const double *c, int q, int a,
                     int b)
{
    const int n = D.len(S.axis), ax = S.axis;
    auto PH = [&](int m) { return S.phi[line_g(D, ax, m, a, b)]; };
    auto DD = [&](int m) { return d[line_n(D, ax, m, a, b)]; };
    auto CC = [&](int m) { return c[line_n(D, ax, m, a, b)]; };
    const double w = S.vel[line_g(D, ax, q, a, b)], dtv = S.dtv;
    double ls;
    if (q == 1) {
        if (w >= 0.0) {
            const double den = ax == 0 ? DD(1) : CC(2) - CC(1);
            ls = PH(1) + divd(divd(DD(1), 2.0) * (1.0 - divd(w * dtv, DD(1))) * (PH(2) - PH(1)), den);
        } else if (ax == 0) {
            ls = PH(2) - divd(divd(DD(2), 2.0) * (1.0 + divd(w * dtv, DD(2))) * (PH(3) - PH(1)), 2.0) * DD(2);
        } else if (ax == 1) {
            ls = PH(2) - divd(divd(DD(2), 2.0) * (1.0 + divd(w * dtv, DD(2))) * (PH(3) - PH(1)), CC(3) - CC(1));
        } else {
            ls = PH(2) + divd(divd(DD(2), 2.0) * (1.0 + divd(w * dtv, DD(2))) * (PH(3) - PH(1)), CC(3) - CC(1));
        }
        return ls * w * dtv;
    }
    if (q == n) {
        if (w > 0.0) {
            ls = PH(n) + divd(divd(DD(n), 2.0) * (1.0 - divd(w * dtv, DD(n))) * (PH(n) - PH(n - 1)), CC(n) - CC(n - 1));
        } else {
            const double scale = ax == 2 ? G.dy[line_n(D, ax, n - 1, a, b)] : DD(n - 1);
            ls = PH(n) - divd(divd(DD(n - 1), 2.0) * (1.0 + divd(w * dtv, scale)) * (PH(n) - PH(n - 1)),
                              CC(n) - CC(n - 1));
        }
        return ls * w * dtv;
    }
    const double dm = DD(q), half = divd(dm, 2.0), step = divd(w * dtv, dm);
    if (w >= 0.0) ls = PH(q) + divd(half * (1.0 - step) * (PH(q + 1) - PH(q - 1)), 2.0 * dm);
    else if (q <= n - 2) ls = PH(q + 1) - divd(half * (1.0 + step) * (PH(q + 2) - PH(q)), 2.0 * dm);
    else ls = PH(q + 1) - divd(half * (1.0 + step) * (PH(q + 1) - PH(q)), dm);
    return w * ls * dtv;
}

// One cell of one sweep, gathered: the VOF and level set after the
// sweep's face fluxes (added in the order the reference's face loops add
// them to this cell), then the sub-step's divergence term -- the first
// sweep divides by 1 - dtv/d (u_m - u_{m-1}), the later two add dtv/d
// times the first sweep's result times that difference -- and the clip of
// the VOF to 0 and 1 within 1e-14 (Clsvof_Scheme 486-780).  Needs n >= 3.
TR_HD void sweep_cell(const Dims &D, const Geo &G, const SweepIn &S, int i, int j, int k, double &vf_out,
                      double &ls_out)
{
    const int ax = S.axis, n = D.len(ax);
    const int m = ax == 0 ? i : ax == 1 ? j : k;
    const int a = ax == 0 ? j : i, b = ax == 2 ? j : k;
    const double *d = ax == 0 ? G.dx : ax == 1 ? G.dy : G.dz;
    const double *c = ax == 0 ? G.x : ax == 1 ? G.y : G.z;
    const size_t g = D.g(i, j, k), nc = D.n(i, j, k);
    const double dm = d[nc];
    // VOF (X_Sweep 835-875)
    double tv = S.vfl[g];
    if (m >= 2) tv = tv + divd(vof_face(D, G, S, m - 1, a, b), dm);
    if (m <= n - 1) tv = tv - divd(vof_face(D, G, S, m, a, b), dm);
    if (m == 1) {
        const size_t gw = ax == 0 ? D.g(0, j, k) : ax == 1 ? D.g(i, 0, k) : D.g(i, j, 0);
        const double flux = S.vfl[g] * S.vel[gw] * S.dtv;
        tv = tv + divd(flux, dm);
    }
    if (m == n) {
        const double flux = S.vfl[g] * S.vel[g] * S.dtv;
        tv = tv - divd(flux, dm);
    }
    // level set (X_Sweep 877-947)
    double tl = S.phi[g];
    if (m >= 3) tl = tl + divd(ls_face(D, G, S, d, c, m - 1, a, b), dm);
    if (m >= 2 && m <= n - 1) tl = tl - divd(ls_face(D, G, S, d, c, m, a, b), dm);
    if (m == 1) {
        tl = tl - divd(ls_face(D, G, S, d, c, 1, a, b), dm);
        const size_t bw = (size_t)(a - 1) + (size_t)D.plane_lead(ax) * (size_t)(b - 1);
        TR_CHECK(bw < D.plane_size(ax), "wall plane");
        const double flux = S.bc_vel[bw] * S.bc_lvs[bw] * S.dtv;
        tl = tl + divd(flux, dm);
    }
    if (m == 2) tl = tl + divd(ls_face(D, G, S, d, c, 1, a, b), dm);
    if (m == n) tl = tl - divd(ls_face(D, G, S, d, c, n, a, b), dm);
    // the divergence term and the clip
    const size_t gm = ax == 0 ? D.g(i - 1, j, k) : ax == 1 ? D.g(i, j - 1, k) : D.g(i, j, k - 1);
    const double du = S.vel[g] - S.vel[gm];
    const double rate = divd(S.dtv, dm);
    if (S.stage == 0) {
        const double den = 1.0 - rate * du;
        tv = divd(tv, den);
        tl = divd(tl, den);
    } else {
        tv = tv + rate * S.vf_first[g] * du;
        tl = tl + rate * S.ls_first[g] * du;
    }
    if (tv <= VOFEPS) tv = 0.0;
    if (tv >= 1.0 - VOFEPS) tv = 1.0;
    vf_out = tv;
    ls_out = tl;
}

// ---- redistancing (Redistance_Levelset 1689-1889) ----------------------

TR_HD bool inside_rect(double d1, double d2, double r10, double r11, double r20, double r21)
{
    return r10 <= d1 && d1 <= r11 && r20 <= d2 && d2 <= r21;
}

// Iscutface (1929-1959): the plane crosses the face at `fp` normal to cas.
TR_HD bool cut_face(double fp, double nxx, double nyy, double nzz, double diss, double dx, double dy, double dz,
                    int cas)
{
    double p1, p2, p3, p4;
    if (cas == 1) {
        p1 = fp * nxx - 0.5 * dy * nyy - 0.5 * dz * nzz + diss;
        p2 = fp * nxx - 0.5 * dy * nyy + 0.5 * dz * nzz + diss;
        p3 = fp * nxx + 0.5 * dy * nyy + 0.5 * dz * nzz + diss;
        p4 = fp * nxx + 0.5 * dy * nyy - 0.5 * dz * nzz + diss;
    } else if (cas == 2) {
        p1 = -0.5 * dx * nxx + fp * nyy - 0.5 * dz * nzz + diss;
        p2 = -0.5 * dx * nxx + fp * nyy + 0.5 * dz * nzz + diss;
        p3 = 0.5 * dx * nxx + fp * nyy + 0.5 * dz * nzz + diss;
        p4 = 0.5 * dx * nxx + fp * nyy - 0.5 * dz * nzz + diss;
    } else {
        p1 = -0.5 * dx * nxx - 0.5 * dy * nyy + fp * nzz + diss;
        p2 = -0.5 * dx * nxx + 0.5 * dy * nyy + fp * nzz + diss;
        p3 = 0.5 * dx * nxx + 0.5 * dy * nyy + fp * nzz + diss;
        p4 = 0.5 * dx * nxx - 0.5 * dy * nyy + fp * nzz + diss;
    }
    return !(p1 * p2 >= 0.0 && p2 * p3 >= 0.0 && p3 * p4 >= 0.0 && p4 * p1 >= 0.0);
}

// Shortest_Point_2d (1961-2060) on the face normal to cas (1, 2, 3), whose
// coordinate the caller has set: writes the other two.  Its y-face case
// solves for x dividing by |nz|, as the reference does.
TR_HD void shortest_point_2d(double nx1, double ny1, double nz1, double dis1, int ii, int jj, int kk, int cas,
                             double dx, double dy, double dz, double &xs, double &ys, double &zs)
{
    const double epsi = 1.0e-30;
    // (u, v) are the face's two in-plane axes in the reference's order.
    const double nu1 = cas == 1 ? ny1 : nx1, nv1 = cas == 3 ? ny1 : nz1;
    const double du = cas == 1 ? dy : dx, dv = cas == 3 ? dy : dz;
    const int iu = cas == 1 ? jj : ii, iv = cas == 3 ? jj : kk;
    const double temp = sqrt(nu1 * nu1 + nv1 * nv1 + epsi * epsi);
    const double nuu = nu1 / temp, nvv = nv1 / temp, diss = dis1 / temp;
    const double dij1 = nuu * du * (double)iu + nvv * dv * (double)iv + diss;
    const double up = du * (double)iu - dij1 * nuu, vp = dv * (double)iv - dij1 * nvv;
    double us, vs;
    if (inside_rect(up, vp, -0.5 * du, 0.5 * du, -0.5 * dv, 0.5 * dv)) {
        us = up;
        vs = vp;
    } else {
        const double uoff = fmax(fabs(up) - 0.5 * du, 0.0), voff = fmax(fabs(vp) - 0.5 * dv, 0.0);
        const double ufc = sgn(up) * 0.5 * du, vfc = sgn(vp) * 0.5 * dv;
        if (uoff * fabs(nuu) > voff * fabs(nvv)) {
            us = ufc;
            vs = (diss + nuu * us) / (sgn(-nvv) * fmax(fabs(nvv), TOLPAR));
        } else {
            vs = vfc;
            const double div = cas == 2 ? fabs(nvv) : fabs(nuu);
            us = (diss + nvv * vs) / (sgn(-nuu) * fmax(div, TOLPAR));
        }
    }
    if (cas == 1) { ys = us; zs = vs; }
    else if (cas == 2) { xs = us; zs = vs; }
    else { xs = us; ys = vs; }
}

// The distance Redistance_Levelset measures from the centre (ii, jj, kk)
// cells away to an interface cell's plane n.x + diss = 0 (diss from the
// cell centre; the interface cell's spacings): the facing boundary point
// when it lies across the plane from the target (`side` = phi there),
// else the foot of the perpendicular inside the cell, else the nearest
// point of the plane's trace on the face it leaves through.
TR_HD double band_distance(double nxx, double nyy, double nzz, double diss, int ii, int jj, int kk, double dx,
                           double dy, double dz, double side)
{
    const int l = ii < -1 ? -1 : ii > 1 ? 1 : ii;
    const int m = jj < -1 ? -1 : jj > 1 ? 1 : jj;
    const int n = kk < -1 ? -1 : kk > 1 ? 1 : kk;
    const double xv = dx * (double)l / 2.0, yv = dy * (double)m / 2.0, zv = dz * (double)n / 2.0;
    const double dv = nxx * xv + nyy * yv + nzz * zv + diss;
    const double X = dx * (double)ii, Y = dy * (double)jj, Z = dz * (double)kk;
    if (dv * sgn(side) <= 0.0) return sqrt((X - xv) * (X - xv) + (Y - yv) * (Y - yv) + (Z - zv) * (Z - zv));
    const double dij1 = nxx * dx * (double)ii + nyy * dy * (double)jj + nzz * dz * (double)kk + diss;
    const double xp = X - dij1 * nxx, yp = Y - dij1 * nyy, zp = Z - dij1 * nzz;
    if (-0.5 * dx <= xp && xp <= 0.5 * dx && -0.5 * dy <= yp && yp <= 0.5 * dy && -0.5 * dz <= zp && zp <= 0.5 * dz)
        return sqrt((X - xp) * (X - xp) + (Y - yp) * (Y - yp) + (Z - zp) * (Z - zp));
    const double ax = fmax(fabs(xp) - 0.5 * dx, 0.0) * fabs(nxx);
    const double ay = fmax(fabs(yp) - 0.5 * dy, 0.0) * fabs(nyy);
    const double az = fmax(fabs(zp) - 0.5 * dz, 0.0) * fabs(nzz);
    const double fc[3] = {sgn(xp) * 0.5 * dx, sgn(yp) * 0.5 * dy, sgn(zp) * 0.5 * dz};
    const double nn[3] = {nxx, nyy, nzz};
    double s[3] = {0.0, 0.0, 0.0};
    const double w[3] = {ax, ay, az};
    for (int c = 0; c < 3; ++c) {
        const int o1 = c == 0 ? 1 : 0, o2 = c == 2 ? 1 : 2;
        if (!(w[c] >= w[o1] && w[c] >= w[o2])) continue;
        int cas;
        if (cut_face(fc[c], nxx, nyy, nzz, diss, dx, dy, dz, c + 1)) cas = c;
        else cas = w[o1] > w[o2] ? o1 : o2;
        s[cas] = fc[cas];
        shortest_point_2d(nxx, nyy, nzz, nn[cas] * s[cas] + diss, ii, jj, kk, cas + 1, dx, dy, dz, s[0], s[1], s[2]);
    }
    return sqrt((X - s[0]) * (X - s[0]) + (Y - s[1]) * (Y - s[1]) + (Z - s[2]) * (Z - s[2]));
}

TR_HD bool band_interface(double v) { return 0.0 + 1.0e-15 < v && v < 1.0 - 1.0e-15; }
TR_HD bool band_target(double v) { return v < 0.0 + 1.0e-15 || v > 1.0 - 1.0e-15; }

// The bits of a non-negative double order like the double.
TR_HD uint64_t key_of(double v) { return bits_of(v); }
TR_HD double value_of(uint64_t u) { return from_bits(u); }

TR_HD void atomic_min_key(unsigned long long *slot, unsigned long long key)
{
#if defined(__CUDA_ARCH__)
    atomicMin(slot, key);
#else
    if (key < *slot) *slot = key;
#endif
}

constexpr int BAND_SPAN = 2 * BAND + 1;
constexpr int BAND_CELLS = BAND_SPAN * BAND_SPAN * BAND_SPAN;   // 729 offsets

// Offset t (0 .. BAND_CELLS-1) of an interface cell's band, ii fastest.
TR_HD void band_offset(int t, int &ii, int &jj, int &kk)
{
    ii = t % BAND_SPAN - BAND;
    jj = (t / BAND_SPAN) % BAND_SPAN - BAND;
    kk = t / (BAND_SPAN * BAND_SPAN) - BAND;
}

// Interior cell of index c (i fastest), the inverse of Dims::n, in 32-bit
// arithmetic (the transport context holds fewer than 2^32 interior cells).
TR_HD void cell_of(const Dims &D, uint32_t c, int &i, int &j, int &k)
{
    const uint32_t r = c / (uint32_t)D.I;
    i = (int)(c - r * (uint32_t)D.I) + 1;
    const uint32_t kq = r / (uint32_t)D.J;
    j = (int)(r - kq * (uint32_t)D.J) + 1;
    k = (int)kq + 1;
}

// One pair of the band (1726-1861): the interface cell (i, j, k) and its
// offset t.  A full or empty target cell within BAND cells in each index is
// marked and keeps the least distance seen; dis holds the distances from
// the cell centres.  The minimum does not depend on the order of the pairs.
TR_HD void band_pair(const Dims &D, const Geo &G, const double *vfl, const double *phi, const double *nx,
                     const double *ny, const double *nz, const double *dis, int i, int j, int k, int t,
                     unsigned long long *key, uint8_t *fix)
{
    int ii, jj, kk;
    band_offset(t, ii, jj, kk);
    const int ti = i + ii, tj = j + jj, tk = k + kk;
    if (!(1 <= ti && ti <= D.I && 1 <= tj && tj <= D.J && 1 <= tk && tk <= D.K)) return;
    const size_t tg = D.g(ti, tj, tk), tc = D.n(ti, tj, tk);
    if (!band_target(vfl[tg])) return;
    const size_t g = D.g(i, j, k), c = D.n(i, j, k);
    fix[tc] = 1;
    const double deuc = band_distance(nx[g], ny[g], nz[g], dis[g], ii, jj, kk, G.dx[c], G.dy[c], G.dz[c], phi[tg]);
    atomic_min_key(key + tc, key_of(deuc));
}

// One interface cell's whole band, pair by pair.
TR_HD void band_scatter(const Dims &D, const Geo &G, const double *vfl, const double *phi, const double *nx,
                        const double *ny, const double *nz, const double *dis, int i, int j, int k,
                        unsigned long long *key, uint8_t *fix)
{
    if (!band_interface(vfl[D.g(i, j, k)])) return;
    for (int t = 0; t < BAND_CELLS; ++t) band_pair(D, G, vfl, phi, nx, ny, nz, dis, i, j, k, t, key, fix);
}

// The level set each cell ends with (1866-1882).
TR_HD double band_value(const Dims &D, const Geo &G, const double *vfl, const double *dis, int i, int j, int k,
                        const unsigned long long *key, const uint8_t *fix)
{
    const size_t g = D.g(i, j, k), c = D.n(i, j, k);
    const double v = vfl[g];
    if (band_interface(v)) return sgn(0.5 - v) * fabs(dis[g]);
    if (fix[c]) return sgn(0.5 - v) * value_of(key[c]);
    return (double)(BAND + 1) * G.dx[c] * sqrt(3.0) * sgn(0.5 - v);
}

// ---- boundary planes (BoundaryConditionLvsVof 2087-2221) -----------------

struct WallIn {
    double *phil, *vofl;                     // ghosted: the sub-step's result
    double *phil_more[2], *vofl_more[2];     // the other ping-pong buffers, whose
                                             // ghost faces must match (or null)
    const double *nxl;                       // liquid normal, ghosted
    const double *nx, *ny, *nz;              // fluid normals, ghosted
    double *lvs_bc[6], *vof_bc[6];           // planes W, E, S, N, B, T
    int lvs_flag[6], vof_flag[6];
    double lvs_const[6], vof_const[6];
};

TR_HD double typical_bc(int flag, double cst, double var, double d) { return flag == 0 ? cst : var - cst * d / 2.0; }

// Point t of the wall planes normal to `axis`, both faces, level set then
// VOF.  W and E level-set planes are phiL -/+ nxL*dx/2 (the reference hands
// BCLvsW/E the liquid normals); the others are TypicalBC; the level-set
// ghosts step by the fluid normal times the spacing, the north one
// subtracting like the south; the VOF ghosts copy the wall cell.
TR_HD void wall_point(const Dims &D, const Geo &G, const WallIn &W, int axis, size_t t)
{
    const int lead = D.plane_lead(axis);
    const int a = (int)(t % (size_t)lead) + 1, b = (int)(t / (size_t)lead) + 1;
    const int n = D.len(axis);
    const size_t g1 = line_g(D, axis, 1, a, b), gn = line_g(D, axis, n, a, b);
    const size_t g0 = line_g(D, axis, 0, a, b), gx = line_g(D, axis, n + 1, a, b);
    const size_t c1 = line_n(D, axis, 1, a, b), cn = line_n(D, axis, n, a, b);
    const double *d = axis == 0 ? G.dx : axis == 1 ? G.dy : G.dz;
    const double *fn = axis == 0 ? W.nx : axis == 1 ? W.ny : W.nz;
    const double d1 = d[c1], dn = d[cn];
    const int lo = 2 * axis, hi = 2 * axis + 1;
    // level set
    double p1 = W.phil[g1], pn = W.phil[gn];
    double wlo = typical_bc(W.lvs_flag[lo], W.lvs_const[lo], p1, d1);
    double whi = typical_bc(W.lvs_flag[hi], W.lvs_const[hi], pn, -dn);
    if (axis == 0) {
        wlo = p1 - W.nxl[g1] * d1 / 2.0;
        whi = pn - W.nxl[gn] * (-dn) / 2.0;
    }
    W.lvs_bc[lo][t] = wlo;
    W.lvs_bc[hi][t] = whi;
    const double lo_ghost = p1 - fn[g1] * d1;
    const double hi_ghost = axis == 1 ? pn - fn[gn] * dn : pn + fn[gn] * dn;
    W.phil[g0] = lo_ghost;
    W.phil[gx] = hi_ghost;
    // VOF
    const double v1 = W.vofl[g1], vn = W.vofl[gn];
    W.vof_bc[lo][t] = typical_bc(W.vof_flag[lo], W.vof_const[lo], v1, d1);
    W.vof_bc[hi][t] = typical_bc(W.vof_flag[hi], W.vof_const[hi], vn, -dn);
    W.vofl[g0] = v1;
    W.vofl[gx] = vn;
    for (int q = 0; q < 2; ++q) {
        if (W.phil_more[q]) {
            W.phil_more[q][g0] = lo_ghost;
            W.phil_more[q][gx] = hi_ghost;
        }
        if (W.vofl_more[q]) {
            W.vofl_more[q][g0] = v1;
            W.vofl_more[q][gx] = vn;
        }
    }
}

// ---- the velocity cells' liquid fields (ComputeUVWLiquidField 174-353) ----

// ConvertTheCoordinateSystem (2458-2465): phi measured from the corner.
TR_HD double corner_level(double dx, double dy, double dz, double nx, double ny, double nz, double phi)
{
    return phi + 0.5 * (fabs(nx) * dx + fabs(ny) * dy + fabs(nz) * dz);
}

// The four averaged fields (phiL, nxL, nyL, nzL) of velocity family `fam`
// (0 U, 1 V, 2 W) at its cell (p, q, r), 0 <= p < I, 0 <= q < J, 0 <= r < K.
// DirectionAverageArray (328-353) writes the average of the P cells
// (i, i+1) along the family's axis into VelCell(i-1, j-1, k-1) -- an
// assumed-shape dummy numbered from 1 over arrays allocated from 0 -- and
// copies the last one once more, so the cell gathers the P pair at
// (p+1, q+1, r+1) with the axis index held at n-1.  d: the P spacing along
// the axis.
TR_HD void family_average(const Dims &D, int fam, const double *d, const double *const pin[4], int p, int q, int r,
                          double out[4])
{
    int i = p + 1, j = q + 1, k = r + 1;
    if (fam == 0 && i == D.I) i = D.I - 1;
    if (fam == 1 && j == D.J) j = D.J - 1;
    if (fam == 2 && k == D.K) k = D.K - 1;
    const int i2 = i + (fam == 0), j2 = j + (fam == 1), k2 = k + (fam == 2);
    const double lamda = divd(d[D.n(i2, j2, k2)], d[D.n(i, j, k)] + d[D.n(i2, j2, k2)]);
    const size_t a = D.g(i, j, k), b = D.g(i2, j2, k2);
    for (int f = 0; f < 4; ++f) out[f] = lamda * pin[f][a] + (1.0 - lamda) * pin[f][b];
}

// The liquid fraction of velocity cell (i, j, k) of family `fam`: the
// liquid in the half of P cell (i, j, k) on its high side plus the half of
// the next P cell on its low side, over the velocity cell's volume; the
// last cell of each line takes the P cell's own fraction (ComputeUVW-
// LiquidField 186-297).  Kept as the reference computes them: the V cell's
// low half cuts with the whole dy and the unshifted level set, its high
// half starts from phiL(i,j,k) with the normal of (i,j+1,k); the W cell's
// high half shifts by +dz/2 where the U cell's shifts by -dx/2.
TR_HD double family_vofl(const Dims &D, int fam, const double *pdx, const double *pdy, const double *pdz,
                         const double *phil, const double *nxl, const double *nyl, const double *nzl,
                         const double *vofl, const double *vdx, const double *vdy, const double *vdz, int i, int j,
                         int k)
{
    const int n = D.len(fam), m = fam == 0 ? i : fam == 1 ? j : k;
    const size_t a = D.g(i, j, k), na = D.n(i, j, k);
    if (m == n) return vofl[a];
    const int i2 = i + (fam == 0), j2 = j + (fam == 1), k2 = k + (fam == 2);
    const size_t b = D.g(i2, j2, k2), nb = D.n(i2, j2, k2);
    double dcell, phinew, dist, left, right;
    if (fam == 0) {
        dcell = pdx[na] / 2.0;
        phinew = phil[a] + dcell * nxl[a];
        dist = corner_level(dcell, pdy[na], pdz[na], nxl[a], nyl[a], nzl[a], phinew);
        left = volume_fraction(dcell, pdy[na], pdz[na], nxl[a], nyl[a], nzl[a], dist);
        left = dcell * pdy[na] * pdz[na] - left;
        dcell = pdx[nb] / 2.0;
        phinew = phil[b] - dcell * nxl[b];
        dist = corner_level(dcell, pdy[nb], pdz[nb], nxl[b], nyl[b], nzl[b], phinew);
        right = volume_fraction(dcell, pdy[nb], pdz[nb], nxl[b], nyl[b], nzl[b], dist);
        right = dcell * pdy[nb] * pdz[nb] - right;
    } else if (fam == 1) {
        dcell = pdy[na] / 2.0;
        dist = corner_level(pdx[na], pdy[na], pdz[na], nxl[a], nyl[a], nzl[a], phil[a]);
        left = volume_fraction(pdx[na], dcell, pdz[na], nxl[a], nyl[a], nzl[a], dist);
        left = pdx[na] * dcell * pdz[na] - left;
        dcell = pdy[nb] / 2.0;
        phinew = phil[a] + dcell * nyl[b];
        dist = corner_level(pdx[nb], dcell, pdz[nb], nxl[b], nyl[b], nzl[b], phinew);
        right = volume_fraction(pdx[nb], dcell, pdz[nb], nxl[b], nyl[b], nzl[b], dist);
        right = pdx[nb] * dcell * pdz[nb] - right;
    } else {
        dcell = pdz[na] / 2.0;
        phinew = phil[a] + dcell * nzl[a];
        dist = corner_level(pdx[na], pdy[na], dcell, nxl[a], nyl[a], nzl[a], phinew);
        left = volume_fraction(pdx[na], pdy[na], dcell, nxl[a], nyl[a], nzl[a], dist);
        left = pdx[na] * pdy[na] * dcell - left;
        dcell = pdz[nb] / 2.0;
        phinew = phil[b] + dcell * nzl[b];
        dist = corner_level(pdx[nb], pdy[nb], dcell, nxl[b], nyl[b], nzl[b], phinew);
        right = volume_fraction(pdx[nb], pdy[nb], dcell, nxl[b], nyl[b], nzl[b], dist);
        right = pdx[nb] * pdy[nb] * dcell - right;
    }
    return divd(divd(divd(left + right, vdx[na]), vdy[na]), vdz[na]);
}

}  // namespace tr
