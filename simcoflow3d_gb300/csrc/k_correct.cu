// k_correct.cu -- pressure scatter, velocity correction, boundary conditions.
//
// Compiled with -fmad=false so that each expression rounds exactly as the
// reference's Fortran statement does.
#include "scf_kernels.h"

// ---------------------------------------------------------------------------
// DeltaPressureGetValues + DeltaPressureBoundaryCondition (ProjectionP.f90:
// 578-643).  With PosNu numbering the active cells in loop order, the
// reference's `PosNu == ctr` test selects exactly the active cells.
__global__ void __launch_bounds__(256) k_scatter(CorrArgs a)
{
    const Dims &d = a.d;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
    if (i > d.I || j > d.J || k > d.K) return;
    const int g = gidx(d, i, j, k);
    a.pp[g] = a.ct[nidx(d, i, j, k)] != 2 ? a.x[g] : 0.0;
}

__global__ void k_pp_ghost(CorrArgs a)
{
    const Dims &d = a.d;
    const int f = blockIdx.z;  // 0..5 = W,E,S,N,B,T
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int axis = f >> 1;
    const int na = axis == 0 ? d.J : d.I;
    const int nb = axis == 2 ? d.J : d.K;
    if (t >= na * nb) return;
    const int p = t % na + 1, q = t / na + 1;
    const double fl = (double)a.bcp_flag[f];
    const bool lo = (f & 1) == 0;
    if (axis == 0) {
        const int src = lo ? 1 : d.I, dst = lo ? 0 : d.I + 1;
        a.pp[gidx(d, dst, p, q)] = fl * a.pp[gidx(d, src, p, q)];
    } else if (axis == 1) {
        const int src = lo ? 1 : d.J, dst = lo ? 0 : d.J + 1;
        a.pp[gidx(d, p, dst, q)] = fl * a.pp[gidx(d, p, src, q)];
    } else {
        const int src = lo ? 1 : d.K, dst = lo ? 0 : d.K + 1;
        a.pp[gidx(d, p, q, dst)] = fl * a.pp[gidx(d, p, q, src)];
    }
}

static int max_plane(const Dims &d)
{
    int m = d.J * d.K;
    if (d.I * d.K > m) m = d.I * d.K;
    if (d.I * d.J > m) m = d.I * d.J;
    return m;
}

void launch_scatter(const CorrArgs &a, cudaStream_t st, int *launches)
{
    const Dims &d = a.d;
    Launch3 l = launch_interior(d.I, d.J, d.K);
    k_scatter<<<l.grid, l.block, 0, st>>>(a);
    dim3 g((max_plane(d) + 255) / 256, 1, 6);
    k_pp_ghost<<<g, 256, 0, st>>>(a);
    *launches += 2;
}

// ---------------------------------------------------------------------------
// Velocity correction (ComputePUVW.f90:181-232).
__global__ void __launch_bounds__(256) k_correct(CorrArgs a)
{
    const Dims &d = a.d;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
    if (i > d.I || j > d.J || k > d.K) return;
    const int g = gidx(d, i, j, k), n = nidx(d, i, j, k);
    const long long N = d.n;
    const double pc = a.pp[g];
    if (a.umoex[n] != 1 && a.uct[n] != 2)
        a.u[g] = a.us[g] - (a.pp[g + 1] - pc) * a.pocoef[n + 3 * N];
    else
        a.u[g] = 0.0;
    if (a.vmoex[n] != 1 && a.vct[n] != 2)
        a.v[g] = a.vs[g] - (a.pp[g + d.gx] - pc) * a.pocoef[n + 4 * N];
    else
        a.v[g] = 0.0;
    if (a.wmoex[n] != 1 && a.wct[n] != 2)
        a.w[g] = a.ws[g] - (a.pp[g + d.gx * d.gy] - pc) * a.pocoef[n + 5 * N];
    else
        a.w[g] = 0.0;
    a.p[g] = pc;
}

// ---------------------------------------------------------------------------
// BoundaryConditionVarNew (ComputePUVW.f90:418-694) with TypicalBC
// (BoundaryFunction.f90:760-781).  For each field the faces are processed in
// the reference's order W,E,S,N,B,T; fields are independent of one another,
// so one launch per face handles u, v, w and p.  The field argument of each
// BC routine is a full ghosted plane section whose lower bound becomes 1, so
// Var(a,b) reads the field at in-plane indices (a-1, b-1).
//
// Per field and face: source plane of the field argument, factor on the
// spacing argument, plane that receives Var (or none), ghost plane written
// from (in -> out) with ComputeGhostVarBoundary (or none).
struct BcStep {
    int src, setpl, gin, gout;  // plane indices; -1 = none
    double dsc;
};

__device__ BcStep bc_step(const Dims &d, int field, int face)
{
    const int I = d.I, J = d.J, K = d.K;
    BcStep s;
    switch (face) {
    case 0: s = {1, -1, 1, 0, 1.0}; break;
    case 1: s = {I, -1, I, I + 1, -1.0}; break;
    case 2: s = {1, -1, 1, 0, 1.0}; break;
    case 3: s = {J, -1, J, J + 1, -1.0}; break;
    case 4: s = {1, -1, 1, 0, 1.0}; break;
    default: s = {K, -1, K, K + 1, -1.0}; break;
    }
    if (field == 0) {          // u: BCUW..BCUT
        if (face == 0) { s.setpl = 0; s.gout = -1; }
        if (face == 1) { s.src = I - 1; s.dsc = -2.0; s.setpl = I; }
    } else if (field == 1) {   // v
        if (face == 2) { s.setpl = 0; s.gout = -1; }
        if (face == 3) { s.src = J - 1; s.dsc = -2.0; s.setpl = J; }
    } else if (field == 2) {   // w
        if (face == 4) { s.setpl = 0; s.gout = -1; }
        if (face == 5) { s.src = K - 1; s.dsc = -2.0; s.setpl = K; }
    } else {                   // p
        if (face == 5) { s.setpl = K; }
    }
    return s;
}

__device__ __forceinline__ int plane_g(const Dims &d, int axis, int pl, int a, int b)
{
    return axis == 0 ? gidx(d, pl, a, b) : axis == 1 ? gidx(d, a, pl, b) : gidx(d, a, b, pl);
}

__device__ __forceinline__ double spacing(const CorrArgs &c, int axis, int face, int a, int b)
{
    const Dims &d = c.d;
    if (axis == 0) return c.pdx[nidx(d, (face & 1) ? d.I : 1, a, b)];
    if (axis == 1) return c.pdy[nidx(d, a, (face & 1) ? d.J : 1, b)];
    return c.pdz[nidx(d, a, b, (face & 1) ? d.K : 1)];
}

// phase 0: compute Var (and write it to the plane/ghost when no hazard);
// phase 1 (top face only): apply the writes from the saved Var.
__global__ void k_bc_face(CorrArgs c, int face, int phase)
{
    const Dims &d = c.d;
    const int axis = face >> 1;
    const int na = axis == 0 ? d.J : d.I;
    const int nb = axis == 2 ? d.J : d.K;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int field = blockIdx.y;
    if (t >= na * nb) return;
    const int a = t % na + 1, b = t / na + 1;
    double *F = field == 0 ? c.u : field == 1 ? c.v : field == 2 ? c.w : c.p;
    const BcStep s = bc_step(d, field, face);
    const int flag = c.flag[field][face];
    double var;
    if (phase == 0) {
        if (flag == 0) {
            var = c.cst[field][face];
        } else {
            const double dxyz = s.dsc * spacing(c, axis, face, a, b);
            var = F[plane_g(d, axis, s.src, a - 1, b - 1)] - c.cst[field][face] * dxyz / 2.0;
        }
        c.bcvar[field][face][t] = var;
        // the top face of p writes the plane it reads: defer to phase 1
        if (face == 5) return;
    } else {
        var = c.bcvar[field][face][t];
    }
    if (s.setpl >= 0) F[plane_g(d, axis, s.setpl, a, b)] = var;
    if (s.gout >= 0) {
        const double xin = F[plane_g(d, axis, s.gin, a, b)];
        F[plane_g(d, axis, s.gout, a, b)] = flag == 1 ? var - xin : 2.0 * var - xin;
    }
}

// Dirichlet-face mass correction (ComputePUVW.f90:260-384): only the first
// Dirichlet pressure face in the order W,E,S,N,B,T is corrected.
__global__ void k_mass_fix(CorrArgs c, int face)
{
    const Dims &d = c.d;
    const int axis = face >> 1;
    const int na = axis == 0 ? d.J : d.I;
    const int nb = axis == 2 ? d.J : d.K;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= na * nb) return;
    const int a = t % na + 1, b = t / na + 1;
    int i, j, k;
    if (axis == 0) { i = (face == 0) ? 1 : d.I; j = a; k = b; }
    else if (axis == 1) { i = a; j = (face == 2) ? 1 : d.J; k = b; }
    else { i = a; j = b; k = (face == 4) ? 1 : d.K; }
    const int g = gidx(d, i, j, k), n = nidx(d, i, j, k);
    const int sy = d.gx, sz = d.gx * d.gy;
    const double DX = c.pdx[n], DY = c.pdy[n], DZ = c.pdz[n];
    const double EE = c.ee[g], NE = c.ne[g], TE = c.te[g];
    double *u = c.u, *v = c.v, *w = c.w;
    switch (face) {
    case 0:
        u[g - 1] = (DX * DZ * (NE * v[g] - NE * v[g - sy]) + DX * DY * (TE * w[g] - TE * w[g - sz]) +
                    DY * DZ * EE * u[g]) / EE / DY / DZ;
        break;
    case 1:
        u[g] = (DX * DZ * (-NE * v[g] + NE * v[g - sy]) + DX * DY * (-TE * w[g] + TE * w[g - sz]) +
                DY * DZ * EE * u[g - 1]) / EE / DY / DZ;
        break;
    case 2:
        v[g - sy] = (DY * DZ * (EE * u[g] - EE * u[g - 1]) + DX * DY * (TE * w[g] - TE * w[g - sz]) +
                     DX * DZ * NE * v[g]) / NE / DX / DZ;
        break;
    case 3:  // the evident intent of ComputePUVW.f90:323-341 (opt-in)
        v[g] = (-DY * DZ * (EE * u[g] - EE * u[g - 1]) - DX * DY * (TE * w[g] - TE * w[g - sz]) +
                DX * DZ * NE * v[g - sy]) / NE / DX / DZ;
        break;
    case 4:
        w[g - sz] = (DY * DZ * (EE * u[g] - EE * u[g - 1]) + DX * DZ * (NE * v[g] - NE * v[g - sy]) +
                     DX * DY * TE * w[g]) / TE / DX / DY;
        break;
    default:
        w[g] = (-DY * DZ * (EE * u[g] - EE * u[g - 1]) - DX * DZ * (NE * v[g] - NE * v[g - sy]) +
                DX * DY * TE * w[g - sz]) / TE / DX / DY;
        break;
    }
}

void launch_correct(const CorrArgs &a, cudaStream_t st, int *launches)
{
    const Dims &d = a.d;
    Launch3 l = launch_interior(d.I, d.J, d.K);
    k_correct<<<l.grid, l.block, 0, st>>>(a);
    *launches += 1;
    for (int face = 0; face < 6; ++face) {
        const int axis = face >> 1;
        const int na = axis == 0 ? d.J : d.I;
        const int nb = axis == 2 ? d.J : d.K;
        dim3 g((na * nb + 255) / 256, 4);
        k_bc_face<<<g, 256, 0, st>>>(a, face, 0);
        *launches += 1;
        if (face == 5) {
            k_bc_face<<<g, 256, 0, st>>>(a, face, 1);
            *launches += 1;
        }
    }
    int first = -1;
    for (int f = 0; f < 6; ++f)
        if (a.bcp_flag[f] == 0) { first = f; break; }
    if (first >= 0 && (first != 3 || a.north_fix)) {
        const int axis = first >> 1;
        const int na = axis == 0 ? d.J : d.I;
        const int nb = axis == 2 ? d.J : d.K;
        k_mass_fix<<<(na * nb + 255) / 256, 256, 0, st>>>(a, first);
        *launches += 1;
    }
}
