// k_predictor.cu -- assembly of the momentum systems and the tail of
// PredictingUVW (src/PredictUVW.f90).  Compiled with -fmad=false: every
// FP64 expression below is evaluated with the reference's operations in its
// order, so Dp is bit-identical to the Fortran and the rows differ from
// HYPRE's only by the Jacobi scaling.
#include "pred_kernels.h"

namespace pred {

dim3 interior_block() { return dim3(32, 4, 2); }
dim3 interior_grid(const Dims &d) { return dim3((d.I + 31) / 32, (d.J + 3) / 4, (d.K + 1) / 2); }

namespace {

__device__ __forceinline__ long long gidx(const Dims &d, int i, int j, int k) { return i + d.sy * j + d.sz * k; }

// The inputs of one row of SetMatrix that do not depend on the velocity
// (the row key): six conductances DF, six cut-face terms EDF, six
// interpolation weights Eta, vof, vofL, dx, dy, dz, Fric; plus which
// boundaries the row touches.
enum { KDFE, KDFW, KDFN, KDFS, KDFT, KDFB, KEE, KEW, KEN, KES, KET, KEB, KETAE, KETAW, KETAN, KETAS, KETAT, KETAB,
       KVOF, KVOFL, KDX, KDY, KDZ, KFRIC, NKEY };
// What a row's key determines (the memo): the scaled couplings a_d / aP
// (W,S,B,E,N,T), 1/aP, Dp, the gravity term of the rhs, and the boundary
// coefficients CWE/CSN/CBT before the cut-cell terms (W,E,S,N,B,T).
enum { MW, MS, MB, ME, MN, MT, MINV, MDP, MG, MCW, MCE, MCS, MCN, MCB, MCT, NMEMO };
constexpr int ASM_NT = 128;   // threads of an assembly block; the stride of the shared-memory slots

// SetMatrix for one row (PredictUVW.f90:904-1040) with the reference's
// operations in its order; called only when the key differs from the
// previous row's (never inlined, so none of it runs speculatively).
__device__ __noinline__ void mom_row(const double *k, const MomParams &o, int comp, int ib, double *mo)
{
    const int iu = comp == 1, iv = comp == 2, iw = comp == 3;
    const double CoefEW = (double)iu + (double)iv / 2.0 + (double)iw / 2.0;
    const double CoefNS = (double)iu / 2.0 + (double)iv + (double)iw / 2.0;
    const double CoefTB = (double)iu / 2.0 + (double)iv / 2.0 + (double)iw;
    auto K = [&](int q) { return k[q * ASM_NT]; };
    const double omb = 1.0 - o.beta_vis;
    const double vof = K(KVOF), vofl = K(KVOFL);
    const double rho = vofl * o.rho_w + (vof - vofl) * o.rho_a;
    // x / rho without a division where that is exact: rho a power of two
    // (the liquid's 1.0 with the water reference density) gives the same
    // rounding as x * (1/rho) (the two real quotients are equal), and
    // x = +-0 over a finite non-zero rho gives the signed zero.
    const long long rb = __double_as_longlong(rho);
    const int rexp = (int)((rb >> 52) & 0x7ff);
    const bool pow2 = (rb & 0xfffffffffffffLL) == 0 && rexp > 0 && rexp < 0x7fe;
    const bool finite_nz = rexp > 0 && rexp < 0x7ff;
    const double rinv = pow2 ? 1.0 / rho : 0.0;
    auto q = [&](double x) {
        if (pow2) return x * rinv;
        if (x == 0.0 && finite_nz) return rho > 0.0 ? x : -x;
        return x / rho;
    };
    double Dfe = q(omb * K(KDFE)), Dfw = q(omb * K(KDFW));
    double Dfn = q(omb * K(KDFN)), Dfs = q(omb * K(KDFS));
    double Dft = q(omb * K(KDFT)), Dfb = q(omb * K(KDFB));
    const double ee = K(KEE), ew = K(KEW), en = K(KEN), es = K(KES), et = K(KET), eb = K(KEB);
    const double etaE = K(KETAE), etaW = K(KETAW), etaN = K(KETAN), etaS = K(KETAS), etaT = K(KETAT),
                 etaB = K(KETAB);
    double Fep = q(ee * (1.0 - etaE)), Fem = q(ee * etaE);
    double Fwp = q(ew * etaW), Fwm = q(ew * (1.0 - etaW));
    double Fnp = q(en * (1.0 - etaN)), Fnm = q(en * etaN);
    double Fsp = q(es * etaS), Fsm = q(es * (1.0 - etaS));
    double Ftp = q(et * (1.0 - etaT)), Ftm = q(et * etaT);
    double Fbp = q(eb * etaB), Fbm = q(eb * (1.0 - etaB));
    // boundary faces (939-1009); ib bits: i = 1, i = ie, j = 1, j = je,
    // k = 1, k = ke; flags 1 = Neumann
    const int *fl = o.flags;
    if (ib & 1) {
        if (fl[0] == 1) { Dfw = 0.0; Fwp = 0.0; Fwm = 0.0; }
        else { Dfw = Dfw * CoefEW; Fwp = Fwp * CoefEW; Fwm = Fwm * CoefEW; }
    }
    if (ib & 2) {
        if (fl[1] == 1) { Dfe = 0.0; Fep = 0.0; Fem = 0.0; }
        else { Dfe = Dfe * CoefEW; Fep = Fep * CoefEW; Fem = Fem * CoefEW; }
    }
    if (ib & 4) {
        if (fl[2] == 1) { Dfs = 0.0; Fsp = 0.0; Fsm = 0.0; }
        else { Dfs = Dfs * CoefNS; Fsp = Fsp * CoefNS; Fsm = Fsm * CoefNS; }
    }
    if (ib & 8) {
        if (fl[3] == 1) { Dfn = 0.0; Fnp = 0.0; Fnm = 0.0; }
        else { Dfn = Dfn * CoefNS; Fnp = Fnp * CoefNS; Fnm = Fnm * CoefNS; }
    }
    if (ib & 16) {
        if (fl[4] == 1) { Dfb = 0.0; Fbp = 0.0; Fbm = 0.0; }
        else { Dfb = Dfb * CoefTB; Fbp = Fbp * CoefTB; Fbm = Fbm * CoefTB; }
    }
    if (ib & 32) {
        if (fl[5] == 1) { Dft = 0.0; Ftp = 0.0; Ftm = 0.0; }
        else { Dft = Dft * CoefTB; Ftp = Ftp * CoefTB; Ftm = Ftm * CoefTB; }
    }
    double aE = Dfe, aW = Dfw, aN = Dfn, aS = Dfs, aT = Dft, aB = Dfb;
    auto M = [&](int r, double val) { mo[r * ASM_NT] = val; };
    M(MCW, aW); M(MCE, aE); M(MCS, aS); M(MCN, aN); M(MCB, aB); M(MCT, aT);   // CWE/CSN/CBT
    const double dx = K(KDX), dy = K(KDY), dz = K(KDZ);
    double aP = vof * dx * dy * dz / o.dt + aE + aW + aN + aS + aT + aB + K(KFRIC);
    aP = aP + Fep - Fwp + Fnp - Fsp + Ftp - Fbp;
    aE = aE - Fem;
    aW = aW + Fwm;
    aN = aN - Fnm;
    aS = aS + Fsm;
    aT = aT - Ftm;
    aB = aB + Fbm;
    const double dp0 = 1.0 / (aP - aE - aW - aN - aS - aT - aB);
    M(MDP, vof * dx * dy * dz * dp0);
    const double G3 = o.gx * (double)iu + o.gy * (double)iv + o.gz * (double)iw;
    M(MG, o.rfr2 * vof * dx * dy * dz * G3 / o.g);   // rfr2 = 1.d0/Fr**2.d0, formed once
    const double inv = 1.0 / aP;
    M(MINV, inv);
    M(MW, aW * inv); M(MS, aS * inv); M(MB, aB * inv);
    M(ME, aE * inv); M(MN, aN * inv); M(MT, aT * inv);
}

// One thread per (i, j) column, marching KZ cells along k.  Active cells of
// the loop range (i <= I-iu, j <= J-iv, k <= K-iw, Cell_Type /= 2) get the
// row of SetMatrix scaled by 1/aP and the rhs of SetVectors (1211-1251),
// every other interior cell an identity row.  Dp: 0 on the loop range,
// vof*dV/(aP - the neighbour coefficients) on its active cells (913, 1040,
// 1226-1237).  Consecutive rows of a column with bit-identical keys (most
// rows away from the interface and the solid) reuse the previous row's
// memo, so the FP64 divisions run only where the inputs change.  The key
// being compared is in registers; the previous key and the memo live in the
// thread's shared-memory slots, which a miss hands to mom_row.
__global__ void __launch_bounds__(ASM_NT, 4) k_mom_assemble(MomDev in, MomParams o, int comp, Dims d, MomSys S,
                                                         int want32, int kz)
{
    __shared__ double sprev[NKEY][ASM_NT];
    __shared__ double smemo[NMEMO][ASM_NT];
    __shared__ int skb[ASM_NT];
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k0 = blockIdx.z * kz + 1, k1 = min(k0 + kz - 1, d.K);
    if (i > d.I || j > d.J) return;
    const int iu = comp == 1, iv = comp == 2, iw = comp == 3;
    const int ie = d.I - iu, je = d.J - iv, ke = d.K - iw;
    const bool col_in = i <= ie && j <= je;
    const int ibase = (i == 1 ? 1 : 0) | (i == ie ? 2 : 0) | (j == 1 ? 4 : 0) | (j == je ? 8 : 0);
    const long long sns = d.I, stb = (long long)d.I * d.J;
    const long long px = ie, pxy = (long long)ie * je;
    double mm[6], minv = 0.0, mdp = 0.0, mg = 0.0, mcb[6];
    float mf[6];   // the FP32 copies of mm
#pragma unroll
    for (int q = 0; q < 6; ++q) { mm[q] = mcb[q] = 0.0; mf[q] = 0.f; }
    bool have = false;
    for (int k = k0; k <= k1; ++k) {
        const long long c = gidx(d, i, j, k);
        const long long n = (i - 1) + (long long)d.I * ((j - 1) + (long long)d.J * (k - 1));
        double mw = 0.0, ms = 0.0, mb = 0.0, me = 0.0, mn = 0.0, mt = 0.0, bh = 0.0;
        float fw = 0.f, fs = 0.f, fb = 0.f, fe = 0.f, fn = 0.f, ft = 0.f;
        if (col_in && k <= ke) {
            double dpv = 0.0;
            if (in.cell_type[n] != 2) {
                const long long few = i + (long long)(d.I + 2) * ((j - 1) + (long long)d.J * (k - 1));
                const long long fns = (i - 1) + (long long)d.I * (j + (long long)(d.J + 2) * (k - 1));
                const long long ftb = (i - 1) + (long long)d.I * ((j - 1) + (long long)d.J * k);
                double v[NKEY];
                v[KDFE] = in.df_ew[few + 1]; v[KDFW] = in.df_ew[few];
                v[KDFN] = in.df_ns[fns + sns]; v[KDFS] = in.df_ns[fns];
                v[KDFT] = in.df_tb[ftb + stb]; v[KDFB] = in.df_tb[ftb];
                v[KEE] = in.edf_ew[few + 1]; v[KEW] = in.edf_ew[few];
                v[KEN] = in.edf_ns[fns + sns]; v[KES] = in.edf_ns[fns];
                v[KET] = in.edf_tb[ftb + stb]; v[KEB] = in.edf_tb[ftb];
                v[KETAE] = in.eta_e[c]; v[KETAW] = in.eta_e[c - 1];
                v[KETAN] = in.eta_n[c]; v[KETAS] = in.eta_n[c - d.sy];
                v[KETAT] = in.eta_t[c]; v[KETAB] = in.eta_t[c - d.sz];
                v[KVOF] = in.vof[c]; v[KVOFL] = in.vofl[c];
                v[KDX] = in.dx[n]; v[KDY] = in.dy[n]; v[KDZ] = in.dz[n];
                v[KFRIC] = in.fric[n];
                const int kb = ibase | (k == 1 ? 16 : 0) | (k == ke ? 32 : 0);
                bool hit = have && skb[tid] == kb;
#pragma unroll
                for (int q = 0; q < NKEY; ++q)
                    hit &= __double_as_longlong(v[q]) == __double_as_longlong(sprev[q][tid]);
                if (!hit) {
#pragma unroll
                    for (int q = 0; q < NKEY; ++q) sprev[q][tid] = v[q];
                    skb[tid] = kb;
                    mom_row(&sprev[0][tid], o, comp, kb, &smemo[0][tid]);
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        mm[q] = smemo[MW + q][tid];
                        mcb[q] = smemo[MCW + q][tid];
                        mf[q] = (float)mm[q];
                    }
                    minv = smemo[MINV][tid]; mdp = smemo[MDP][tid]; mg = smemo[MG][tid];
                    have = true;
                }
                dpv = mdp;
                // SetVectors: u.vof.dV/dt - u.dV.dvof/dt + gravity - flux +
                // boundary values, in the reference's order
                const double vof = v[KVOF], dx = v[KDX], dy = v[KDY], dz = v[KDZ];
                const double U = in.tvar[c] + 0.0;
                const double dv = vof - in.vof_old[c];
                const double t1 = U * vof * dx * dy * dz / o.dt;
                const double t2 = dv == 0.0 ? U * dv * dx * dy * dz : U * dv * dx * dy * dz / o.dt;
                double rhs = t1 - t2 + mg;
                rhs = rhs - in.flux_div[n];
                if (kb & 1) rhs = rhs + mcb[0] * in.bc[0][(j - 1) + (long long)d.J * (k - 1)];
                if (kb & 2) rhs = rhs + mcb[1] * in.bc[1][(j - 1) + (long long)d.J * (k - 1)];
                if (kb & 4) rhs = rhs + mcb[2] * in.bc[2][(i - 1) + (long long)d.I * (k - 1)];
                if (kb & 8) rhs = rhs + mcb[3] * in.bc[3][(i - 1) + (long long)d.I * (k - 1)];
                if (kb & 16) rhs = rhs + mcb[4] * in.bc[4][(i - 1) + (long long)d.I * (j - 1)];
                if (kb & 32) rhs = rhs + mcb[5] * in.bc[5][(i - 1) + (long long)d.I * (j - 1)];
                // a neighbour couples when it is inside the loop range and
                // numbered (PosNu /= -1, 1044-1097)
                const long long pn = (i - 1) + px * (j - 1) + pxy * (k - 1);
                if (i > 1 && in.posnu[pn - 1] != -1) { mw = mm[0]; fw = mf[0]; }
                if (j > 1 && in.posnu[pn - px] != -1) { ms = mm[1]; fs = mf[1]; }
                if (k > 1 && in.posnu[pn - pxy] != -1) { mb = mm[2]; fb = mf[2]; }
                if (i < ie && in.posnu[pn + 1] != -1) { me = mm[3]; fe = mf[3]; }
                if (j < je && in.posnu[pn + px] != -1) { mn = mm[4]; fn = mf[4]; }
                if (k < ke && in.posnu[pn + pxy] != -1) { mt = mm[5]; ft = mf[5]; }
                bh = rhs * minv;
            }
            S.dp[c] = dpv;
        }
        S.m[0][c] = mw; S.m[1][c] = ms; S.m[2][c] = mb;
        S.m[3][c] = me; S.m[4][c] = mn; S.m[5][c] = mt;
        S.b[c] = bh;
        if (want32) {
            S.m32[0][c] = fw; S.m32[1][c] = fs; S.m32[2][c] = fb;
            S.m32[3][c] = fe; S.m32[4][c] = fn; S.m32[5][c] = ft;
        }
    }
}

}  // namespace

namespace {

// counts[0]: active cells of the loop range; counts[1]: cells of the loop
// range whose PosNu is -1 when active, or not -1 when solid.
__global__ void __launch_bounds__(256) k_mom_numbering(MomDev in, int comp, Dims d, unsigned long long *counts)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
    const int ie = d.I - (comp == 1), je = d.J - (comp == 2), ke = d.K - (comp == 3);
    unsigned act = 0, bad = 0;
    if (i <= ie && j <= je && k <= ke) {
        const bool solid = in.cell_type[(i - 1) + (long long)d.I * ((j - 1) + (long long)d.J * (k - 1))] == 2;
        const int32_t q = in.posnu[(i - 1) + (long long)ie * ((j - 1) + (long long)je * (k - 1))];
        act = !solid;
        bad = solid ? q != -1 : q < 0;
    }
    const unsigned a = __syncthreads_count(act), b = __syncthreads_count(bad);
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
        if (a) atomicAdd(counts, (unsigned long long)a);
        if (b) atomicAdd(counts + 1, (unsigned long long)b);
    }
}

// Dp ghost planes (PredictUVW.f90:766-788), one phase per axis; within a
// phase each line along the axis is copied in the reference's order.
// phase 0: lines along i over (j, k) in [0,J+1]x[0,K+1]; 1: along j; 2: along k.
__global__ void k_dp_phase(double *dp, Dims d, int comp, int phase)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    long long base, s;
    int n;
    if (phase == 0) {
        if (a > d.J + 1) return;
        base = d.sy * a + d.sz * b; s = 1; n = d.I;
    } else if (phase == 1) {
        if (a > d.I + 1) return;
        base = a + d.sz * b; s = d.sy; n = d.J;
    } else {
        if (a > d.I + 1) return;
        base = a + d.sy * b; s = d.sz; n = d.K;
    }
    double *p = dp + base;
    p[0] = p[s];
    if (comp == phase + 1) p[(long long)n * s] = p[(long long)(n - 1) * s];
    p[(long long)(n + 1) * s] = p[(long long)n * s];
}

// PredictorVelocityBoundaryCondition (3796-3894) for the component's own
// axis, then PredictorVelocityInternalCellCondition (3896-3914) on the one
// plane the boundary condition writes inside 1..I (i = I for u, ...); the
// loop-range cells of solid type already hold 0.
__global__ void k_pred_bc(double *pred, MomDev in, Dims d, int comp)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int b = blockIdx.y + 1;
    long long base, s;
    int n, ct_idx;
    const double *varlo, *varhi;
    int flo, fhi;
    long long bidx;
    if (comp == 1) {   // a = j, b = k
        if (a > d.J) return;
        base = d.sy * a + d.sz * b; s = 1; n = d.I;
        bidx = (a - 1) + (long long)d.J * (b - 1);
        varlo = in.bc[0]; varhi = in.bc[1]; flo = in.flag[0]; fhi = in.flag[1];
        ct_idx = (d.I - 1) + d.I * ((a - 1) + d.J * (b - 1));
    } else if (comp == 2) {   // a = i, b = k
        if (a > d.I) return;
        base = a + d.sz * b; s = d.sy; n = d.J;
        bidx = (a - 1) + (long long)d.I * (b - 1);
        varlo = in.bc[2]; varhi = in.bc[3]; flo = in.flag[2]; fhi = in.flag[3];
        ct_idx = (a - 1) + d.I * ((d.J - 1) + d.J * (b - 1));
    } else {   // a = i, b = j
        if (a > d.I) return;
        base = a + d.sy * b; s = d.sz; n = d.K;
        bidx = (a - 1) + (long long)d.I * (b - 1);
        varlo = in.bc[4]; varhi = in.bc[5]; flo = in.flag[4]; fhi = in.flag[5];
        ct_idx = (a - 1) + d.I * ((b - 1) + d.J * (d.K - 1));
    }
    double *p = pred + base;
    p[0] = flo == 1 ? p[s] : varlo[bidx];
    const double vh = varhi[bidx];
    p[(long long)n * s] = fhi == 1 ? p[(long long)(n - 1) * s] : vh;
    p[(long long)(n + 1) * s] = 2.0 * vh - p[(long long)(n - 1) * s];
    if (in.cell_type[ct_idx] == 2) p[(long long)n * s] = 0.0;
}

}  // namespace

void mom_assemble(const MomDev &in, const MomParams &o, int comp, const Dims &d, const MomSys &S, bool want32,
                  cudaStream_t st)
{
    const int kz = 16;
    const dim3 grid((d.I + 31) / 32, (d.J + 3) / 4, (d.K + kz - 1) / kz);
    k_mom_assemble<<<grid, dim3(32, 4, 1), 0, st>>>(in, o, comp, d, S, want32 ? 1 : 0, kz);
}

void mom_check_numbering(const MomDev &in, int comp, const Dims &d, unsigned long long *counts, cudaStream_t st)
{
    k_mom_numbering<<<interior_grid(d), interior_block(), 0, st>>>(in, comp, d, counts);
}

void mom_tail_comp(const MomDev &in, const Dims &d, int c, double *pred, double *dp, cudaStream_t st,
                   int *launches)
{
    k_dp_phase<<<dim3((d.J + 2 + 127) / 128, d.K + 2), 128, 0, st>>>(dp, d, c + 1, 0);
    k_dp_phase<<<dim3((d.I + 2 + 127) / 128, d.K + 2), 128, 0, st>>>(dp, d, c + 1, 1);
    k_dp_phase<<<dim3((d.I + 2 + 127) / 128, d.J + 2), 128, 0, st>>>(dp, d, c + 1, 2);
    if (c == 0) k_pred_bc<<<dim3((d.J + 127) / 128, d.K), 128, 0, st>>>(pred, in, d, 1);
    else if (c == 1) k_pred_bc<<<dim3((d.I + 127) / 128, d.K), 128, 0, st>>>(pred, in, d, 2);
    else k_pred_bc<<<dim3((d.I + 127) / 128, d.J), 128, 0, st>>>(pred, in, d, 3);
    *launches += 4;
}

}  // namespace pred
