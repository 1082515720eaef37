"""Pure-Python literal restatements of small pieces of the reference, used
only to pin the C oracle (independent code, same loops and statements).

Indices follow the Fortran: arrays are accessed with the reference's own
(i, j, k) bounds through small accessor helpers.
"""
import math

import numpy as np


def pocoef_literal(w, stale_init=float("nan"), epsi=1.0e-3, tol=1.0e-30):
    """Compute1DGFMCoefficient x6 (ProjectionP.f90:123-265), statement by
    statement, returning PoCoef (I,J,K,6)."""
    I, J, K = w.imax, w.jmax, w.kmax
    a = w.arrays
    phil, vofl, vof = a["phil"], a["vofl"], a["vof"]
    row = w.rho_l
    betap = 1.0 / (w.rho_l / row)
    betam = 1.0 / (w.rho_g / row)
    out = np.zeros((I, J, K, 6), order="F")
    calls = [(a["dp_u"], a["ugrid_dx"], 1, 0, 0, 0, 0, 0), (a["dp_v"], a["vgrid_dy"], 0, 1, 0, 0, 0, 0),
             (a["dp_w"], a["wgrid_dz"], 0, 0, 1, 0, 0, 0), (a["dp_u"], a["ugrid_dx"], 0, 0, 0, 1, 0, 0),
             (a["dp_v"], a["vgrid_dy"], 0, 0, 0, 0, 1, 0), (a["dp_w"], a["wgrid_dz"], 0, 0, 0, 0, 0, 1)]

    def wet(x):
        return (vofl[x] >= 0.5 and vof[x] > 1.0 - epsi) or (phil[x] < 0.0 and vof[x] <= 1.0 - epsi and vof[x] > epsi)

    def dry(x):
        return (vofl[x] < 0.5 and vof[x] > 1.0 - epsi) or (phil[x] >= 0.0 and vof[x] <= 1.0 - epsi and vof[x] > epsi)

    for f, (dp, dg, ium, jvm, kwm, iup, jvp, kwp) in enumerate(calls):
        T = np.zeros((I, J, K))
        betaw = stale_init
        betad = stale_init
        for i in range(1, I + 1):
            for j in range(1, J + 1):
                for k in range(1, K + 1):
                    ii, jj, kk = i - ium + iup, j - jvm + jvp, k - kwm + kwp
                    im, jm, km = i - ium, j - jvm, k - kwm
                    dgrid = dg[max(im, 1) - 1, max(jm, 1) - 1, max(km, 1) - 1]
                    c, n = (i, j, k), (ii, jj, kk)
                    lam = abs(phil[c]) / (abs(phil[c]) + abs(phil[n]) + tol)
                    if wet(c):
                        if dry(n):
                            betaw = lam * betam + (1.0 - lam) * betap
                        elif wet(n):
                            betaw = betam
                        T[i - 1, j - 1, k - 1] = dp[im, jm, km] / dgrid * betap * betam / betaw
                    elif dry(c):
                        if wet(n):
                            betad = lam * betap + (1.0 - lam) * betam
                        elif dry(n):
                            betad = betap
                        T[i - 1, j - 1, k - 1] = dp[im, jm, km] / dgrid * betap * betam / betad
        if ium or iup:
            T[(ium * 1 + iup * I) - 1, :, :] = T[(ium * 2 + iup * (I - 1)) - 1, :, :]
        if jvm or jvp:
            T[:, (jvm * 1 + jvp * J) - 1, :] = T[:, (jvm * 2 + jvp * (J - 1)) - 1, :]
        if kwm or kwp:
            T[:, :, (kwm * 1 + kwp * K) - 1] = T[:, :, (kwm * 2 + kwp * (K - 1)) - 1]
        out[..., f] = T
    return out


def typical_bc(varin_plane, dxyz, flag, const):
    """TypicalBC (BoundaryFunction.f90:760-781) with the Fortran dummy
    argument semantics: Varin is the full ghosted plane section whose lower
    bound becomes 1, so Array(a,b) uses the section element (a,b), i.e. the
    field at in-plane ghosted indices (a-1, b-1)."""
    n1, n2 = dxyz.shape
    out = np.zeros((n1, n2))
    for a_ in range(1, n1 + 1):
        for b_ in range(1, n2 + 1):
            if flag == 0:
                out[a_ - 1, b_ - 1] = const
            else:
                out[a_ - 1, b_ - 1] = varin_plane[a_ - 1, b_ - 1] - const * dxyz[a_ - 1, b_ - 1] / 2.0
    return out


def ghost(flag, varin, bcin):
    """ComputeGhostVarBoundary (ComputePUVW.f90:696-708)."""
    return bcin - varin if flag == 1 else 2.0 * bcin - varin


def bc_var_new_literal(w, u, v, ww, p):
    """BoundaryConditionVarNew (ComputePUVW.f90:418-694) with the TypicalBC
    procedure pointers of the reference drivers; modifies u, v, ww, p in place
    and returns the 24 Var planes (field-major)."""
    I, J, K = w.imax, w.jmax, w.kmax
    a = w.arrays
    dx, dy, dz = a["pgrid_dx"], a["pgrid_dy"], a["pgrid_dz"]
    fu, fv, fw, fp = w.bcu_flag, w.bcv_flag, w.bcw_flag, w.bcp_flag
    cu, cv, cw, cp = w.bcu_const, w.bcv_const, w.bcw_const, w.bcp_const
    out = []
    # U
    VarW = typical_bc(u[1, :, :], dx[0, :, :], fu[0], cu[0]); u[0, 1:J + 1, 1:K + 1] = VarW
    VarE = typical_bc(u[I - 1, :, :], -dx[I - 1, :, :] * 2.0, fu[1], cu[1]); u[I, 1:J + 1, 1:K + 1] = VarE
    u[I + 1, 1:J + 1, 1:K + 1] = ghost(fu[1], u[I, 1:J + 1, 1:K + 1], VarE)
    VarS = typical_bc(u[:, 1, :], dy[:, 0, :], fu[2], cu[2]); u[1:I + 1, 0, 1:K + 1] = ghost(fu[2], u[1:I + 1, 1, 1:K + 1], VarS)
    VarN = typical_bc(u[:, J, :], -dy[:, J - 1, :], fu[3], cu[3]); u[1:I + 1, J + 1, 1:K + 1] = ghost(fu[3], u[1:I + 1, J, 1:K + 1], VarN)
    VarB = typical_bc(u[:, :, 1], dz[:, :, 0], fu[4], cu[4]); u[1:I + 1, 1:J + 1, 0] = ghost(fu[4], u[1:I + 1, 1:J + 1, 1], VarB)
    VarT = typical_bc(u[:, :, K], -dz[:, :, K - 1], fu[5], cu[5]); u[1:I + 1, 1:J + 1, K + 1] = ghost(fu[5], u[1:I + 1, 1:J + 1, K], VarT)
    out.append([VarW, VarE, VarS, VarN, VarB, VarT])
    # V
    VarW = typical_bc(v[1, :, :], dx[0, :, :], fv[0], cv[0]); v[0, 1:J + 1, 1:K + 1] = ghost(fv[0], v[1, 1:J + 1, 1:K + 1], VarW)
    VarE = typical_bc(v[I, :, :], -dx[I - 1, :, :], fv[1], cv[1]); v[I + 1, 1:J + 1, 1:K + 1] = ghost(fv[1], v[I, 1:J + 1, 1:K + 1], VarE)
    VarS = typical_bc(v[:, 1, :], dy[:, 0, :], fv[2], cv[2]); v[1:I + 1, 0, 1:K + 1] = VarS
    VarN = typical_bc(v[:, J - 1, :], -dy[:, J - 1, :] * 2.0, fv[3], cv[3]); v[1:I + 1, J, 1:K + 1] = VarN
    v[1:I + 1, J + 1, 1:K + 1] = ghost(fv[3], v[1:I + 1, J, 1:K + 1], VarN)
    VarB = typical_bc(v[:, :, 1], dz[:, :, 0], fv[4], cv[4]); v[1:I + 1, 1:J + 1, 0] = ghost(fv[4], v[1:I + 1, 1:J + 1, 1], VarB)
    VarT = typical_bc(v[:, :, K], -dz[:, :, K - 1], fv[5], cv[5]); v[1:I + 1, 1:J + 1, K + 1] = ghost(fv[5], v[1:I + 1, 1:J + 1, K], VarT)
    out.append([VarW, VarE, VarS, VarN, VarB, VarT])
    # W
    VarW = typical_bc(ww[1, :, :], dx[0, :, :], fw[0], cw[0]); ww[0, 1:J + 1, 1:K + 1] = ghost(fw[0], ww[1, 1:J + 1, 1:K + 1], VarW)
    VarE = typical_bc(ww[I, :, :], -dx[I - 1, :, :], fw[1], cw[1]); ww[I + 1, 1:J + 1, 1:K + 1] = ghost(fw[1], ww[I, 1:J + 1, 1:K + 1], VarE)
    VarS = typical_bc(ww[:, 1, :], dy[:, 0, :], fw[2], cw[2]); ww[1:I + 1, 0, 1:K + 1] = ghost(fw[2], ww[1:I + 1, 1, 1:K + 1], VarS)
    VarN = typical_bc(ww[:, J, :], -dy[:, J - 1, :], fw[3], cw[3]); ww[1:I + 1, J + 1, 1:K + 1] = ghost(fw[3], ww[1:I + 1, J, 1:K + 1], VarN)
    VarB = typical_bc(ww[:, :, 1], dz[:, :, 0], fw[4], cw[4]); ww[1:I + 1, 1:J + 1, 0] = VarB
    VarT = typical_bc(ww[:, :, K - 1], -dz[:, :, K - 1] * 2.0, fw[5], cw[5]); ww[1:I + 1, 1:J + 1, K] = VarT
    ww[1:I + 1, 1:J + 1, K + 1] = ghost(fw[5], ww[1:I + 1, 1:J + 1, K], VarT)
    out.append([VarW, VarE, VarS, VarN, VarB, VarT])
    # P
    VarW = typical_bc(p[1, :, :], dx[0, :, :], fp[0], cp[0]); p[0, 1:J + 1, 1:K + 1] = ghost(fp[0], p[1, 1:J + 1, 1:K + 1], VarW)
    VarE = typical_bc(p[I, :, :], -dx[I - 1, :, :], fp[1], cp[1]); p[I + 1, 1:J + 1, 1:K + 1] = ghost(fp[1], p[I, 1:J + 1, 1:K + 1], VarE)
    VarS = typical_bc(p[:, 1, :], dy[:, 0, :], fp[2], cp[2]); p[1:I + 1, 0, 1:K + 1] = ghost(fp[2], p[1:I + 1, 1, 1:K + 1], VarS)
    VarN = typical_bc(p[:, J, :], -dy[:, J - 1, :], fp[3], cp[3]); p[1:I + 1, J + 1, 1:K + 1] = ghost(fp[3], p[1:I + 1, J, 1:K + 1], VarN)
    VarB = typical_bc(p[:, :, 1], dz[:, :, 0], fp[4], cp[4]); p[1:I + 1, 1:J + 1, 0] = ghost(fp[4], p[1:I + 1, 1:J + 1, 1], VarB)
    VarT = typical_bc(p[:, :, K], -dz[:, :, K - 1], fp[5], cp[5]); p[1:I + 1, 1:J + 1, K] = VarT
    p[1:I + 1, 1:J + 1, K + 1] = ghost(fp[5], p[1:I + 1, 1:J + 1, K], VarT)
    out.append([VarW, VarE, VarS, VarN, VarB, VarT])
    return out
