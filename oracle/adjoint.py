"""FP64 reference gradient of the projection (test infrastructure only).

Loss (the pressure force on the solid plus the squared divergence of the
corrected velocity):

    J = sum_c g_c p_c + 1/2 sum_{c active} (D u)_c^2

with p the zero-mean pressure of the projection (ProjectionP.f90:33-121),
u the corrected face velocity of ComputePUVW.f90:181-232 before the boundary
routines (the west/south/bottom boundary faces keep u*), and
(D u)_c = dy dz (EE(i) u(i) - EE(i-1) u(i-1)) + dx dz (...) + dx dy (...)
the discrete divergence of SetPoissonVectors (ProjectionP.f90:521-526).

Densities are a per-cell field rho_c; a face between fluid cells a (owner)
and b has the GFM density rho_f = lam*rho_a + (1-lam)*rho_b with
lam = |phiL_a|/(|phiL_a|+|phiL_b|) and coefficient Dp/DGrid * rho_ref/rho_f,
which is the reference's coefficient (ProjectionP.f90:155-235) when rho_c is
the density of the cell's phase.  A face towards a solid cell uses rho_a.

This module restates the forward in numpy on top of the oracle's literal
matrix and solver and derives the gradient with the adjoint equations; it is
the checker of the CUDA adjoint and is itself checked against central finite
differences.  All-Neumann pressure boundaries only.
"""
from __future__ import annotations

import numpy as np

from oracle import oracle as O


def phase(w):
    """1 wet, 2 dry, 0 neither, ghosted (ProjectionP.f90:170-174,212-221)."""
    a = w.arrays
    vofl, vof, phil = a["vofl"], a["vof"], a["phil"]
    e = 1.0e-3
    wet = ((vofl >= 0.5) & (vof > 1 - e)) | ((phil < 0) & (vof <= 1 - e) & (vof > e))
    dry = ((vofl < 0.5) & (vof > 1 - e)) | ((phil >= 0) & (vof <= 1 - e) & (vof > e))
    return np.where(wet, 1, np.where(dry, 2, 0))


def phase_density(w):
    ph = phase(w)
    return np.asfortranarray(np.where(ph == 1, w.rho_l, np.where(ph == 2, w.rho_g, w.rho_l)).astype(np.float64))


_OFF = [(-1, 0, 0), (0, -1, 0), (0, 0, -1), (1, 0, 0), (0, 1, 0), (0, 0, 1)]


def _faces(w):
    """Per face direction f: Dp/DGrid ratio at each interior cell (I,J,K)."""
    a = w.arrays
    I, J, K = w.imax, w.jmax, w.kmax
    out = []
    for f, (di, dj, dk) in enumerate(_OFF):
        dp = {0: a["dp_u"], 1: a["dp_v"], 2: a["dp_w"]}[f % 3]
        dg = {0: a["ugrid_dx"], 1: a["vgrid_dy"], 2: a["wgrid_dz"]}[f % 3]
        minus = f < 3
        ii = np.arange(1, I + 1) - (1 if (minus and di) else 0)
        jj = np.arange(1, J + 1) - (1 if (minus and dj) else 0)
        kk = np.arange(1, K + 1) - (1 if (minus and dk) else 0)
        dpv = dp[np.ix_(ii, jj, kk)]
        dgv = dg[np.ix_(np.maximum(ii, 1) - 1, np.maximum(jj, 1) - 1, np.maximum(kk, 1) - 1)]
        out.append(dpv / dgv)
    return out


def pocoef_rho(w, rho, rho_ref=None, tol=1.0e-30):
    """Face coefficients (I,J,K,6) with per-cell densities, and the face
    densities/lambdas used for the derivative."""
    a = w.arrays
    I, J, K = w.imax, w.jmax, w.kmax
    rho_ref = rho_ref or w.rho_l
    ph = phase(w)
    phil = a["phil"]
    ratios = _faces(w)
    pc = np.zeros((I, J, K, 6), order="F")
    lam_all = np.zeros((I, J, K, 6))
    rf_all = np.ones((I, J, K, 6))
    c = (slice(1, I + 1), slice(1, J + 1), slice(1, K + 1))
    for f, (di, dj, dk) in enumerate(_OFF):
        n = (slice(1 + di, I + 1 + di), slice(1 + dj, J + 1 + dj), slice(1 + dk, K + 1 + dk))
        pcv, pnv = ph[c], ph[n]
        lam = np.abs(phil[c]) / (np.abs(phil[c]) + np.abs(phil[n]) + tol)
        lam = np.where(pnv == 0, 1.0, lam)
        rf = lam * rho[c] + (1 - lam) * rho[n]
        v = ratios[f] * rho_ref / rf
        pc[..., f] = np.where(pcv == 0, 0.0, v)
        lam_all[..., f] = lam
        rf_all[..., f] = rf
    # boundary planes copy the neighbouring plane (ProjectionP.f90:256-264)
    pc[0, :, :, 0] = pc[1, :, :, 0]; pc[-1, :, :, 3] = pc[-2, :, :, 3]
    pc[:, 0, :, 1] = pc[:, 1, :, 1]; pc[:, -1, :, 4] = pc[:, -2, :, 4]
    pc[:, :, 0, 2] = pc[:, :, 1, 2]; pc[:, :, -1, 5] = pc[:, :, -2, 5]
    return pc, lam_all, rf_all


def _masks(w):
    a = w.arrays
    return [(a[m] != 1) & (a[t] != 2) for m, t in (("ucell_moexcell", "ucell_cell_type"),
                                                   ("vcell_moexcell", "vcell_cell_type"),
                                                   ("wcell_moexcell", "wcell_cell_type"))]


def _area_faces(w):
    """a_f for the E/N/T face of every interior cell and for face 0."""
    a = w.arrays
    dx, dy, dz = a["pgrid_dx"], a["pgrid_dy"], a["pgrid_dz"]
    EE, NE, TE = a["eearea"], a["nearea"], a["tearea"]
    aE = dy * dz * EE[1:-1, 1:-1, 1:-1]
    aW = dy * dz * EE[:-2, 1:-1, 1:-1]
    aN = dx * dz * NE[1:-1, 1:-1, 1:-1]
    aS = dx * dz * NE[1:-1, :-2, 1:-1]
    aT = dx * dy * TE[1:-1, 1:-1, 1:-1]
    aB = dx * dy * TE[1:-1, 1:-1, :-2]
    return (aW, aS, aB, aE, aN, aT)


def forward(w, rho, g, rel_tol=1e-13):
    """Returns J and the intermediate fields."""
    if any(f == 0 for f in w.bcp_flag):
        raise ValueError("adjoint: all-Neumann pressure boundaries only")
    a = w.arrays
    I, J, K = w.imax, w.jmax, w.kmax
    pc, lam, rf = pocoef_rho(w, rho)
    A = O.csr(w, pc)
    b = O.rhs(w, pc)
    x, its, rr = O.csr_pcg(A, b, tol=rel_tol, singular_=True)
    pp = O.scatter(w, x)
    p = pp[1:-1, 1:-1, 1:-1]
    act = a["cell_type"] != 2
    mU, mV, mW = _masks(w)
    aW, aS, aB, aE, aN, aT = _area_faces(w)
    us, vs, ws = a["u_star"], a["v_star"], a["w_star"]
    # corrected velocities at the upper face of each interior cell
    u = np.where(mU, us[1:-1, 1:-1, 1:-1] - (pp[2:, 1:-1, 1:-1] - p) * pc[..., 3], 0.0)
    v = np.where(mV, vs[1:-1, 1:-1, 1:-1] - (pp[1:-1, 2:, 1:-1] - p) * pc[..., 4], 0.0)
    ww = np.where(mW, ws[1:-1, 1:-1, 1:-1] - (pp[1:-1, 1:-1, 2:] - p) * pc[..., 5], 0.0)
    # lower faces: the neighbour's upper face, or u* on face 0
    um = np.concatenate([us[0:1, 1:-1, 1:-1], u[:-1]], axis=0)
    vm = np.concatenate([vs[1:-1, 0:1, 1:-1], v[:, :-1]], axis=1)
    wm = np.concatenate([ws[1:-1, 1:-1, 0:1], ww[:, :, :-1]], axis=2)
    r = (aE * u - aW * um) + (aN * v - aS * vm) + (aT * ww - aB * wm)
    r = np.where(act, r, 0.0)
    Jv = float(np.sum(g * p) + 0.5 * np.sum(r * r))
    return Jv, dict(pc=pc, lam=lam, rf=rf, A=A, b=b, x=x, pp=pp, p=p, r=r, u=u, v=v, w=ww, act=act,
                    masks=(mU, mV, mW), areas=(aW, aS, aB, aE, aN, aT))


def _upper(arr, axis):
    """Value at the +1 neighbour (zero beyond the last cell)."""
    out = np.zeros_like(arr)
    sl_dst = [slice(None)] * 3
    sl_src = [slice(None)] * 3
    sl_dst[axis] = slice(0, -1)
    sl_src[axis] = slice(1, None)
    out[tuple(sl_dst)] = arr[tuple(sl_src)]
    return out


def gradient(w, rho, g, rel_tol=1e-13):
    """J, dJ/du*, dJ/dv*, dJ/dw* (ghosted, face-indexed like u*), dJ/drho
    (ghosted, interior values) by the adjoint."""
    Jv, F = forward(w, rho, g, rel_tol)
    pc, lam, rf, p, r, act = F["pc"], F["lam"], F["rf"], F["p"], F["r"], F["act"]
    aW, aS, aB, aE, aN, aT = F["areas"]
    masks = F["masks"]
    aU = (aE, aN, aT)
    I, J, K = w.imax, w.jmax, w.kmax
    # adjoint rhs: P g + A_m r  (masked face weights of the correction)
    s = np.where(act, g, 0.0)
    s = np.where(act, s - s[act].mean(), 0.0)
    for ax in range(3):
        wf = masks[ax] * pc[..., 3 + ax] * aU[ax]
        rn = _upper(r, ax)
        flux = wf * (r - rn)
        # interior faces only (the last upper face is a Neumann boundary)
        sl = [slice(None)] * 3
        sl[ax] = slice(-1, None)
        flux[tuple(sl)] = 0.0
        s += flux
        lower = np.zeros_like(flux)
        sl_dst = [slice(None)] * 3
        sl_src = [slice(None)] * 3
        sl_dst[ax] = slice(1, None)
        sl_src[ax] = slice(0, -1)
        lower[tuple(sl_dst)] = flux[tuple(sl_src)]
        s -= lower
    s = np.where(act, s, 0.0)
    pos = w.arrays["posnu"]
    sv = np.zeros(w.ext_cell + 1)
    sv[pos[act]] = s[act]
    lv, its, rr = O.csr_pcg(F["A"], sv, tol=rel_tol, singular_=True)
    lmb = np.zeros((I, J, K))
    lmb[act] = lv[pos[act]]
    # gradients with respect to u*: face-indexed ghosted arrays
    grads = []
    ustar = ("u_star", "v_star", "w_star")
    lower_area = (aW, aS, aB)
    for ax in range(3):
        gg = np.zeros(w.shape_g, order="F")
        rn = _upper(r, ax)
        ln = _upper(lmb, ax)
        m = masks[ax]
        # upper face of each interior cell: direct term (masked) minus b term
        direct = m * aU[ax] * (r - rn)
        via_b = aU[ax] * (lmb - ln)
        sl = [slice(1, -1)] * 3
        gg[tuple(sl)] = direct - via_b
        # face 0 (west/south/bottom boundary): u* enters u and b unmodified
        sl0 = [slice(1, -1)] * 3
        sl0[ax] = slice(0, 1)
        first = [slice(None)] * 3
        first[ax] = slice(0, 1)
        gg[tuple(sl0)] = (-lower_area[ax][tuple(first)] * r[tuple(first)]
                          + lower_area[ax][tuple(first)] * lmb[tuple(first)])
        grads.append(gg)
    # gradients with respect to the face coefficients (E/N/T faces)
    grho = np.zeros((I, J, K))
    for ax in range(3):
        f = 3 + ax
        pn = _upper(p, ax)
        rn = _upper(r, ax)
        ln = _upper(lmb, ax)
        inner = np.ones((I, J, K), dtype=bool)
        sl = [slice(None)] * 3
        sl[ax] = slice(-1, None)
        inner[tuple(sl)] = False
        gcoef = np.where(inner, -aU[ax] * (lmb - ln) * (p - pn) - masks[ax] * aU[ax] * (r - rn) * (pn - p), 0.0)
        # coef = ratio*rho_ref/rho_f, rho_f = lam*rho_c + (1-lam)*rho_n
        dcoef = -pc[..., f] / rf[..., f]
        grho += gcoef * dcoef * lam[..., f]
        contrib = gcoef * dcoef * (1 - lam[..., f])
        sl_dst = [slice(None)] * 3
        sl_src = [slice(None)] * 3
        sl_dst[ax] = slice(1, None)
        sl_src[ax] = slice(0, -1)
        grho[tuple(sl_dst)] += contrib[tuple(sl_src)]
    grho_g = np.zeros(w.shape_g, order="F")
    grho_g[1:-1, 1:-1, 1:-1] = np.where(act, grho, 0.0)
    return Jv, grads, grho_g
