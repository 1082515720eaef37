"""The oracle of the momentum predictor's implicit solves (oracle/predictor.c)
against an independent vectorised restatement of SetMatrix/SetVectors
(PredictUVW.f90:856-1292), closed forms, and the rules of DeltaGetValues and
the tail of PredictingUVW.  CPU only."""
import numpy as np
import pytest

from simcoflow3d_gb300 import geometry as GM, predictor as PR
from oracle import oracle as O


def _geo(name="c1", n=16, **kw):
    return O.grid_preprocess(GM.geometry_inputs(name, n=n, **kw))


@pytest.fixture(scope="module")
def sphere():
    return PR.momentum_inputs(_geo("c1", 16), vof_old_noise=0.01)


@np.errstate(divide="ignore", invalid="ignore")
def numpy_rows(inp, opts, comp):
    """SetMatrix + SetVectors of component comp as numpy arrays over the loop
    range (same FP64 operations in the same order): aW..aT, aP, rhs, Dp."""
    I, J, K = inp.imax, inp.jmax, inp.kmax
    iu, iv, iw = comp == 0, comp == 1, comp == 2
    ie, je, ke = I - iu, J - iv, K - iw
    a = inp.comps[comp].arrays
    g = lambda x, di=0, dj=0, dk=0: x[1 + di:1 + di + ie, 1 + dj:1 + dj + je, 1 + dk:1 + dk + ke]
    n = lambda x: x[:ie, :je, :ke]
    CoefEW = float(iu) + float(iv) / 2.0 + float(iw) / 2.0
    CoefNS = float(iu) / 2.0 + float(iv) + float(iw) / 2.0
    CoefTB = float(iu) / 2.0 + float(iv) / 2.0 + float(iw)
    omb = 1.0 - opts.beta_vis
    vof, vofl = g(a["vof"]), g(a["vofl"])
    rho = vofl * opts.rho_w_ref + (vof - vofl) * opts.rho_a_ref
    Dfe = omb * a["df_ew"][2:2 + ie, :je, :ke] / rho
    Dfw = omb * a["df_ew"][1:1 + ie, :je, :ke] / rho
    Dfn = omb * a["df_ns"][:ie, 2:2 + je, :ke] / rho
    Dfs = omb * a["df_ns"][:ie, 1:1 + je, :ke] / rho
    Dft = omb * a["df_tb"][:ie, :je, 2:2 + ke] / rho
    Dfb = omb * a["df_tb"][:ie, :je, 1:1 + ke] / rho
    ee, ew = a["edf_ew"][2:2 + ie, :je, :ke], a["edf_ew"][1:1 + ie, :je, :ke]
    en, es = a["edf_ns"][:ie, 2:2 + je, :ke], a["edf_ns"][:ie, 1:1 + je, :ke]
    et, eb = a["edf_tb"][:ie, :je, 2:2 + ke], a["edf_tb"][:ie, :je, 1:1 + ke]
    etaE, etaW = g(a["eta_e"]), g(a["eta_e"], di=-1)
    etaN, etaS = g(a["eta_n"]), g(a["eta_n"], dj=-1)
    etaT, etaB = g(a["eta_t"]), g(a["eta_t"], dk=-1)
    Fep, Fem = ee * (1.0 - etaE) / rho, ee * etaE / rho
    Fwp, Fwm = ew * etaW / rho, ew * (1.0 - etaW) / rho
    Fnp, Fnm = en * (1.0 - etaN) / rho, en * etaN / rho
    Fsp, Fsm = es * etaS / rho, es * (1.0 - etaS) / rho
    Ftp, Ftm = et * (1.0 - etaT) / rho, et * etaT / rho
    Fbp, Fbm = eb * etaB / rho, eb * (1.0 - etaB) / rho
    fl = inp.comps[comp].bc_flag

    def bnd(sl, flag, coef, *arrs):
        out = []
        for x in arrs:
            x = x.copy()
            x[sl] = 0.0 if flag == 1 else x[sl] * coef
            out.append(x)
        return out

    Dfw, Fwp, Fwm = bnd(np.s_[0, :, :], fl[0], CoefEW, Dfw, Fwp, Fwm)
    Dfe, Fep, Fem = bnd(np.s_[-1, :, :], fl[1], CoefEW, Dfe, Fep, Fem)
    Dfs, Fsp, Fsm = bnd(np.s_[:, 0, :], fl[2], CoefNS, Dfs, Fsp, Fsm)
    Dfn, Fnp, Fnm = bnd(np.s_[:, -1, :], fl[3], CoefNS, Dfn, Fnp, Fnm)
    Dfb, Fbp, Fbm = bnd(np.s_[:, :, 0], fl[4], CoefTB, Dfb, Fbp, Fbm)
    Dft, Ftp, Ftm = bnd(np.s_[:, :, -1], fl[5], CoefTB, Dft, Ftp, Ftm)
    dx, dy, dz = n(a["grid_dx"]), n(a["grid_dy"]), n(a["grid_dz"])
    aE, aW, aN, aS, aT, aB = Dfe, Dfw, Dfn, Dfs, Dft, Dfb
    cw, ce, cs, cn, cb, ct = aW, aE, aS, aN, aB, aT
    aP = vof * dx * dy * dz / opts.dt + aE + aW + aN + aS + aT + aB + n(a["fric"])
    aP = aP + Fep - Fwp + Fnp - Fsp + Ftp - Fbp
    aE, aW, aN, aS, aT, aB = aE - Fem, aW + Fwm, aN - Fnm, aS + Fsm, aT - Ftm, aB + Fbm
    dp = vof * dx * dy * dz * (1.0 / (aP - aE - aW - aN - aS - aT - aB))
    U = g(a["tvar"]) + 0.0
    G3 = opts.gx * float(iu) + opts.gy * float(iv) + opts.gz * float(iw)
    rhs = (U * vof * dx * dy * dz / opts.dt - U * (vof - g(a["vof_old"])) * dx * dy * dz / opts.dt
           + 1.0 / (opts.fr * opts.fr) * vof * dx * dy * dz * G3 / opts.g)
    rhs = rhs - n(a["flux_div"])
    bv = inp.comps[comp].bc_var
    rhs[0, :, :] = rhs[0, :, :] + cw[0, :, :] * bv[0][:je, :ke]
    rhs[-1, :, :] = rhs[-1, :, :] + ce[-1, :, :] * bv[1][:je, :ke]
    rhs[:, 0, :] = rhs[:, 0, :] + cs[:, 0, :] * bv[2][:ie, :ke]
    rhs[:, -1, :] = rhs[:, -1, :] + cn[:, -1, :] * bv[3][:ie, :ke]
    rhs[:, :, 0] = rhs[:, :, 0] + cb[:, :, 0] * bv[4][:ie, :je]
    rhs[:, :, -1] = rhs[:, :, -1] + ct[:, :, -1] * bv[5][:ie, :je]
    return dict(aW=aW, aS=aS, aB=aB, aP=aP, aE=aE, aN=aN, aT=aT, rhs=rhs, dp=dp)


@pytest.mark.parametrize("comp", [0, 1, 2])
def test_rows_match_vectorised_restatement(sphere, comp):
    """CSR values, rhs and Dp of the oracle equal the numpy restatement bit
    for bit (same operations, same order)."""
    inp, opts = sphere, PR.default_opts()
    I, J, K = inp.imax, inp.jmax, inp.kmax
    (rp, ci, va), rhs, dp = O.mom_system(inp, opts, comp)
    R = numpy_rows(inp, opts, comp)
    a = inp.comps[comp].arrays
    ie, je, ke = I - (comp == 0), J - (comp == 1), K - (comp == 2)
    ct = a["cell_type"][:ie, :je, :ke]
    pos = a["posnu"]
    act = ct != 2
    assert np.array_equal(pos == -1, ~act)
    rows = pos[act]
    # diagonal and rhs by row
    diag = np.empty(rhs.size)
    for r in range(rhs.size):
        sel = np.nonzero(ci[rp[r]:rp[r + 1]] == r)[0]
        diag[r] = va[rp[r] + sel[0]]
    assert (diag[rows].view(np.int64) == R["aP"][act].view(np.int64)).all()
    assert (rhs[rows].view(np.int64) == R["rhs"][act].view(np.int64)).all()
    g = dp[1:1 + ie, 1:1 + je, 1:1 + ke]
    assert (g[act].view(np.int64) == R["dp"][act].view(np.int64)).all()
    assert (g[~act] == 0.0).all()
    # off-diagonals: -a_d towards each numbered neighbour, W,S,B,P,E,N,T order
    idx = np.argwhere(act)
    for (i, j, k) in idx[:: max(1, len(idx) // 400)]:
        r = pos[i, j, k]
        want = []
        for key, di, dj, dk, ok in (("aW", -1, 0, 0, i > 0), ("aS", 0, -1, 0, j > 0), ("aB", 0, 0, -1, k > 0),
                                    ("aP", 0, 0, 0, True), ("aE", 1, 0, 0, i < ie - 1),
                                    ("aN", 0, 1, 0, j < je - 1), ("aT", 0, 0, 1, k < ke - 1)):
            if not ok:
                continue
            q = pos[i + di, j + dj, k + dk]
            if key == "aP":
                want.append((r, R["aP"][i, j, k]))
            elif q != -1:
                want.append((q, -R[key][i, j, k]))
        got = list(zip(ci[rp[r]:rp[r + 1]], va[rp[r]:rp[r + 1]]))
        assert [w[0] for w in want] == [int(x[0]) for x in got]
        assert np.array_equal(np.array([w[1] for w in want]).view(np.int64),
                              np.array([x[1] for x in got]).view(np.int64))


def test_diagonal_system_closed_form():
    """No viscosity, no cut-cell terms, no friction: the rows are diagonal
    and Pred = rhs / (vof dV/dt), Dp = vof dV * (1 / (vof dV/dt))."""
    inp = PR.momentum_inputs(_geo("box", shape=(6, 5, 7), solid=None), rey=1e300, edf=0.0, vof_old_noise=0.0)
    for c in inp.comps:
        c.arrays["fric"][:] = 0.0
    opts = PR.default_opts()
    pred, dp, info = O.predict_solves(inp, opts)
    for comp in range(3):
        a = inp.comps[comp].arrays
        I, J, K = inp.imax, inp.jmax, inp.kmax
        ie, je, ke = I - (comp == 0), J - (comp == 1), K - (comp == 2)
        sl = np.s_[1:1 + ie, 1:1 + je, 1:1 + ke]
        vof = a["vof"][sl]
        aP = vof * a["grid_dx"][:ie, :je, :ke] * a["grid_dy"][:ie, :je, :ke] * a["grid_dz"][:ie, :je, :ke] / opts.dt
        R = numpy_rows(inp, opts, comp)
        assert np.array_equal(R["aP"], aP)
        np.testing.assert_allclose(pred[comp][sl], R["rhs"] / aP, rtol=1e-13, atol=0)
        want = vof * a["grid_dx"][:ie, :je, :ke] * a["grid_dy"][:ie, :je, :ke] * a["grid_dz"][:ie, :je, :ke] * (1.0 / aP)
        assert np.array_equal(dp[comp][sl], want)
        np.testing.assert_allclose(dp[comp][sl], opts.dt, rtol=1e-14)


def test_solution_satisfies_the_rows(sphere):
    opts = PR.default_opts()
    pred, dp, info = O.predict_solves(inp := sphere, opts)
    for comp in range(3):
        A, b, _ = O.mom_system(inp, opts, comp)
        ie, je, ke = inp.imax - (comp == 0), inp.jmax - (comp == 1), inp.kmax - (comp == 2)
        pos = inp.comps[comp].arrays["posnu"]
        x = np.zeros(b.size)
        act = pos >= 0
        x[pos[act]] = pred[comp][1:1 + ie, 1:1 + je, 1:1 + ke][act]
        r = b - O.csr_apply(A, x)
        assert np.linalg.norm(r) <= 1e-13 * np.linalg.norm(b)
        assert info[comp]["iterations"] >= 1


def test_tail_boundary_rules(sphere):
    """Dp ghost planes are copies of the planes next to them (the loop-range
    end plane too), and the velocity BC planes follow
    PredictorVelocityBoundaryCondition."""
    inp, opts = sphere, PR.default_opts()
    rng = np.random.default_rng(5)
    shp = inp.shape_g()
    pred = [np.asfortranarray(rng.normal(size=shp)) for _ in range(3)]
    dp = [np.asfortranarray(rng.normal(size=shp)) for _ in range(3)]
    p0 = [p.copy(order="F") for p in pred]
    O.predict_solves(inp, opts, pred, dp)
    I, J, K = inp.imax, inp.jmax, inp.kmax
    du, dv, dw = dp
    assert np.array_equal(du[I, 1:-1, 1:-1], du[I - 1, 1:-1, 1:-1])
    assert np.array_equal(du[I + 1], du[I]) and np.array_equal(du[0, 1:-1], du[1, 1:-1])
    assert np.array_equal(dv[:, J], dv[:, J - 1]) and np.array_equal(dv[:, J + 1], dv[:, J])
    assert np.array_equal(dw[:, :, K], dw[:, :, K - 1]) and np.array_equal(dw[:, :, 0], dw[:, :, 1])
    u, v, w = pred
    cu = inp.comps[0]
    # u: W, E Dirichlet 0 (walls); the east ghost is 2 VarE - u(I-1)
    assert (u[0, 1:-1, 1:-1] == cu.bc_var[0]).all()
    ct_u = cu.arrays["cell_type"]
    assert (u[I, 1:-1, 1:-1][ct_u[I - 1] != 2] == 0.0).all()
    assert np.array_equal(u[I + 1, 1:-1, 1:-1], 2.0 * cu.bc_var[1] - u[I - 1, 1:-1, 1:-1])
    # entries the reference does not write keep their values
    assert np.array_equal(u[:, 0, :], p0[0][:, 0, :]) and np.array_equal(u[:, :, -1], p0[0][:, :, -1])
    assert np.array_equal(v[0, :, :], p0[1][0, :, :]) and np.array_equal(w[:, 0, :], p0[2][:, 0, :])
    # solid cells are zero in all three
    for c in range(3):
        ct = inp.comps[c].arrays["cell_type"]
        assert (pred[c][1:-1, 1:-1, 1:-1][ct == 2] == 0.0).all()


def test_neumann_bc_copies_the_interior():
    inp = PR.momentum_inputs(_geo("box", shape=(7, 6, 5), solid=None))
    for c in inp.comps:
        c.bc_flag[:] = [1] * 6
    pred, dp, _ = O.predict_solves(inp, PR.default_opts())
    I, J, K = inp.imax, inp.jmax, inp.kmax
    u, v, w = pred
    assert np.array_equal(u[0, 1:-1, 1:-1], u[1, 1:-1, 1:-1])
    assert np.array_equal(u[I, 1:-1, 1:-1], u[I - 1, 1:-1, 1:-1])
    assert np.array_equal(v[1:-1, J, 1:-1], v[1:-1, J - 1, 1:-1])
    assert np.array_equal(w[1:-1, 1:-1, 0], w[1:-1, 1:-1, 1])


def test_get_values_follows_the_running_counter():
    """DeltaGetValues hands out solution values in walk order while PosNu
    matches the counter; a cell with a different PosNu gets 0 (the
    reference's own rule, PredictUVW.f90:1320-1331)."""
    inp = PR.momentum_inputs(_geo("box", shape=(4, 3, 3), solid=None))
    comp = 2
    pos = inp.comps[comp].arrays["posnu"].copy(order="F")
    x = np.arange(1.0, pos.size + 1.0)
    import ctypes as C
    st = inp.comps[comp].struct()
    out = np.zeros(inp.shape_g(), order="F")
    O.lib().oracle_mom_get_values(4, 3, 3, comp + 1, C.byref(st), x.ctypes.data_as(C.POINTER(C.c_double)),
                                  out.ctypes.data_as(C.POINTER(C.c_double)))
    ie, je, ke = 4, 3, 2
    walk = [(i, j, k) for i in range(ie) for j in range(je) for k in range(ke)]
    for q, (i, j, k) in enumerate(walk):
        assert pos[i, j, k] == q
        assert out[i + 1, j + 1, k + 1] == x[q]


def _all_dirichlet(inp, seed=11):
    rng = np.random.default_rng(seed)
    for c in inp.comps:
        c.bc_flag[:] = [0] * 6
        c.bc_var[:] = [np.asfortranarray(rng.normal(size=v.shape)) for v in c.bc_var]
    return inp


@pytest.mark.parametrize("comp", [0, 1, 2])
def test_rows_match_with_dirichlet_faces(comp):
    """All six faces Dirichlet with seeded boundary values: the boundary
    scaling by CoefEW/NS/TB and the CWE/CSN/CBT terms of the rhs agree bit
    for bit with the vectorised restatement."""
    inp = _all_dirichlet(PR.momentum_inputs(_geo("c1", 12), vof_old_noise=0.02, edf=0.5))
    opts = PR.default_opts()
    (rp, ci, va), rhs, dp = O.mom_system(inp, opts, comp)
    R = numpy_rows(inp, opts, comp)
    a = inp.comps[comp].arrays
    I, J, K = inp.imax, inp.jmax, inp.kmax
    ie, je, ke = I - (comp == 0), J - (comp == 1), K - (comp == 2)
    act = a["cell_type"][:ie, :je, :ke] != 2
    rows = a["posnu"][act]
    assert (rhs[rows].view(np.int64) == R["rhs"][act].view(np.int64)).all()
    g = dp[1:1 + ie, 1:1 + je, 1:1 + ke]
    assert (g[act].view(np.int64) == R["dp"][act].view(np.int64)).all()


def test_tiny_grid_solves():
    """The smallest grids the numbering allows still give consistent rows
    and a converged solve."""
    inp = PR.momentum_inputs(_geo("box", shape=(3, 2, 4), solid=None))
    pred, dp, info = O.predict_solves(inp, PR.default_opts())
    assert all(x["rel_residual"] <= 1e-13 for x in info)
    assert np.isfinite(pred[0]).all() and np.isfinite(dp[2]).all()
