"""CPU tests of the oracle: known answers, invariants, literal restatements.

The reference (Fortran + MPI + HYPRE) cannot run here and its own tests pin
no values on this path, so the oracle is pinned by (1) exact discrete
eigenmodes of the uniform operator, (2) the closed-form GFM pressure of a
stratified column, (3) independent pure-Python restatements of the
coefficient loop and the boundary routines, (4) symmetry and discrete
divergence invariants, and (5) committed golden fixtures.
"""
import math
import os

import numpy as np
import pytest

from simcoflow3d_gb300 import workloads as W
from oracle import oracle as O

from literal import pocoef_literal, bc_var_new_literal

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _vec(w, field):
    pos = w.arrays["posnu"]
    act = pos >= 0
    out = np.zeros(w.ext_cell + 1)
    out[pos[act]] = field[1:-1, 1:-1, 1:-1][act]
    return out


def test_uniform_operator_eigenmodes():
    """One phase (rho_l = rho_g), no solid, all-Neumann: the reference's
    matrix is dt*h times the graph Laplacian, whose eigenvectors are products
    of cosines; A v = lambda v to rounding."""
    n = 12
    w = W.build_workload("uni", n, n, n, liquid=W._surface(0.5, 0.0, None), rho_l=1.0, rho_g=1.0)
    pc = O.pocoef(w, rho_ref=1.0)
    A = O.csr(w, pc)
    h, dt = 1.0 / n, w.dt
    i = np.arange(1, n + 1) - 0.5
    for (a, b, c) in [(1, 0, 0), (2, 3, 1), (5, 5, 7)]:
        v = (np.cos(math.pi * a * i / n)[:, None, None] * np.cos(math.pi * b * i / n)[None, :, None]
             * np.cos(math.pi * c * i / n)[None, None, :])
        vg = np.zeros(w.shape_g, order="F")
        vg[1:-1, 1:-1, 1:-1] = v
        lam = dt * h * sum(2.0 * (1.0 - math.cos(math.pi * m / n)) for m in (a, b, c))
        y = O.csr_apply(A, _vec(w, vg))
        assert np.abs(y - lam * _vec(w, vg)).max() <= 1e-12 * lam
    # and the solve recovers a mode from its image
    v = _vec(w, vg)
    b = O.csr_apply(A, v)
    x, its, rr = O.csr_pcg(A, b, tol=1e-13, singular_=True)
    assert np.abs(x - (v - v.mean())).max() <= 1e-9


def _beta(pc, pn, lam, bp, bm):
    if pc == 1:
        return lam * bm + (1 - lam) * bp if pn == 2 else bm
    return lam * bp + (1 - lam) * bm if pn == 1 else bp


def test_stratified_column_closed_form():
    """Planar interface z=0.5 between cell centres, liquid below, Dirichlet
    p=0 on top, w* = W0 inside: the corrected flux is zero, so the face
    pressure jumps are W0/c_k with the GFM face coefficients c_k, and
    p_k = -W0 * sum_{m>=k} 1/c_m (series conductances of the two phases)."""
    I = J = 4
    K = 32
    w = W.build_workload("col", I, J, K, liquid=W._surface(0.5, 0.0, None), rho_l=1000.0, rho_g=1.2,
                         bcp_flag=(1, 1, 1, 1, 1, 0))
    a = w.arrays
    W0 = 0.05
    a["u_star"][...] = 0.0
    a["v_star"][...] = 0.0
    a["w_star"][...] = 0.0
    a["w_star"][:, :, 1:K + 1] = W0
    ref = O.project(w, solver="csr", rel_tol=1e-14)
    pp = ref["pp"]
    # independent face coefficients of the column (uniform h, Dp = dt)
    h, dt = 1.0 / K, w.dt
    bp, bm = 1.0, 1000.0 / 1.2
    phil = a["phil"][2, 2, :]
    ph = [1 if z < 0.5 else 2 for z in (np.arange(K) + 0.5) * h]
    c = np.zeros(K + 1)  # c[k]: face between k and k+1 (1-based cells)
    for k in range(1, K):
        pc, pn = ph[k - 1], ph[k]
        lam = abs(phil[k]) / (abs(phil[k]) + abs(phil[k + 1]) + 1e-30)
        c[k] = (dt / h) * bp * bm / _beta(pc, pn, lam, bp, bm)
    c[K] = c[K - 1]          # top boundary face copies its neighbour plane
    pk = np.array([-W0 * sum(1.0 / c[m] for m in range(k, K + 1)) for k in range(1, K + 1)])
    got = pp[2, 2, 1:K + 1]
    assert np.abs(got - pk).max() <= 1e-8 * np.abs(pk).max()
    # pressure gradient is ~rho_l/rho_g times steeper in the liquid
    assert (pk[1] - pk[0]) / (pk[-1] - pk[-2]) > 800
    # corrected w vanishes inside the column
    assert np.abs(ref["w"][1:-1, 1:-1, 1:K]).max() <= 1e-8 * W0


@pytest.mark.parametrize("name,n,stale", [("c1", 8, float("nan")), ("c2", 10, float("nan"))])
def test_pocoef_matches_literal_restatement(name, n, stale):
    w = W.config(name, n=n)
    assert np.array_equal(O.pocoef(w, stale_init=stale), pocoef_literal(w, stale_init=stale), equal_nan=True)


def test_pocoef_carry_matches_literal_restatement():
    """A solid wall at i=1: W coefficients of the i=2 cells come from the
    uninitialised BetaW; cells beside the sphere carry earlier values."""
    w = W.build_workload("wall", 6, 5, 9, solid=("xslab", 0.2), liquid=W._surface(0.5, 0.02, None),
                         rho_l=1000.0, rho_g=1.2)
    for init in (1.0, 3.0, float("nan")):
        ref = pocoef_literal(w, stale_init=init)
        got = O.pocoef(w, stale_init=init)
        assert np.array_equal(got, ref, equal_nan=True)
    assert not np.array_equal(O.pocoef(w, stale_init=1.0), O.pocoef(w, stale_init=3.0))


def test_bcs_match_literal_restatement():
    rng = np.random.default_rng(3)
    w = W.config("c1", n=7, random_tvar=True)
    w.bcu_flag, w.bcv_flag, w.bcw_flag = (1, 0, 1, 0, 1, 0), (0, 1, 0, 1, 0, 1), (1, 1, 0, 0, 1, 1)
    w.bcp_flag = (1, 1, 1, 1, 1, 1)
    for key in ("bcu_const", "bcv_const", "bcw_const", "bcp_const"):
        setattr(w, key, tuple(rng.normal(0, 0.1, 6)))
    pc = O.pocoef(w)
    pp = np.asfortranarray(rng.normal(size=w.shape_g))
    u, v, ww, p, bc, rc = O.correct(w, pc, pp)
    # the correction loop first (ComputePUVW.f90:181-232), then BCs literally
    I, J, K = w.imax, w.jmax, w.kmax
    a = w.arrays
    lu, lv, lw, lp = (a[k].copy(order="F") for k in ("tvar_u", "tvar_v", "tvar_w", "tvar_p"))
    for i in range(1, I + 1):
        for j in range(1, J + 1):
            for k in range(1, K + 1):
                n = (i - 1, j - 1, k - 1)
                lu[i, j, k] = (a["u_star"][i, j, k] - (pp[i + 1, j, k] - pp[i, j, k]) * pc[n + (3,)]
                               if a["ucell_moexcell"][n] != 1 and a["ucell_cell_type"][n] != 2 else 0.0)
                lv[i, j, k] = (a["v_star"][i, j, k] - (pp[i, j + 1, k] - pp[i, j, k]) * pc[n + (4,)]
                               if a["vcell_moexcell"][n] != 1 and a["vcell_cell_type"][n] != 2 else 0.0)
                lw[i, j, k] = (a["w_star"][i, j, k] - (pp[i, j, k + 1] - pp[i, j, k]) * pc[n + (5,)]
                               if a["wcell_moexcell"][n] != 1 and a["wcell_cell_type"][n] != 2 else 0.0)
                lp[i, j, k] = pp[i, j, k]
    lbc = bc_var_new_literal(w, lu, lv, lw, lp)
    for x, y in ((u, lu), (v, lv), (ww, lw), (p, lp)):
        assert np.array_equal(x, y)
    for f in range(4):
        for q in range(6):
            assert np.array_equal(bc[f][q], lbc[f][q])


def test_matrix_symmetric_and_dominant():
    w = W.config("c1", n=14)
    pc = O.pocoef(w)
    rp, ci, va, bad = O.csr(w, pc)
    assert bad == 0
    n = rp.size - 1
    ent = {}
    for r in range(n):
        for e in range(rp[r], rp[r + 1]):
            ent[(r, int(ci[e]))] = va[e]
    for (r, c), v in ent.items():
        assert abs(v - ent[(c, r)]) <= 1e-15 * abs(v) + 1e-300


def test_divergence_free_after_correction():
    """Corrected fluxes of every active cell whose six faces are corrected
    (no solid/MoEx velocity cell, no domain boundary) sum to ~0."""
    w = W.config("c1", n=16)
    ref = O.project(w, rel_tol=1e-13)
    a = w.arrays
    I, J, K = w.imax, w.jmax, w.kmax
    u, v, ww = ref["u"], ref["v"], ref["w"]
    EE, NE, TE = a["eearea"], a["nearea"], a["tearea"]
    h = 1.0 / I
    worst, scale, checked = 0.0, np.abs(ref["b"]).max(), 0
    for i in range(2, I):
        for j in range(2, J):
            for k in range(2, K):
                if a["cell_type"][i - 1, j - 1, k - 1] == 2:
                    continue
                ok = all(a[key][idx] != 1 and a[key2][idx] != 2 for key, key2, idx in (
                    ("ucell_moexcell", "ucell_cell_type", (i - 1, j - 1, k - 1)),
                    ("ucell_moexcell", "ucell_cell_type", (i - 2, j - 1, k - 1)),
                    ("vcell_moexcell", "vcell_cell_type", (i - 1, j - 1, k - 1)),
                    ("vcell_moexcell", "vcell_cell_type", (i - 1, j - 2, k - 1)),
                    ("wcell_moexcell", "wcell_cell_type", (i - 1, j - 1, k - 1)),
                    ("wcell_moexcell", "wcell_cell_type", (i - 1, j - 1, k - 2))))
                if not ok:
                    continue
                div = h * h * ((EE[i, j, k] * u[i, j, k] - EE[i - 1, j, k] * u[i - 1, j, k]) +
                               (NE[i, j, k] * v[i, j, k] - NE[i, j - 1, k] * v[i, j - 1, k]) +
                               (TE[i, j, k] * ww[i, j, k] - TE[i, j, k - 1] * ww[i, j, k - 1]))
                worst = max(worst, abs(div))
                checked += 1
    assert checked > 1000
    assert worst <= 1e-9 * scale


def test_cpu_multigrid_matches_literal_system():
    for name, n in (("c0", 12), ("c1", 14), ("c4", 8)):
        w = W.config(name, n=n)
        ref = O.project(w, solver="csr", rel_tol=1e-13)
        x, st = O.gmg_solve(w, ref["pocoef"], ref["b"], rel_tol=1e-12)
        assert O.csr_relres(ref["A"], ref["b"], x, ref["singular"]) <= 1.1e-12
        d = x - ref["x"]
        if ref["singular"]:
            d -= d.mean()
        assert np.linalg.norm(d) <= 1e-7 * np.linalg.norm(ref["x"])
        xm, sm = O.gmg_solve(w, ref["pocoef"], ref["b"], rel_tol=1e-8, precision=1)
        assert sm["rel_residual"] <= 1e-8 and abs(sm["iterations"] - O.gmg_solve(
            w, ref["pocoef"], ref["b"], rel_tol=1e-8)[1]["iterations"]) <= 2


def test_north_mass_correction_undefined():
    w = W.config("c1", n=8)
    w.bcp_flag = (1, 1, 1, 0, 1, 1)
    pc = O.pocoef(w)
    pp = np.zeros(w.shape_g, order="F")
    assert O.correct(w, pc, pp)[5] == 7
    assert O.correct(w, pc, pp, north_mass_fix=1)[5] == 0


@pytest.mark.parametrize("case", ["c1_12_quirks", "c4_8_dirichlet_top"])
def test_golden_fixtures(case):
    from golden.make_golden import build_case
    w = build_case(case)
    g = np.load(os.path.join(GOLDEN, f"{case}.npz"))
    pc = O.pocoef(w)
    assert np.array_equal(pc, g["pocoef"], equal_nan=True)
    b = O.rhs(w, pc)
    assert np.array_equal(b, g["rhs"])
    ref = O.project(w, solver="csr", rel_tol=1e-13)
    d = ref["x"] - g["x"]
    if ref["singular"]:
        d -= d.mean()
    assert np.abs(d).max() <= 1e-8 * np.abs(g["x"]).max()
    for key in ("u", "v", "w"):
        assert np.abs(ref[key] - g[key]).max() <= 1e-8 * max(1.0, np.abs(g[key]).max())
