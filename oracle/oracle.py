"""Python front end of the oracle (test infrastructure only).

The oracle is the CPU restatement of the SIMCOFlow routines this repository
rebuilds:
- ``oracle.c``: the projection path (coefficients, literal CSR matrix, rhs,
  scatter, correction, boundary conditions), with the CPU
  multigrid-preconditioned CG of ``gmg.cpp``;
- ``geometry.c``: the cut-cell geometry preprocessing;
- ``predictor.c``: the momentum predictor's SetMatrix / SetVectors,
  DeltaGetValues and the tail of PredictingUVW, with a Jacobi BiCGStab;
- ``vtr.py``: the VTK RectilinearGrid writer;
- ``clsvof.c``: the CLSVOF interface transport: Clsvof_Scheme with its
  directional sweeps, Interface_Reconstruct, BoundaryConditionLvsVof and
  Redistance_Levelset, and ComputeUVWLiquidField.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` use it, and only as the checker or the timed CPU path.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from typing import Optional

import numpy as np

from simcoflow3d_gb300 import capi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


def build(quiet: bool = True) -> str:
    subprocess.run(["make", "-C", _HERE], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        dp, ip = capi.c_double_p, capi.c_int32_p
        i64p = C.POINTER(C.c_int64)
        L.oracle_pocoef.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(capi.ScfPoissonIn), C.c_double,
                                    C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, dp]
        L.oracle_matrix_csr.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(capi.ScfPoissonIn), dp, i64p, ip, dp]
        L.oracle_matrix_csr.restype = C.c_int64
        L.oracle_rhs.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(capi.ScfPoissonIn), dp, dp]
        L.oracle_scatter.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(capi.ScfPoissonIn), dp, dp]
        L.oracle_correct.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(capi.ScfPoissonIn),
                                     C.POINTER(capi.ScfCorrectIn), dp, dp, dp, dp, dp, dp, dp, C.c_int]
        L.oracle_grid_preprocess.argtypes = [C.c_int, C.c_int, C.c_int] + [C.POINTER(capi.ScfGeoCells)] * 4
        L.oracle_face_geo_cal.argtypes = [C.c_double] * 7 + [dp, dp]
        L.oracle_csr_apply.argtypes = [C.c_int32, i64p, ip, dp, dp, dp]
        L.oracle_csr_pcg.argtypes = [C.c_int32, i64p, ip, dp, dp, dp, C.c_double, C.c_int, C.c_int,
                                     C.POINTER(C.c_double)]
        L.oracle_csr_relres.argtypes = [C.c_int32, i64p, ip, dp, dp, dp, C.c_int]
        L.oracle_csr_relres.restype = C.c_double
        L.oracle_gmg_solve.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(capi.ScfPoissonIn), dp, dp, dp,
                                       C.POINTER(GmgParams)]
        L.oracle_num_threads.restype = C.c_int
        PM, PO = C.POINTER(capi.ScfMomIn), C.POINTER(capi.ScfMomOpts)
        L.oracle_mom_system.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, PM, PO, i64p, ip, dp, dp, dp]
        L.oracle_mom_system.restype = C.c_long
        L.oracle_csr_bicgstab.argtypes = [C.c_long, i64p, ip, dp, dp, dp, C.c_double, C.c_int,
                                          C.POINTER(C.c_double)]
        L.oracle_csr_bicgstab.restype = C.c_int
        L.oracle_mom_get_values.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, PM, dp, dp]
        L.oracle_predict_tail.argtypes = [C.c_int, C.c_int, C.c_int, PM] + [dp] * 6
        L.oracle_volume_fraction_calc.argtypes = [C.c_double] * 7
        L.oracle_volume_fraction_calc.restype = C.c_double
        L.oracle_convert_coord.argtypes = [C.c_double] * 7
        L.oracle_convert_coord.restype = C.c_double
        DP3 = dp * 3
        L.oracle_uvw_liquid_field.argtypes = [C.c_int, C.c_int, C.c_int] + [dp] * 8 + [DP3] * 9
        L.oracle_find_distance.argtypes = [C.c_double] * 7
        L.oracle_find_distance.restype = C.c_double
        L.oracle_interface_reconstruct.argtypes = [C.c_int, C.c_int, C.c_int] + [dp] * 12
        L.oracle_clsvof_sweep.argtypes = [C.c_int] * 4 + [dp] * 11 + [C.c_double] + [dp] * 6
        L.oracle_clsvof_scheme.argtypes = [C.POINTER(ClsvofArgs)]
        for name in ("oracle_cube_rn", "oracle_pow_third"):
            getattr(L, name).argtypes = [C.c_double]
            getattr(L, name).restype = C.c_double
        L.oracle_clsvof_redistance.argtypes = [C.c_int] * 3 + [dp] * 11
        _lib = L
    return _lib


class ClsvofArgs(C.Structure):
    """struct oracle_clsvof_args (oracle/clsvof.c)."""
    _fields_ = [("imax", C.c_int), ("jmax", C.c_int), ("kmax", C.c_int)] + [
        (n, capi.c_double_p) for n in ("x", "y", "z", "dx", "dy", "dz", "vofl", "phil", "nxl", "nyl", "nzl",
                                       "nx", "ny", "nz", "u", "v", "w")] + [
        ("bc_vel", capi.c_double_p * 3), ("lvs_bc", capi.c_double_p * 6), ("vof_bc", capi.c_double_p * 6),
        ("lvs_flag", C.c_int * 6), ("vof_flag", C.c_int * 6), ("lvs_const", C.c_double * 6),
        ("vof_const", C.c_double * 6), ("dt", C.c_double)]


class GmgParams(C.Structure):
    _fields_ = [
        ("precision", C.c_int), ("rel_tol", C.c_double), ("max_iter", C.c_int), ("max_rounds", C.c_int),
        ("inner_rtol", C.c_double), ("degree", C.c_int), ("ratio", C.c_double), ("coarse_max", C.c_int),
        ("line_seg", C.c_int),
        ("iterations", C.c_int), ("rounds", C.c_int), ("levels", C.c_int),
        ("rel_residual", C.c_double), ("rhs_norm", C.c_double),
    ]


def _dp(a):
    return a.ctypes.data_as(capi.c_double_p)


def singular(w) -> bool:
    return all(f == 1 for f in w.bcp_flag)


def pocoef(w, rho_ref=None, epsi=1.0e-3, tol=1.0e-30, stale_init=float("nan")):
    """PoCoef (I,J,K,6) by Compute1DGFMCoefficient (ProjectionP.f90:123-265)."""
    I, J, K = w.imax, w.jmax, w.kmax
    out = np.zeros((I, J, K, 6), order="F")
    s = capi.poisson_in(w)
    lib().oracle_pocoef(I, J, K, C.byref(s), w.rho_l, w.rho_g, rho_ref or w.rho_l, epsi, tol, stale_init, _dp(out))
    return out


def csr(w, pc):
    """Literal SetPoissonMatrix (ProjectionP.f90:301-482): CSR in PosNu order."""
    I, J, K = w.imax, w.jmax, w.kmax
    n = w.ext_cell + 1
    rp = np.zeros(n + 1, dtype=np.int64)
    ci = np.zeros(7 * n, dtype=np.int32)
    va = np.zeros(7 * n, dtype=np.float64)
    s = capi.poisson_in(w)
    bad = lib().oracle_matrix_csr(I, J, K, C.byref(s), _dp(pc), rp.ctypes.data_as(C.POINTER(C.c_int64)),
                                  ci.ctypes.data_as(capi.c_int32_p), _dp(va))
    if bad < 0:
        raise ValueError("PosNu inconsistent with ExtCell")
    nnz = int(rp[-1])
    return rp, ci[:nnz].copy(), va[:nnz].copy(), int(bad)


def rhs(w, pc):
    """Literal SetPoissonVectors (ProjectionP.f90:484-576): b in PosNu order."""
    I, J, K = w.imax, w.jmax, w.kmax
    b = np.zeros(w.ext_cell + 1)
    s = capi.poisson_in(w)
    lib().oracle_rhs(I, J, K, C.byref(s), _dp(pc), _dp(b))
    return b


def csr_apply(A, x):
    rp, ci, va = A[:3]
    y = np.zeros(rp.size - 1)
    lib().oracle_csr_apply(rp.size - 1, rp.ctypes.data_as(C.POINTER(C.c_int64)), ci.ctypes.data_as(capi.c_int32_p),
                           _dp(va), _dp(np.ascontiguousarray(x, dtype=np.float64)), _dp(y))
    return y


def csr_pcg(A, b, tol=1e-13, maxit=200000, singular_=False):
    rp, ci, va = A[:3]
    x = np.zeros(rp.size - 1)
    rr = C.c_double(0)
    it = lib().oracle_csr_pcg(rp.size - 1, rp.ctypes.data_as(C.POINTER(C.c_int64)), ci.ctypes.data_as(capi.c_int32_p),
                              _dp(va), _dp(b), _dp(x), tol, maxit, int(singular_), C.byref(rr))
    return x, it, rr.value


def csr_relres(A, b, x, singular_=False):
    rp, ci, va = A[:3]
    return lib().oracle_csr_relres(rp.size - 1, rp.ctypes.data_as(C.POINTER(C.c_int64)),
                                   ci.ctypes.data_as(capi.c_int32_p), _dp(va), _dp(b),
                                   _dp(np.ascontiguousarray(x, dtype=np.float64)), int(singular_))


def cheb_ratio(degree: int) -> float:
    """lmax/lmin of the Chebyshev smoother for a degree: max(6, 2 degree), as
    the library's smoother."""
    return 2.0 * degree if degree > 3 else 6.0


def gmg_solve(w, pc, b, precision=0, rel_tol=1e-13, max_iter=400, degree=2, ratio=None, coarse_max=64,
              max_rounds=12, inner_rtol=1e-4, line_seg=0):
    """CPU multigrid-preconditioned CG; returns (x in PosNu order, stats)."""
    I, J, K = w.imax, w.jmax, w.kmax
    x = np.zeros(w.ext_cell + 1)
    prm = GmgParams(precision=precision, rel_tol=rel_tol, max_iter=max_iter, max_rounds=max_rounds,
                    inner_rtol=inner_rtol, degree=degree, ratio=ratio or cheb_ratio(degree), coarse_max=coarse_max,
                    line_seg=line_seg)
    s = capi.poisson_in(w)
    rc = lib().oracle_gmg_solve(I, J, K, C.byref(s), _dp(pc), _dp(b), _dp(x), C.byref(prm))
    st = {f: getattr(prm, f) for f, _ in GmgParams._fields_}
    st["rc"] = rc
    return x, st


def gmg_vcycle(w, pc, r, precision=0, degree=3, ratio=None, coarse_max=64, line_seg=0):
    """One CPU V-cycle z = M r of the multigrid hierarchy of (w, pc); r and z
    ghosted FP64 arrays."""
    I, J, K = w.imax, w.jmax, w.kmax
    z = np.zeros(w.shape_g, order="F")
    prm = GmgParams(precision=precision, degree=degree, ratio=ratio or cheb_ratio(degree), coarse_max=coarse_max,
                    line_seg=line_seg)
    s = capi.poisson_in(w)
    rr = np.asfortranarray(r, dtype=np.float64)
    lib().oracle_gmg_vcycle(I, J, K, C.byref(s), _dp(pc), _dp(rr), _dp(z), C.byref(prm))
    return z


def scatter(w, x, pp0: Optional[np.ndarray] = None):
    """DeltaPressureGetValues + DeltaPressureBoundaryCondition."""
    I, J, K = w.imax, w.jmax, w.kmax
    pp = np.zeros(w.shape_g, order="F") if pp0 is None else pp0.copy(order="F")
    s = capi.poisson_in(w)
    lib().oracle_scatter(I, J, K, C.byref(s), _dp(np.ascontiguousarray(x)), _dp(pp))
    return pp


def correct(w, pc, pp, north_mass_fix=0):
    """Velocity correction + BoundaryConditionVarNew + mass correction.
    Returns (u, v, w, p, bcvar[4][6], status)."""
    I, J, K = w.imax, w.jmax, w.kmax
    a = w.arrays
    u, v, ww, p = (a[k].copy(order="F") for k in ("tvar_u", "tvar_v", "tvar_w", "tvar_p"))
    shapes = capi.bc_plane_shapes(I, J, K)
    total = 4 * sum(x * y for x, y in shapes)
    bc = np.zeros(total)
    s = capi.poisson_in(w)
    c = capi.correct_in(w)
    rc = lib().oracle_correct(I, J, K, C.byref(s), C.byref(c), _dp(pc), _dp(pp), _dp(u), _dp(v), _dp(ww), _dp(p),
                              _dp(bc), int(north_mass_fix))
    planes = []
    off = 0
    for f in range(4):
        row = []
        for shp in shapes:
            n = shp[0] * shp[1]
            row.append(bc[off:off + n].reshape(shp, order="F").copy(order="F"))
            off += n
        planes.append(row)
    return u, v, ww, p, planes, rc


def project(w, solver="gmg", rel_tol=1e-13, precision=0, north_mass_fix=0, **kw):
    """Whole projection on the CPU.  Returns a dict with PoCoef, the CSR
    system, the solution, Pp and the corrected fields."""
    pc = pocoef(w)
    A = csr(w, pc)
    b = rhs(w, pc)
    sing = singular(w)
    if solver == "csr":
        x, its, rr = csr_pcg(A, b, tol=rel_tol, singular_=sing)
        st = {"iterations": its, "rel_residual": rr}
    else:
        x, st = gmg_solve(w, pc, b, precision=precision, rel_tol=rel_tol, **kw)
    st["csr_relres"] = csr_relres(A, b, x, sing)
    pp = scatter(w, x)
    u, v, ww, p, bcv, rc = correct(w, pc, pp, north_mass_fix=north_mass_fix)
    return {"pocoef": pc, "A": A, "b": b, "x": x, "stats": st, "pp": pp, "u": u, "v": v, "w": ww, "p": p,
            "bcvar": bcv, "correct_rc": rc, "singular": sing}


def pressure_error(w, pp, pp_ref, singular_: bool) -> float:
    """Relative L2 difference of two ghosted pressures over the active
    interior cells (Cell_Type /= 2); for an all-Neumann system, where the
    pressure is defined up to a constant, the mean difference is removed."""
    act = w.arrays["cell_type"] != 2
    a = pp[1:-1, 1:-1, 1:-1][act]
    b = pp_ref[1:-1, 1:-1, 1:-1][act]
    d = a - b
    if singular_:
        d = d - d.mean()
        b = b - b.mean()
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(d)) / nb if nb > 0 else float(np.linalg.norm(d))


def velocity_error(fields, ref) -> float:
    """Largest relative L2 difference of the corrected u, v, w (whole
    ghosted arrays) against the reference fields."""
    out = 0.0
    for a, b in zip(fields, ref):
        nb = float(np.linalg.norm(b))
        e = float(np.linalg.norm(a - b))
        out = max(out, e / nb if nb > 0 else e)
    return out


def num_threads() -> int:
    return int(lib().oracle_num_threads())


def face_geo_cal(d1, d2, n1, n2, n3, d3, phi):
    """FaceGeoCal (CutCell.f90:883-981) of one face: (area, (c1, c2, c3))."""
    area = C.c_double()
    cent = (C.c_double * 3)()
    lib().oracle_face_geo_cal(d1, d2, n1, n2, n3, d3, phi, C.byref(area), cent)
    return area.value, tuple(cent)


def grid_preprocess(g):
    """GridPreprocess + DefineMomentumExchangeCell + NumberExternalCell x4
    (Main.f90:203-214) on a copy of ``g`` (simcoflow3d_gb300.geometry.GeoInputs);
    returns the copy."""
    from simcoflow3d_gb300 import geometry as GM
    out = g.copy()
    ss = [out.fams[f].struct() for f in GM.FAMILIES]
    rc = lib().oracle_grid_preprocess(out.imax, out.jmax, out.kmax, *(C.byref(s) for s in ss))
    if rc != 0:
        raise ValueError("grid too small")
    for f, s in zip(GM.FAMILIES, ss):
        out.fams[f].ext_cell = s.ext_cell
    return out


def mom_system(inp, opts, comp: int, dp_arr=None):
    """SetMatrix + SetVectors (PredictUVW.f90:856-1292) of component comp
    (0 = u): (CSR (rowptr, cols, vals), rhs, dp).  ``dp_arr`` (ghosted) is
    updated on the loop range like PUVW%Dp; a new zero array if None."""
    I, J, K = inp.imax, inp.jmax, inp.kmax
    n = inp.comps[comp].extcell + 1
    rp = np.zeros(n + 1, np.int64)
    ci = np.zeros(7 * max(n, 1), np.int32)
    va = np.zeros(7 * max(n, 1))
    rhs = np.zeros(max(n, 1))
    dp_arr = np.zeros(inp.shape_g(), order="F") if dp_arr is None else dp_arr
    st = inp.comps[comp].struct()
    nnz = lib().oracle_mom_system(I, J, K, comp + 1, C.byref(st), C.byref(opts),
                                  rp.ctypes.data_as(C.POINTER(C.c_int64)), ci.ctypes.data_as(capi.c_int32_p),
                                  _dp(va), _dp(rhs), _dp(dp_arr))
    if nnz < 0:
        raise ValueError("PosNu numbering does not match Cell_Type / ExtCell")
    return (rp, ci[:nnz], va[:nnz]), rhs[:n], dp_arr


def csr_bicgstab(A, b, tol=1e-14, maxit=20000):
    rp, ci, va = A
    x = np.zeros_like(b)
    rel = C.c_double()
    it = lib().oracle_csr_bicgstab(rp.size - 1, rp.ctypes.data_as(C.POINTER(C.c_int64)),
                                   ci.ctypes.data_as(capi.c_int32_p), _dp(va), _dp(b), _dp(x), tol, maxit,
                                   C.byref(rel))
    return x, it, rel.value


def predict_solves(inp, opts, pred=None, dp=None, tol=1e-14):
    """The solve part of PredictingUVW (PredictUVW.f90:691-802) on the CPU:
    per component SetMatrix/SetVectors, a BiCGStab solve to ``tol`` (true
    residual), DeltaGetValues; then the Dp ghost planes, the predictor's
    velocity BCs and the solid cells.  ``pred``/``dp`` are updated in place
    (new zero arrays if None).  Returns (pred, dp, info)."""
    I, J, K = inp.imax, inp.jmax, inp.kmax
    shp = inp.shape_g()
    pred = pred if pred is not None else [np.zeros(shp, order="F") for _ in range(3)]
    dp = dp if dp is not None else [np.zeros(shp, order="F") for _ in range(3)]
    info = []
    for c in range(3):
        A, b, _ = mom_system(inp, opts, c, dp[c])
        x, it, rel = csr_bicgstab(A, b, tol=tol)
        if it < 0:
            raise RuntimeError("oracle BiCGStab did not converge (component %d, rel %.3e)" % (c, rel))
        st = inp.comps[c].struct()
        lib().oracle_mom_get_values(I, J, K, c + 1, C.byref(st), _dp(x), _dp(pred[c]))
        info.append({"iterations": it, "rel_residual": rel, "rows": b.size})
    structs = inp.structs()
    lib().oracle_predict_tail(I, J, K, structs, *(_dp(a) for a in pred), *(_dp(a) for a in dp))
    return pred, dp, info


def volume_fraction_calc(dx, dy, dz, nx, ny, nz, s):
    """Volume_Fraction_Calc (Clsvof.f90:1475-1550) of one box."""
    return lib().oracle_volume_fraction_calc(dx, dy, dz, nx, ny, nz, s)


def uvw_liquid_field(pgrid, pcell, vgrids, vcells):
    """ComputeUVWLiquidField (Clsvof.f90:174-298).  ``pgrid``: (dx, dy, dz)
    interior arrays of the P grid; ``pcell``: dict of ghosted phil, nxl, nyl,
    nzl, vofl; ``vgrids``: three (dx, dy, dz) of the U, V, W grids;
    ``vcells``: three dicts with ghosted phil, nxl, nyl, nzl, vofl (updated
    in place) and vof."""
    I, J, K = pgrid[0].shape
    P = lambda a: _dp(a)
    arr3 = lambda key: (capi.c_double_p * 3)(*(P(c[key]) for c in vcells))
    g3 = lambda q: (capi.c_double_p * 3)(*(P(g[q]) for g in vgrids))
    lib().oracle_uvw_liquid_field(I, J, K, P(pgrid[0]), P(pgrid[1]), P(pgrid[2]), P(pcell["phil"]),
                                  P(pcell["nxl"]), P(pcell["nyl"]), P(pcell["nzl"]), P(pcell["vofl"]),
                                  g3(0), g3(1), g3(2), arr3("phil"), arr3("nxl"), arr3("nyl"), arr3("nzl"),
                                  arr3("vofl"), arr3("vof"))


def find_distance(dx, dy, dz, nx, ny, nz, f):
    """Find_Distance (Clsvof.f90:1311-1378) of one box."""
    return lib().oracle_find_distance(dx, dy, dz, nx, ny, nz, f)


def interface_reconstruct(centres, spacings, vfl, phi):
    """Interface_Reconstruct (Clsvof.f90:1216-1309).  ``centres``: the P
    grid's x, y, z; ``spacings``: dx, dy, dz (interior arrays); ``vfl``,
    ``phi`` ghosted.  Returns the ghosted nx, ny, nz, dis."""
    I, J, K = spacings[0].shape
    shp = (I + 2, J + 2, K + 2)
    out = [np.zeros(shp, order="F") for _ in range(4)]
    lib().oracle_interface_reconstruct(I, J, K, *(_dp(a) for a in centres), *(_dp(a) for a in spacings),
                                       _dp(vfl), _dp(phi), *(_dp(a) for a in out))
    return out


def clsvof_sweep(axis, centres, spacings, vfl, phi, vel, bc_vel, bc_lvs, dtv):
    """One directional sweep of Clsvof_Scheme: Interface_Reconstruct, then
    X_Sweep / Y_Sweep / Z_Sweep (Clsvof.f90:817-1214) for ``axis`` 0/1/2.
    ``vfl``, ``phi``, ``vel`` ghosted; ``bc_vel``, ``bc_lvs`` the wall planes
    at the low face of the axis ((J, K) for x, (I, K) for y, (I, J) for z).
    Returns the swept (temvf, temls), ghosted, and the normals nx, ny, nz,
    dis the sweep used."""
    I, J, K = spacings[0].shape
    shp = (I + 2, J + 2, K + 2)
    rec = [np.zeros(shp, order="F") for _ in range(4)]
    temvf = np.array(vfl, order="F", copy=True)
    temls = np.array(phi, order="F", copy=True)
    args = [np.asfortranarray(a, dtype=np.float64) for a in (vel, bc_vel, bc_lvs)]
    lib().oracle_clsvof_sweep(I, J, K, int(axis), *(_dp(a) for a in centres), *(_dp(a) for a in spacings),
                              _dp(vfl), _dp(phi), *(_dp(a) for a in args), float(dtv),
                              *(_dp(a) for a in rec), _dp(temvf), _dp(temls))
    return temvf, temls, rec


def clsvof_redistance(centres, spacings, vfl, phi):
    """The tail of a CLSVOF sub-step (Clsvof.f90:767-780): reconstruct the
    interface from ``vfl`` and ``phi`` (ghosted), then Redistance_Levelset.
    Returns the redistanced phi (ghosts as given) and the liquid normals."""
    I, J, K = spacings[0].shape
    out = np.array(phi, order="F", copy=True)
    nl = [np.zeros((I + 2, J + 2, K + 2), order="F") for _ in range(3)]
    rc = lib().oracle_clsvof_redistance(I, J, K, *(_dp(a) for a in centres), *(_dp(a) for a in spacings),
                                        _dp(vfl), _dp(out), *(_dp(a) for a in nl))
    if rc != 0:
        raise MemoryError("oracle_clsvof_redistance")
    return out, nl


def clsvof_scheme(centres, spacings, state, vel, fluid_normals, bc_vel, lvs_bc, dt, lvs_flag=(1,) * 6,
                  lvs_const=(0.0,) * 6, vof_flag=(1,) * 6, vof_const=(0.0,) * 6):
    """One Clsvof_Scheme step (Clsvof.f90:355-798).  ``state``: dict of the
    ghosted vofl, phil, nxl, nyl, nzl, updated in place; ``vel``: the
    ghosted u, v, w; ``fluid_normals``: the ghosted nx, ny, nz of the fluid;
    ``bc_vel``: the wall velocities BCu%VarW, BCv%VarS, BCw%VarB; ``lvs_bc``:
    the six level-set wall planes W, E, S, N, B, T, updated in place.
    Returns the six VOF wall planes."""
    I, J, K = spacings[0].shape
    shapes = [(J, K), (J, K), (I, K), (I, K), (I, J), (I, J)]
    for q, a in enumerate(lvs_bc):
        assert a.shape == shapes[q] and a.flags.f_contiguous and a.dtype == np.float64
    for key in ("vofl", "phil", "nxl", "nyl", "nzl"):
        assert state[key].flags.f_contiguous and state[key].dtype == np.float64
    vof_bc = [np.zeros(sh, order="F") for sh in shapes]
    keep = [np.asfortranarray(a, dtype=np.float64) for a in (*centres, *spacings, *fluid_normals, *vel, *bc_vel)]
    cx, cy, cz, dx, dy, dz, nx, ny, nz, u, v, w, bu, bv, bw = keep
    args = ClsvofArgs(I, J, K, _dp(cx), _dp(cy), _dp(cz), _dp(dx), _dp(dy), _dp(dz), _dp(state["vofl"]),
                      _dp(state["phil"]), _dp(state["nxl"]), _dp(state["nyl"]), _dp(state["nzl"]), _dp(nx),
                      _dp(ny), _dp(nz), _dp(u), _dp(v), _dp(w))
    args.bc_vel[:] = [_dp(bu), _dp(bv), _dp(bw)]
    args.lvs_bc[:] = [_dp(a) for a in lvs_bc]
    args.vof_bc[:] = [_dp(a) for a in vof_bc]
    args.lvs_flag[:] = list(lvs_flag)
    args.vof_flag[:] = list(vof_flag)
    args.lvs_const[:] = list(lvs_const)
    args.vof_const[:] = list(vof_const)
    args.dt = float(dt)
    if lib().oracle_clsvof_scheme(C.byref(args)) != 0:
        raise MemoryError("oracle_clsvof_scheme")
    return vof_bc
