"""Host side of the momentum predictor's implicit solves on GB300
(include/scf_predictor.h): the inputs of the three velocity components in the
reference's layouts, the call through the C ABI, and a synthetic input
generator for tests and benchmarks.

The reference computes these inputs in PredictingUVW (src/PredictUVW.f90:
49-690: convective fluxes, DiffusiveFlux 3349-3674, wall friction, FluxDiv)
and hands them to SetMatrix/SetVectors (856-1292).  Those upstream routines
are outside this path; ``momentum_inputs`` synthesises inputs of the same
kind (viscous face conductances from the cut-cell apertures and the liquid
fraction, cut-face corrections, wall friction at cut cells) from a
preprocessed cut-cell geometry.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import Dict, List, Optional

import numpy as np

from . import capi

COMPONENTS = ("u", "v", "w")
ARRAYS = ("grid_dx", "grid_dy", "grid_dz", "vof", "vofl", "eta_e", "eta_n", "eta_t", "cell_type", "posnu",
          "vof_old", "df_ew", "df_ns", "df_tb", "edf_ew", "edf_ns", "edf_tb", "fric", "flux_div", "tvar")

# water and air (StateVariables.f90:9-10)
MU_W, MU_A = 1.002e-3, 1.506e-5
RHO_W, RHO_A = 998.3, 1.205
G = 9.80665


def array_shape(name: str, comp: int, I: int, J: int, K: int):
    """Shape of one input array of component comp (0 = u, 1 = v, 2 = w)."""
    if name in ("vof", "vofl", "eta_e", "eta_n", "eta_t", "vof_old", "tvar"):
        return (I + 2, J + 2, K + 2)
    if name in ("df_ew", "edf_ew"):
        return (I + 2, J, K)
    if name in ("df_ns", "edf_ns"):
        return (I, J + 2, K)
    if name in ("df_tb", "edf_tb"):
        return (I, J, K + 2)
    if name == "posnu":
        return (I - (comp == 0), J - (comp == 1), K - (comp == 2))
    return (I, J, K)


def bc_shapes(I: int, J: int, K: int):
    """VarW, VarE (J,K), VarS, VarN (I,K), VarB, VarT (I,J)."""
    return [(J, K), (J, K), (I, K), (I, K), (I, J), (I, J)]


@dataclasses.dataclass
class MomComponent:
    arrays: Dict[str, np.ndarray]
    bc_flag: List[int]
    bc_var: List[np.ndarray]
    extcell: int

    def struct(self) -> capi.ScfMomIn:
        s = capi.ScfMomIn()
        for f in ARRAYS:
            a = self.arrays[f]
            setattr(s, f, capi.iptr(a) if a.dtype == np.int32 else capi.dptr(a))
        s.extcell = self.extcell
        for q in range(6):
            s.bc_flag[q] = int(self.bc_flag[q])
            s.bc_var[q] = capi.dptr(self.bc_var[q])
        return s


@dataclasses.dataclass
class MomInputs:
    imax: int
    jmax: int
    kmax: int
    comps: List[MomComponent]
    meta: Dict[str, object] = dataclasses.field(default_factory=dict)

    def structs(self):
        arr = (capi.ScfMomIn * 3)()
        for c in range(3):
            arr[c] = self.comps[c].struct()
        return arr

    def shape_g(self):
        return (self.imax + 2, self.jmax + 2, self.kmax + 2)


def default_opts(dt: float = 1.0e-3, precision: int = capi.SCF_PREC_FP64, rel_tol: float = 1.0e-10,
                 max_iter: int = 1000, fr: float = 1.0) -> capi.ScfMomOpts:
    """Options of a dam-break-like run: water reference density (Roref = row),
    gravity along -z, Fr = 1 (Uref = sqrt(g Lref), Dambreak.f90:45,58),
    beta_vis = 0.5 (PredictUVW.f90:35)."""
    o = capi.ScfMomOpts()
    o.dt = dt
    o.rho_a_ref = RHO_A / RHO_W
    o.rho_w_ref = 1.0
    o.fr = fr
    o.gx, o.gy, o.gz, o.g = 0.0, 0.0, -G, G
    o.beta_vis = 0.5
    o.rel_tol = rel_tol
    o.max_iter = max_iter
    o.precision = precision
    return o


def _clip_idx(n, lo, hi):
    return np.clip(np.arange(n), lo, hi)


def momentum_inputs(geo, seed: int = 20261203, rey: float = 300.0, dt: float = 1.0e-3,
                    vof_old_noise: float = 0.0, edf: float = 0.2, lid: float = 1.0) -> MomInputs:
    """Synthetic inputs of the three momentum systems on a preprocessed
    geometry ``geo`` (simcoflow3d_gb300.geometry.GeoInputs after
    GridPreprocess; families u, v, w).

    - DF: mu_f * aperture * face area / spacing / Rey on every face, mu_f the
      mean of the two cells' mixture viscosities (liquid fraction vofL/vof,
      water/air with the water reference); Rey = 300 as the dam-break case
      (src/Test/Dambreak/input.dat).
    - EDF: edf * DF * U(-1, 1) on partly open faces, 0 elsewhere.
    - Eta: 0.5, U(0.3, 0.7) on cut cells.  Fric: U(0, 0.05) vof dV/dt on cut
      cells.  FluxDiv: N(0, (0.01 dV/dt)^2).  TVar: smoothed N(0, 0.1^2).
    - vofO = vof (+ vof_old_noise * N(0,1) on cut cells, clipped to [0, 1]).
    - BCs: the wall-normal component is Dirichlet 0 on its two faces, the
      tangential ones Neumann, except u on the top face: Dirichlet ``lid``.
    """
    from .workloads import _smoothed_velocity
    rng = np.random.default_rng(seed)
    I, J, K = geo.imax, geo.jmax, geo.kmax
    shp_g = (I + 2, J + 2, K + 2)
    F = lambda a: np.asfortranarray(a, dtype=np.float64)
    mu_ref = MU_W
    comps = []
    for c, fam in enumerate(COMPONENTS):
        fa = geo.fams[fam].arrays
        vof, vofl = fa["vof"], fa["vofl"]
        dx, dy, dz = fa["dx"], fa["dy"], fa["dz"]
        frac = np.clip(vofl / (vof + 1.0e-15), 0.0, 1.0)
        mu = frac * (MU_W / mu_ref) + (1.0 - frac) * (MU_A / mu_ref)   # ghosted
        cut = (vof > 0.0) & (vof < 1.0)
        ci, cj, ck = _clip_idx(I + 2, 1, I) - 1, _clip_idx(J + 2, 1, J) - 1, _clip_idx(K + 2, 1, K) - 1
        # east-west faces: DFEW(i) between ghosted cells i-1 and i, i = 0..I+1
        ii = np.arange(I + 2)
        lo, hi = np.clip(ii - 1, 0, I + 1), ii
        mu_ew = 0.5 * (mu[lo, 1:-1, 1:-1] + mu[hi, 1:-1, 1:-1])
        ap_ew = fa["eearea"][lo, 1:-1, 1:-1]
        dfew = mu_ew * ap_ew * (dy[ci] * dz[ci]) / dx[ci] / rey
        jj = np.arange(J + 2)
        lo, hi = np.clip(jj - 1, 0, J + 1), jj
        mu_ns = 0.5 * (mu[1:-1, lo, 1:-1] + mu[1:-1, hi, 1:-1])
        ap_ns = fa["nearea"][1:-1, lo, 1:-1]
        dfns = mu_ns * ap_ns * (dx[:, cj] * dz[:, cj]) / dy[:, cj] / rey
        kk = np.arange(K + 2)
        lo, hi = np.clip(kk - 1, 0, K + 1), kk
        mu_tb = 0.5 * (mu[1:-1, 1:-1, lo] + mu[1:-1, 1:-1, hi])
        ap_tb = fa["tearea"][1:-1, 1:-1, lo]
        dftb = mu_tb * ap_tb * (dx[:, :, ck] * dy[:, :, ck]) / dz[:, :, ck] / rey

        def edf_of(df, ap):
            part = (ap > 0.0) & (ap < 1.0)
            return np.where(part, edf * df * rng.uniform(-1.0, 1.0, size=df.shape), 0.0)

        eta = []
        for _ in range(3):
            e = np.full(shp_g, 0.5)
            e[cut] = rng.uniform(0.3, 0.7, size=int(cut.sum()))
            eta.append(F(e))
        dV = dx * dy * dz
        cut_i = cut[1:-1, 1:-1, 1:-1]
        fric = np.where(cut_i, rng.uniform(0.0, 0.05, size=dV.shape) * vof[1:-1, 1:-1, 1:-1] * dV / dt, 0.0)
        flux = rng.normal(0.0, 1.0, size=dV.shape) * 0.01 * dV / dt
        tvar = _smoothed_velocity(rng, shp_g)
        vo = vof.copy(order="F")
        if vof_old_noise:
            vo[cut] = np.clip(vof[cut] + vof_old_noise * rng.normal(size=int(cut.sum())), 0.0, 1.0)
        arrays = {
            "grid_dx": F(dx), "grid_dy": F(dy), "grid_dz": F(dz),
            "vof": F(vof), "vofl": F(vofl), "eta_e": eta[0], "eta_n": eta[1], "eta_t": eta[2],
            "cell_type": np.asfortranarray(fa["cell_type"], dtype=np.int32),
            "posnu": np.asfortranarray(fa["posnu"], dtype=np.int32),
            "vof_old": vo,
            "df_ew": F(dfew), "df_ns": F(dfns), "df_tb": F(dftb),
            "edf_ew": F(edf_of(dfew, ap_ew)), "edf_ns": F(edf_of(dfns, ap_ns)), "edf_tb": F(edf_of(dftb, ap_tb)),
            "fric": F(fric), "flux_div": F(flux), "tvar": F(tvar),
        }
        flags = [1] * 6
        flags[2 * c] = flags[2 * c + 1] = 0
        bvars = [np.zeros(s, order="F") for s in bc_shapes(I, J, K)]
        if c == 0:
            flags[5] = 0
            bvars[5][:] = lid
        comps.append(MomComponent(arrays, flags, bvars, int(geo.fams[fam].ext_cell)))
    return MomInputs(I, J, K, comps, {"rey": rey, "dt": dt, "seed": seed})


def new_outputs(inp: MomInputs, fill: float = 0.0):
    """Host arrays for Pred%u/v/w and PU/PV/PW%Dp (ghosted, Fortran order)."""
    shp = inp.shape_g()
    return ([np.full(shp, fill, order="F") for _ in range(3)], [np.full(shp, fill, order="F") for _ in range(3)])


class PredictSolves:
    """The momentum predictor's implicit solves on the GPU for one grid size."""

    def __init__(self, imax: int, jmax: int, kmax: int, device: int = 0, lib=None):
        from .projection import load_library
        self.L = lib or load_library()
        self.shape = (imax, jmax, kmax)
        self.ctx = C.c_void_p()
        rc = self.L.scf_mom_create(C.byref(self.ctx), imax, jmax, kmax, device)
        if rc != 0:
            raise RuntimeError("scf_mom_create failed with status %d" % rc)

    def close(self):
        if self.ctx:
            self.L.scf_mom_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _err(self, rc):
        from .projection import ScfError
        buf = C.create_string_buffer(512)
        self.L.scf_mom_last_error(self.ctx, buf, 512)
        raise ScfError(rc, buf.value.decode(errors="replace"))

    def __call__(self, inp: MomInputs, opts: capi.ScfMomOpts, pred=None, dp=None, check: bool = True):
        """scf_predict_solves: returns (pred [u, v, w], dp [PU, PV, PW], stats).
        ``pred``/``dp`` are the host arrays written (new zero arrays if None)."""
        if pred is None or dp is None:
            p0, d0 = new_outputs(inp)
            pred = pred if pred is not None else p0
            dp = dp if dp is not None else d0
        st = capi.ScfMomStats()
        rc = self.L.scf_predict_solves(self.ctx, self.structs_of(inp), C.byref(opts),
                                       *(capi.dptr(a) for a in pred), *(capi.dptr(a) for a in dp), C.byref(st))
        if rc != 0 and check:
            self._err(rc)
        return pred, dp, st.as_dict()

    def structs_of(self, inp: MomInputs):
        self._keep = inp.structs()
        return self._keep

    def stage(self, inp: MomInputs):
        rc = self.L.scf_mom_stage(self.ctx, self.structs_of(inp))
        if rc != 0:
            self._err(rc)

    def run(self, opts: capi.ScfMomOpts, check: bool = True) -> dict:
        st = capi.ScfMomStats()
        rc = self.L.scf_mom_run(self.ctx, C.byref(opts), C.byref(st))
        if rc != 0 and check:
            self._err(rc)
        return st.as_dict()

    def fetch(self, pred=None, dp=None):
        pred = pred or [None] * 3
        dp = dp or [None] * 3
        rc = self.L.scf_mom_fetch(self.ctx, *(capi.dptr(a) for a in pred), *(capi.dptr(a) for a in dp))
        if rc != 0:
            self._err(rc)

    def device_fields(self):
        ptrs = [C.c_void_p() for _ in range(6)]
        rc = self.L.scf_mom_device_fields(self.ctx, *(C.byref(p) for p in ptrs))
        if rc != 0:
            self._err(rc)
        return [p.value for p in ptrs]
