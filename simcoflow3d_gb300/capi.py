"""ctypes mirror of ``include/scf_projection.h`` and the Python-side binding.

This is the binding a Python caller (or the test-suite) uses; the Fortran
host binds the same symbols through ISO_C_BINDING.  The structures below must
match the header field for field.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libscf_projection.so")

c_double_p = C.POINTER(C.c_double)
c_int32_p = C.POINTER(C.c_int32)

SCF_OK = 0
SCF_ERR_BAD_ARG = 1
SCF_ERR_NOT_CONVERGED = 2
SCF_ERR_NONFINITE = 3
SCF_ERR_CUDA = 4
SCF_ERR_OUT_OF_MEMORY = 5
SCF_ERR_BAD_INPUT = 6
SCF_ERR_UNDEFINED_IN_REFERENCE = 7
SCF_ERR_NO_DEVICE = 8
SCF_ERR_NO_SOLVE = 9

SCF_K_SMOOTH = 0
SCF_K_SPMV = 1
SCF_K_RESTRICT = 2
SCF_K_PROLONG = 3
SCF_K_CGUPDATE = 4
SCF_K_SMOOTH2 = 5

SCF_PREC_FP64 = 0
SCF_PREC_MIXED = 1


class ScfOpts(C.Structure):
    _fields_ = [
        ("precision", C.c_int32),
        ("rel_tol", C.c_double),
        ("max_iter", C.c_int32),
        ("max_rounds", C.c_int32),
        ("inner_rtol", C.c_double),
        ("smoother_degree", C.c_int32),
        ("coarse_max_cells", C.c_int32),
        ("rho_l", C.c_double),
        ("rho_g", C.c_double),
        ("rho_ref", C.c_double),
        ("epsi", C.c_double),
        ("gfm_tol", C.c_double),
        ("stale_init", C.c_double),
        ("warm_start", C.c_int32),
        ("north_mass_fix", C.c_int32),
        ("check_inputs", C.c_int32),
        ("device", C.c_int32),
        ("time_limit_s", C.c_double),
        ("smoother_lines", C.c_int32),
    ]


class ScfStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32),
        ("rounds", C.c_int32),
        ("converged", C.c_int32),
        ("singular", C.c_int32),
        ("levels", C.c_int32),
        ("gpu_launches", C.c_int32),
        ("rel_residual", C.c_double),
        ("rhs_norm", C.c_double),
        ("ms_assemble", C.c_double),
        ("ms_solve", C.c_double),
        ("ms_correct", C.c_double),
        ("ms_h2d", C.c_double),
        ("ms_d2h", C.c_double),
        ("ms_total", C.c_double),
        ("bytes_h2d", C.c_int64),
        ("bytes_d2h", C.c_int64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class ScfPoissonIn(C.Structure):
    _fields_ = [
        ("pgrid_dx", c_double_p), ("pgrid_dy", c_double_p), ("pgrid_dz", c_double_p),
        ("ugrid_dx", c_double_p), ("vgrid_dy", c_double_p), ("wgrid_dz", c_double_p),
        ("pcell_phil", c_double_p), ("pcell_vofl", c_double_p), ("pcell_vof", c_double_p),
        ("pcell_eearea", c_double_p), ("pcell_nearea", c_double_p), ("pcell_tearea", c_double_p),
        ("pcell_cell_type", c_int32_p), ("pcell_posnu", c_int32_p),
        ("pcell_extcell", C.c_int32),
        ("vof_old", c_double_p),
        ("pred_u", c_double_p), ("pred_v", c_double_p), ("pred_w", c_double_p),
        ("pu_dp", c_double_p), ("pv_dp", c_double_p), ("pw_dp", c_double_p),
        ("bcp_flag", C.c_int32 * 6),
        ("bcp_var", c_double_p * 6),
        ("dt", C.c_double),
    ]


class ScfCorrectIn(C.Structure):
    _fields_ = [
        ("ucell_moexcell", c_int32_p), ("ucell_cell_type", c_int32_p),
        ("vcell_moexcell", c_int32_p), ("vcell_cell_type", c_int32_p),
        ("wcell_moexcell", c_int32_p), ("wcell_cell_type", c_int32_p),
        ("bcu_flag", C.c_int32 * 6), ("bcv_flag", C.c_int32 * 6), ("bcw_flag", C.c_int32 * 6),
        ("bcu_const", C.c_double * 6), ("bcv_const", C.c_double * 6),
        ("bcw_const", C.c_double * 6), ("bcp_const", C.c_double * 6),
    ]


class ScfBcOut(C.Structure):
    _fields_ = [("var", (c_double_p * 6) * 4)]


class ScfGeoCells(C.Structure):
    """scf_geo_cells of include/scf_geometry.h: one cell family."""
    _fields_ = [
        ("dx", c_double_p), ("dy", c_double_p), ("dz", c_double_p),
        ("phi", c_double_p), ("nx", c_double_p), ("ny", c_double_p), ("nz", c_double_p),
        ("vof", c_double_p), ("vofl", c_double_p),
        ("cell_type", c_int32_p),
        ("eearea", c_double_p), ("nearea", c_double_p), ("tearea", c_double_p),
        ("fce", c_double_p), ("fcn", c_double_p), ("fct", c_double_p),
        ("cell_cent", c_double_p), ("wllh", c_double_p), ("delh", c_double_p),
        ("moexcell", c_int32_p), ("posnu", c_int32_p),
        ("ext_cell", C.c_int32),
    ]


class ScfGeoStats(C.Structure):
    _fields_ = [
        ("gpu_launches", C.c_int32), ("exact_faces", C.c_int32),
        ("ms_h2d", C.c_double), ("ms_device", C.c_double), ("ms_d2h", C.c_double), ("ms_total", C.c_double),
        ("bytes_h2d", C.c_int64), ("bytes_d2h", C.c_int64),
        ("ms_faces", C.c_double), ("bytes_faces", C.c_int64),
    ]


class ScfVtrField(C.Structure):
    """scf_vtr_field of include/scf_output.h."""
    _fields_ = [("name", C.c_char_p), ("data", C.c_void_p), ("on_device", C.c_int32)]


class ScfVtrStats(C.Structure):
    _fields_ = [("ms_convert", C.c_double), ("ms_d2h", C.c_double), ("ms_write", C.c_double),
                ("ms_total", C.c_double), ("bytes_file", C.c_int64), ("gpu_launches", C.c_int32)]


class ScfMomIn(C.Structure):
    """scf_mom_in of include/scf_predictor.h: one velocity component."""
    _fields_ = [
        ("grid_dx", c_double_p), ("grid_dy", c_double_p), ("grid_dz", c_double_p),
        ("vof", c_double_p), ("vofl", c_double_p),
        ("eta_e", c_double_p), ("eta_n", c_double_p), ("eta_t", c_double_p),
        ("cell_type", c_int32_p), ("posnu", c_int32_p), ("extcell", C.c_int32),
        ("vof_old", c_double_p),
        ("df_ew", c_double_p), ("df_ns", c_double_p), ("df_tb", c_double_p),
        ("edf_ew", c_double_p), ("edf_ns", c_double_p), ("edf_tb", c_double_p),
        ("fric", c_double_p), ("flux_div", c_double_p), ("tvar", c_double_p),
        ("bc_flag", C.c_int32 * 6), ("bc_var", c_double_p * 6),
    ]


class ScfMomOpts(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("rho_a_ref", C.c_double), ("rho_w_ref", C.c_double), ("fr", C.c_double),
        ("gx", C.c_double), ("gy", C.c_double), ("gz", C.c_double), ("g", C.c_double),
        ("beta_vis", C.c_double), ("rel_tol", C.c_double), ("max_iter", C.c_int32), ("precision", C.c_int32),
        ("kernel_timing", C.c_int32),
    ]


class ScfMomStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32 * 3), ("rounds", C.c_int32 * 3), ("converged", C.c_int32 * 3),
        ("rel_residual", C.c_double * 3),
        ("ms_assemble", C.c_double), ("ms_solve", C.c_double), ("ms_tail", C.c_double),
        ("ms_h2d", C.c_double), ("ms_d2h", C.c_double), ("ms_total", C.c_double),
        ("bytes_h2d", C.c_int64), ("bytes_d2h", C.c_int64), ("gpu_launches", C.c_int32),
        ("timed_iterations", C.c_int32), ("ms_kernels", C.c_double * 4),
    ]

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


class ScfClsvofIn(C.Structure):
    """scf_clsvof_in of include/scf_clsvof.h."""
    _fields_ = [(n, c_double_p) for n in ("x", "y", "z", "dx", "dy", "dz", "u", "v", "w", "nx", "ny", "nz",
                                          "bc_u_w", "bc_v_s", "bc_w_b")] + [
        ("lvs_flag", C.c_int32 * 6), ("vof_flag", C.c_int32 * 6), ("lvs_const", C.c_double * 6),
        ("vof_const", C.c_double * 6), ("dt", C.c_double)]


class ScfClsvofState(C.Structure):
    """scf_clsvof_state of include/scf_clsvof.h."""
    _fields_ = [(n, c_double_p) for n in ("vofl", "phil", "nxl", "nyl", "nzl")] + [
        ("lvs_bc", c_double_p * 6), ("vof_bc", c_double_p * 6)]


class ScfClsvofVcell(C.Structure):
    """scf_clsvof_vcell of include/scf_clsvof.h: one velocity family."""
    _fields_ = [(n, c_double_p) for n in ("dx", "dy", "dz", "phil", "nxl", "nyl", "nzl", "vofl")]


class ScfClsvofStats(C.Structure):
    _fields_ = [("ms_h2d", C.c_double), ("ms_run", C.c_double), ("ms_d2h", C.c_double), ("ms_total", C.c_double),
                ("bytes_h2d", C.c_int64), ("bytes_d2h", C.c_int64), ("steps", C.c_int32),
                ("gpu_launches", C.c_int32), ("ms_kernels", C.c_double * 4)]

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


def require(cond: bool, message: str) -> None:
    """Argument check that stays active under ``python -O``: a wrong array
    handed to the C side would be read or written past its end."""
    if not cond:
        raise ValueError(message)


def require_shape(a: np.ndarray, shape, name: str = "array") -> None:
    require(tuple(a.shape) == tuple(shape), f"{name} has shape {tuple(a.shape)}, expected {tuple(shape)}")


def dptr(a: Optional[np.ndarray]):
    if a is None:
        return c_double_p()
    require(a.dtype == np.float64 and (a.flags.f_contiguous or a.ndim <= 1), "FP64 Fortran-contiguous array required")
    return a.ctypes.data_as(c_double_p)


def iptr(a: Optional[np.ndarray]):
    if a is None:
        return c_int32_p()
    require(a.dtype == np.int32 and (a.flags.f_contiguous or a.ndim <= 1), "int32 Fortran-contiguous array required")
    return a.ctypes.data_as(c_int32_p)


BCP_KEYS = ("bcp_var_w", "bcp_var_e", "bcp_var_s", "bcp_var_n", "bcp_var_b", "bcp_var_t")


def poisson_in(w, pred=None) -> ScfPoissonIn:
    """Builds the input struct from a ``workloads.Workload``.  The caller
    keeps ``w`` (and ``pred``) alive while the struct is used."""
    a = w.arrays
    pu, pv, pw = (pred if pred is not None else (a["u_star"], a["v_star"], a["w_star"]))
    s = ScfPoissonIn()
    s.pgrid_dx, s.pgrid_dy, s.pgrid_dz = dptr(a["pgrid_dx"]), dptr(a["pgrid_dy"]), dptr(a["pgrid_dz"])
    s.ugrid_dx, s.vgrid_dy, s.wgrid_dz = dptr(a["ugrid_dx"]), dptr(a["vgrid_dy"]), dptr(a["wgrid_dz"])
    s.pcell_phil, s.pcell_vofl, s.pcell_vof = dptr(a["phil"]), dptr(a["vofl"]), dptr(a["vof"])
    s.pcell_eearea, s.pcell_nearea, s.pcell_tearea = dptr(a["eearea"]), dptr(a["nearea"]), dptr(a["tearea"])
    s.pcell_cell_type, s.pcell_posnu = iptr(a["cell_type"]), iptr(a["posnu"])
    s.pcell_extcell = int(w.ext_cell)
    s.vof_old = dptr(a["vof_old"])
    s.pred_u, s.pred_v, s.pred_w = dptr(pu), dptr(pv), dptr(pw)
    s.pu_dp, s.pv_dp, s.pw_dp = dptr(a["dp_u"]), dptr(a["dp_v"]), dptr(a["dp_w"])
    for q in range(6):
        s.bcp_flag[q] = int(w.bcp_flag[q])
        s.bcp_var[q] = dptr(a[BCP_KEYS[q]])
    s.dt = float(w.dt)
    return s


def correct_in(w) -> ScfCorrectIn:
    a = w.arrays
    s = ScfCorrectIn()
    s.ucell_moexcell, s.ucell_cell_type = iptr(a["ucell_moexcell"]), iptr(a["ucell_cell_type"])
    s.vcell_moexcell, s.vcell_cell_type = iptr(a["vcell_moexcell"]), iptr(a["vcell_cell_type"])
    s.wcell_moexcell, s.wcell_cell_type = iptr(a["wcell_moexcell"]), iptr(a["wcell_cell_type"])
    for q in range(6):
        s.bcu_flag[q], s.bcv_flag[q], s.bcw_flag[q] = int(w.bcu_flag[q]), int(w.bcv_flag[q]), int(w.bcw_flag[q])
        s.bcu_const[q], s.bcv_const[q] = float(w.bcu_const[q]), float(w.bcv_const[q])
        s.bcw_const[q], s.bcp_const[q] = float(w.bcw_const[q]), float(w.bcp_const[q])
    return s


def bc_plane_shapes(I, J, K):
    return [(J, K), (J, K), (I, K), (I, K), (I, J), (I, J)]


def new_bc_out(I, J, K):
    """Allocates BC Var output planes; returns (struct, list[4][6] arrays)."""
    arrs = [[np.zeros(shp, order="F") for shp in bc_plane_shapes(I, J, K)] for _ in range(4)]
    s = ScfBcOut()
    for f in range(4):
        for q in range(6):
            s.var[f][q] = dptr(arrs[f][q])
    return s, arrs
