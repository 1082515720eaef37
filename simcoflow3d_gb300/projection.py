"""Python mirror of SIMCOFlow's projection interface over the C ABI.

``Projection.poisson_solve`` stands in for ``PoissonEquationSolver``
(``src/ProjectionP.f90:33-121``) and ``Projection.update_puvw`` for the
projection part of ``UpdatePUVW`` (``src/ComputePUVW.f90:127-129,179-384``).
Arguments are the reference's arrays (Fortran-ordered numpy arrays, ghosted
where the reference ghosts them), bundled in a ``workloads.Workload``.

There is no CPU fallback: if ``libscf_projection.so`` is missing or no GPU is
visible, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import capi

_lib = None


class ScfError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{capi_status(status)} ({status}): {message}")
        self.status = status


def load_library(path: Optional[str] = None):
    """Loads the CUDA library (never a substitute)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or capi.LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with __graft_entry__.build() "
                           "(there is no CPU fallback)")
    L = C.CDLL(path)
    P = C.POINTER
    L.scf_opts_default.argtypes = [P(capi.ScfOpts)]
    L.scf_opts_default.restype = None
    L.scf_ctx_create.argtypes = [P(C.c_void_p), C.c_int32, C.c_int32, C.c_int32, P(capi.ScfOpts)]
    L.scf_ctx_destroy.argtypes = [C.c_void_p]
    L.scf_ctx_set_opts.argtypes = [C.c_void_p, P(capi.ScfOpts)]
    L.scf_poisson_solve.argtypes = [C.c_void_p, P(capi.ScfPoissonIn), capi.c_double_p, capi.c_double_p,
                                    P(capi.ScfStats)]
    L.scf_update_puvw.argtypes = [C.c_void_p, P(capi.ScfPoissonIn), P(capi.ScfCorrectIn), capi.c_double_p,
                                  capi.c_double_p, capi.c_double_p, capi.c_double_p, P(capi.ScfBcOut),
                                  P(capi.ScfStats)]
    L.scf_stage_inputs.argtypes = [C.c_void_p, P(capi.ScfPoissonIn), P(capi.ScfCorrectIn), capi.c_double_p,
                                   capi.c_double_p, capi.c_double_p, capi.c_double_p]
    L.scf_run_projection.argtypes = [C.c_void_p, P(capi.ScfStats)]
    L.scf_fetch_outputs.argtypes = [C.c_void_p, capi.c_double_p, capi.c_double_p, capi.c_double_p,
                                    capi.c_double_p, capi.c_double_p, capi.c_double_p, P(capi.ScfBcOut)]
    L.scf_debug_apply.argtypes = [C.c_void_p, capi.c_double_p, capi.c_double_p]
    L.scf_debug_operator.argtypes = [C.c_void_p] + [capi.c_double_p] * 5
    L.scf_debug_operator_f32.argtypes = [C.c_void_p] + [C.POINTER(C.c_float)] * 9 + [capi.c_double_p]
    L.scf_debug_precondition.argtypes = [C.c_void_p, capi.c_double_p, capi.c_double_p]
    L.scf_status_string.argtypes = [C.c_int]
    L.scf_status_string.restype = C.c_char_p
    L.scf_last_error.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t]
    L.scf_host_register.argtypes = [C.c_void_p, C.c_size_t]
    L.scf_host_unregister.argtypes = [C.c_void_p]
    L.scf_abi_version.argtypes = []
    L.scf_debug_time_kernel.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.scf_kernel_timing.argtypes = [C.c_void_p, C.c_int]
    L.scf_kernel_timing_read.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_longlong),
                                         C.POINTER(C.c_double)]
    L.scf_loss_forward.argtypes = [C.c_void_p, P(capi.ScfPoissonIn), P(capi.ScfCorrectIn), capi.c_double_p,
                                   capi.c_double_p, capi.c_double_p, P(capi.ScfStats)]
    L.scf_loss_backward.argtypes = [C.c_void_p] + [capi.c_double_p] * 4 + [P(capi.ScfStats)]
    P_G = P(capi.ScfGeoCells)
    L.scf_geo_create.argtypes = [P(C.c_void_p), C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    L.scf_geo_destroy.argtypes = [C.c_void_p]
    L.scf_grid_preprocess.argtypes = [C.c_void_p, P_G, P_G, P_G, P_G, P(capi.ScfGeoStats)]
    L.scf_geo_stage.argtypes = [C.c_void_p, P_G, P_G, P_G, P_G]
    L.scf_geo_run.argtypes = [C.c_void_p, P(capi.ScfGeoStats)]
    L.scf_geo_fetch.argtypes = [C.c_void_p, P_G, P_G, P_G, P_G]
    L.scf_geo_last_error.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t]
    L.scf_write_vtr.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.c_int32] + [capi.c_double_p] * 6 + [
        C.c_int32, P(capi.ScfVtrField), C.c_int32, P(capi.ScfVtrStats)]
    L.scf_write_vtr_binary.argtypes = L.scf_write_vtr.argtypes
    L.scf_ctx_device_fields.argtypes = [C.c_void_p] + [P(C.c_void_p)] * 7
    L.scf_apply_operator_noalloc.argtypes = [C.c_int32, C.c_int32, C.c_int32] + [C.c_void_p] * 8
    L.scf_debug_smoother_pairs.argtypes = [C.c_int, C.c_int]
    L.scf_debug_smoother_pair_counts.argtypes = [C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    P_M = P(capi.ScfMomIn)
    L.scf_mom_create.argtypes = [P(C.c_void_p), C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    L.scf_mom_destroy.argtypes = [C.c_void_p]
    L.scf_mom_stage.argtypes = [C.c_void_p, P_M]
    L.scf_mom_run.argtypes = [C.c_void_p, P(capi.ScfMomOpts), P(capi.ScfMomStats)]
    L.scf_mom_fetch.argtypes = [C.c_void_p] + [capi.c_double_p] * 6
    L.scf_predict_solves.argtypes = [C.c_void_p, P_M, P(capi.ScfMomOpts)] + [capi.c_double_p] * 6 + [
        P(capi.ScfMomStats)]
    L.scf_mom_device_fields.argtypes = [C.c_void_p] + [P(C.c_void_p)] * 6
    L.scf_mom_last_error.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t]
    L.scf_clsvof_create.argtypes = [P(C.c_void_p), C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    L.scf_clsvof_destroy.argtypes = [C.c_void_p]
    L.scf_clsvof_stage.argtypes = [C.c_void_p, P(capi.ScfClsvofIn), P(capi.ScfClsvofState)]
    L.scf_clsvof_run.argtypes = [C.c_void_p, C.c_int32, P(capi.ScfClsvofStats)]
    L.scf_clsvof_fetch.argtypes = [C.c_void_p, P(capi.ScfClsvofState), P(capi.ScfClsvofStats)]
    L.scf_clsvof_step.argtypes = [C.c_void_p, P(capi.ScfClsvofIn), P(capi.ScfClsvofState),
                                  P(capi.ScfClsvofStats)]
    L.scf_clsvof_uvw_liquid_field.argtypes = [C.c_void_p, P(capi.ScfClsvofVcell), P(capi.ScfClsvofStats)]
    L.scf_clsvof_set_timing.argtypes = [C.c_void_p, C.c_int32]
    L.scf_clsvof_device_fields.argtypes = [C.c_void_p, P(C.c_void_p), P(C.c_void_p)]
    L.scf_clsvof_last_error.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t]
    _lib = L
    return L


def capi_status(s: int) -> str:
    try:
        return load_library().scf_status_string(int(s)).decode()
    except Exception:
        return f"status {s}"


def smoother_pairs(on: int = 1, planes: int = 0):
    """Fused pairs of Chebyshev steps: 1 on the large FP32 V-cycle levels
    where they are faster (the default), 2 on every FP32 level of at least
    2^18 cells, 0 one step per pass; all give the same bits."""
    L = load_library()
    rc = L.scf_debug_smoother_pairs(int(on), int(planes))
    if rc != capi.SCF_OK:
        raise ScfError(rc, capi_status(rc))


def smoother_pair_counts():
    """(launches of the TMA-staged pair kernel, pairs that fell back to
    one-step launches), process-wide."""
    L = load_library()
    t, f = C.c_int64(0), C.c_int64(0)
    L.scf_debug_smoother_pair_counts(C.byref(t), C.byref(f))
    return t.value, f.value


def default_opts(**kw) -> capi.ScfOpts:
    o = capi.ScfOpts()
    load_library().scf_opts_default(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


class Projection:
    """One device context for an I x J x K grid."""

    def __init__(self, imax: int, jmax: int, kmax: int, **opts):
        self.L = load_library()
        self.shape = (imax, jmax, kmax)
        self.opts = default_opts(**opts)
        self.ctx = C.c_void_p()
        rc = self.L.scf_ctx_create(C.byref(self.ctx), imax, jmax, kmax, C.byref(self.opts))
        if rc != 0:
            raise ScfError(rc, "scf_ctx_create failed")

    @classmethod
    def for_workload(cls, w, **opts):
        opts.setdefault("rho_l", w.rho_l)
        opts.setdefault("rho_g", w.rho_g)
        return cls(w.imax, w.jmax, w.kmax, **opts)

    # -- helpers ---------------------------------------------------------------
    def last_error(self) -> str:
        buf = C.create_string_buffer(512)
        self.L.scf_last_error(self.ctx, buf, 512)
        return buf.value.decode(errors="replace")

    def _check(self, rc: int, allow=()):
        if rc != 0 and rc not in allow:
            raise ScfError(rc, self.last_error())
        return rc

    def set_opts(self, **kw):
        for k, v in kw.items():
            setattr(self.opts, k, v)
        self._check(self.L.scf_ctx_set_opts(self.ctx, C.byref(self.opts)))

    def close(self):
        if self.ctx:
            self.L.scf_ctx_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- the reference's entry points ------------------------------------------
    def poisson_solve(self, w, want_pocoef: bool = True, allow_not_converged: bool = False):
        """PoissonEquationSolver: returns (PoCoef (I,J,K,6) or None, Pp ghosted, stats)."""
        I, J, K = self.shape
        pin = capi.poisson_in(w)
        pc = np.zeros((I, J, K, 6), order="F") if want_pocoef else None
        pp = np.zeros(w.shape_g, order="F")
        st = capi.ScfStats()
        rc = self.L.scf_poisson_solve(self.ctx, C.byref(pin), capi.dptr(pc), capi.dptr(pp), C.byref(st))
        self._check(rc, (capi.SCF_ERR_NOT_CONVERGED,) if allow_not_converged else ())
        return pc, pp, st.as_dict()

    def update_puvw(self, w, tvar=None, want_bc: bool = True, allow_not_converged: bool = False, pred=None,
                    bc_out=None):
        """UpdatePUVW's projection: returns (u, v, w, p, bcvar[4][6] or None, stats).
        ``tvar`` defaults to copies of the workload's TVar arrays; ``pred``
        optionally replaces the workload's (u*, v*, w*); ``bc_out``
        optionally gives the 4 x 6 BC Var planes to write (else new arrays)."""
        a = w.arrays
        if tvar is None:
            tvar = [a[k].copy(order="F") for k in ("tvar_u", "tvar_v", "tvar_w", "tvar_p")]
        u, v, ww, p = tvar
        pin = capi.poisson_in(w, pred)
        cin = capi.correct_in(w)
        if want_bc and bc_out is not None:
            bc = bc_out
            bc_struct = capi.ScfBcOut()
            shapes = capi.bc_plane_shapes(*self.shape)
            for f in range(4):
                for q in range(6):
                    capi.require_shape(bc[f][q], shapes[q], "BC plane")
                    bc_struct.var[f][q] = capi.dptr(bc[f][q])
        else:
            bc_struct, bc = (capi.new_bc_out(*self.shape) if want_bc else (None, None))
        st = capi.ScfStats()
        rc = self.L.scf_update_puvw(self.ctx, C.byref(pin), C.byref(cin), capi.dptr(u), capi.dptr(v),
                                    capi.dptr(ww), capi.dptr(p), C.byref(bc_struct) if want_bc else None,
                                    C.byref(st))
        self._check(rc, (capi.SCF_ERR_NOT_CONVERGED,) if allow_not_converged else ())
        return u, v, ww, p, bc, st.as_dict()

    # -- split API ---------------------------------------------------------------
    def stage(self, w, tvar=None, correction: bool = True, pred=None):
        a = w.arrays
        self._pred = pred
        self._pin = capi.poisson_in(w, pred)
        if correction:
            if tvar is None:
                tvar = [a[k] for k in ("tvar_u", "tvar_v", "tvar_w", "tvar_p")]
            self._cin = capi.correct_in(w)
            rc = self.L.scf_stage_inputs(self.ctx, C.byref(self._pin), C.byref(self._cin),
                                         *(capi.dptr(t) for t in tvar))
        else:
            rc = self.L.scf_stage_inputs(self.ctx, C.byref(self._pin), None, None, None, None, None)
        self._check(rc)

    def run(self, allow_not_converged: bool = False):
        st = capi.ScfStats()
        self._check(self.L.scf_run_projection(self.ctx, C.byref(st)),
                    (capi.SCF_ERR_NOT_CONVERGED,) if allow_not_converged else ())
        return st.as_dict()

    def fetch(self, u=None, v=None, w=None, p=None, pocoef=None, pp=None, bc=None):
        self._check(self.L.scf_fetch_outputs(self.ctx, capi.dptr(u), capi.dptr(v), capi.dptr(w), capi.dptr(p),
                                             capi.dptr(pocoef), capi.dptr(pp), C.byref(bc) if bc else None))

    # -- loss and adjoint gradient -------------------------------------------------
    def loss_forward(self, w, g, rho=None, pred=None):
        """(J_pressure, J_divergence) of the projection of workload ``w``.
        ``g``: interior weights of the pressure term; ``rho``: optional
        ghosted per-cell densities; ``pred``: optional (u*, v*, w*)."""
        self._lpin = capi.poisson_in(w, pred)
        self._lcin = capi.correct_in(w)
        self._lg = np.asfortranarray(g, dtype=np.float64)
        self._lrho = None if rho is None else np.asfortranarray(rho, dtype=np.float64)
        J = (C.c_double * 2)()
        st = capi.ScfStats()
        self._check(self.L.scf_loss_forward(self.ctx, C.byref(self._lpin), C.byref(self._lcin),
                                            capi.dptr(self._lrho), capi.dptr(self._lg),
                                            C.cast(J, capi.c_double_p), C.byref(st)))
        return float(J[0]), float(J[1]), st.as_dict()

    def loss_backward(self, shape_g):
        """Gradients of J_pressure + J_divergence: (du*, dv*, dw*, drho), ghosted."""
        out = [np.zeros(shape_g, order="F") for _ in range(4)]
        st = capi.ScfStats()
        self._check(self.L.scf_loss_backward(self.ctx, *(capi.dptr(o) for o in out), C.byref(st)))
        return out, st.as_dict()

    # -- diagnostics ---------------------------------------------------------------
    def debug_apply(self, x: np.ndarray) -> np.ndarray:
        y = np.zeros(x.shape, order="F")
        self._check(self.L.scf_debug_apply(self.ctx, capi.dptr(np.asfortranarray(x)), capi.dptr(y)))
        return y

    def time_kernel(self, kernel: int, reps: int = 20):
        """(ms per launch, algorithmic bytes per launch) of one kernel class."""
        ms, by = C.c_double(), C.c_double()
        self._check(self.L.scf_debug_time_kernel(self.ctx, int(kernel), int(reps), C.byref(ms), C.byref(by)))
        return ms.value, by.value

    def debug_precondition(self, r: np.ndarray) -> np.ndarray:
        """z = M r, one V-cycle of the last run's hierarchy (ghosted arrays)."""
        z = np.zeros_like(r, order="F")
        self._check(self.L.scf_debug_precondition(self.ctx, capi.dptr(np.asfortranarray(r)), capi.dptr(z)))
        return z

    def kernel_timing(self, enable: bool = True):
        """Starts (or stops) live per-launch timing; resets the totals."""
        self._check(self.L.scf_kernel_timing(self.ctx, 1 if enable else 0))

    def kernel_timing_read(self, kernel: int):
        """(total ms, launches, algorithmic bytes per launch) of a kernel class."""
        ms, n, by = C.c_double(), C.c_longlong(), C.c_double()
        self._check(self.L.scf_kernel_timing_read(self.ctx, int(kernel), C.byref(ms), C.byref(n), C.byref(by)))
        return ms.value, n.value, by.value

    def debug_operator(self):
        I, J, K = self.shape
        outs = [np.zeros((I, J, K), order="F") for _ in range(5)]
        self._check(self.L.scf_debug_operator(self.ctx, *(capi.dptr(o) for o in outs)))
        return dict(zip(("diag", "cpl_e", "cpl_n", "cpl_t", "rhs"), outs))

    def device_fields(self) -> dict:
        """Device pointers (ghosted FP64) of the context's u, v, w, p, phiL, vofL
        and vof (scf_ctx_device_fields), for output without a host copy."""
        ptrs = [C.c_void_p() for _ in range(7)]
        self._check(self.L.scf_ctx_device_fields(self.ctx, *(C.byref(q) for q in ptrs)))
        return dict(zip(("u", "v", "w", "p", "phil", "vofl", "vof"), (q.value for q in ptrs)))

    def debug_operator_f32(self):
        """FP32 hi/lo forms of the operator of a mixed context and the FP64
        extra diagonal part (interior arrays)."""
        I, J, K = self.shape
        names = ("diag_hi", "e_hi", "n_hi", "t_hi", "extra_hi", "diag_lo", "e_lo", "n_lo", "t_lo")
        outs = [np.zeros((I, J, K), dtype=np.float32, order="F") for _ in names]
        extra = np.zeros((I, J, K), order="F")
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        self._check(self.L.scf_debug_operator_f32(self.ctx, *(fp(o) for o in outs), capi.dptr(extra)))
        r = dict(zip(names, outs))
        r["extra"] = extra
        return r
