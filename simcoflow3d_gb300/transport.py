"""The CLSVOF interface transport on the GPU (include/scf_clsvof.h).

``ClsvofScheme`` mirrors Clsvof_Scheme (src/Clsvof.f90:355-798): one call
advances the liquid fraction ``vofl``, the level set ``phil``, the liquid
normals and the level-set wall planes of BCLvs by one time step, and
writes the VOF wall planes of BCVof.  Arrays are Fortran-ordered float64:
ghosted fields (I+2, J+2, K+2), interior grid arrays (I, J, K), wall planes
(J, K) for W/E, (I, K) for S/N, (I, J) for B/T.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, List, Sequence

import numpy as np

from . import capi

FACES = ("W", "E", "S", "N", "B", "T")


def plane_shapes(I: int, J: int, K: int):
    return [(J, K), (J, K), (I, K), (I, K), (I, J), (I, J)]


def _f64(a) -> np.ndarray:
    a = np.asarray(a)
    if a.dtype != np.float64 or not a.flags.f_contiguous:
        raise ValueError("expected a Fortran-ordered float64 array")
    return a


class ClsvofScheme:
    """Clsvof_Scheme on the GPU for one grid size (I, J, K >= 3)."""

    def __init__(self, imax: int, jmax: int, kmax: int, device: int = 0, lib=None):
        from .projection import load_library
        self.L = lib or load_library()
        self.shape = (imax, jmax, kmax)
        self.ctx = C.c_void_p()
        rc = self.L.scf_clsvof_create(C.byref(self.ctx), imax, jmax, kmax, device)
        if rc != 0:
            raise RuntimeError("scf_clsvof_create failed with status %d" % rc)

    def close(self):
        if self.ctx:
            self.L.scf_clsvof_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _err(self, rc):
        from .projection import ScfError
        buf = C.create_string_buffer(512)
        self.L.scf_clsvof_last_error(self.ctx, buf, 512)
        raise ScfError(rc, buf.value.decode(errors="replace"))

    def _in(self, centres, spacings, vel, fluid_normals, bc_vel, dt, lvs_flag, lvs_const, vof_flag, vof_const):
        I, J, K = self.shape
        arrs = [_f64(a) for a in (*centres, *spacings, *vel, *fluid_normals, *bc_vel)]
        for a in arrs[:6]:
            capi.require_shape(a, (I, J, K))
        for a in arrs[6:12]:
            capi.require_shape(a, (I + 2, J + 2, K + 2))
        for a, sh in zip(arrs[12:], ((J, K), (I, K), (I, J))):
            capi.require_shape(a, sh)
        s = capi.ScfClsvofIn(*(capi.dptr(a) for a in arrs))
        s.lvs_flag[:] = list(lvs_flag)
        s.vof_flag[:] = list(vof_flag)
        s.lvs_const[:] = [float(c) for c in lvs_const]
        s.vof_const[:] = [float(c) for c in vof_const]
        s.dt = float(dt)
        self._keep_in = arrs
        return s

    def _state(self, state: Dict[str, np.ndarray], lvs_bc: Sequence[np.ndarray], vof_bc: Sequence[np.ndarray]):
        I, J, K = self.shape
        fields = [_f64(state[k]) for k in ("vofl", "phil", "nxl", "nyl", "nzl")]
        for a in fields:
            capi.require_shape(a, (I + 2, J + 2, K + 2))
        planes = [_f64(a) for a in (*lvs_bc, *vof_bc)]
        for a, sh in zip(planes, plane_shapes(I, J, K) * 2):
            capi.require_shape(a, sh)
        s = capi.ScfClsvofState(*(capi.dptr(a) for a in fields))
        s.lvs_bc[:] = [capi.dptr(a) for a in planes[:6]]
        s.vof_bc[:] = [capi.dptr(a) for a in planes[6:]]
        self._keep_state = (fields, planes)
        return s

    def __call__(self, centres, spacings, state, vel, fluid_normals, bc_vel, lvs_bc, dt,
                 lvs_flag=(1,) * 6, lvs_const=(0.0,) * 6, vof_flag=(1,) * 6, vof_const=(0.0,) * 6,
                 vof_bc: List[np.ndarray] = None):
        """scf_clsvof_step: advances ``state`` (dict of vofl, phil, nxl, nyl,
        nzl) and ``lvs_bc`` in place; returns the VOF wall planes and the
        call's statistics."""
        I, J, K = self.shape
        if vof_bc is None:
            vof_bc = [np.zeros(sh, order="F") for sh in plane_shapes(I, J, K)]
        sin = self._in(centres, spacings, vel, fluid_normals, bc_vel, dt, lvs_flag, lvs_const, vof_flag, vof_const)
        sst = self._state(state, lvs_bc, vof_bc)
        st = capi.ScfClsvofStats()
        rc = self.L.scf_clsvof_step(self.ctx, C.byref(sin), C.byref(sst), C.byref(st))
        if rc != 0:
            self._err(rc)
        return vof_bc, st.as_dict()

    def stage(self, centres, spacings, state, vel, fluid_normals, bc_vel, lvs_bc, dt, lvs_flag=(1,) * 6,
              lvs_const=(0.0,) * 6, vof_flag=(1,) * 6, vof_const=(0.0,) * 6):
        I, J, K = self.shape
        self._vof_bc = [np.zeros(sh, order="F") for sh in plane_shapes(I, J, K)]
        sin = self._in(centres, spacings, vel, fluid_normals, bc_vel, dt, lvs_flag, lvs_const, vof_flag, vof_const)
        sst = self._state(state, lvs_bc, self._vof_bc)
        rc = self.L.scf_clsvof_stage(self.ctx, C.byref(sin), C.byref(sst))
        if rc != 0:
            self._err(rc)

    def set_timing(self, on: bool):
        """Per-kernel CUDA-event timing of run() (stats["ms_kernels"]:
        reconstruct, sweep, walls, redistancing)."""
        rc = self.L.scf_clsvof_set_timing(self.ctx, int(bool(on)))
        if rc != 0:
            self._err(rc)

    def run(self, steps: int = 1) -> dict:
        st = capi.ScfClsvofStats()
        rc = self.L.scf_clsvof_run(self.ctx, int(steps), C.byref(st))
        if rc != 0:
            self._err(rc)
        return st.as_dict()

    def fetch(self, state, lvs_bc, vof_bc=None):
        I, J, K = self.shape
        if vof_bc is None:
            vof_bc = [np.zeros(sh, order="F") for sh in plane_shapes(I, J, K)]
        sst = self._state(state, lvs_bc, vof_bc)
        st = capi.ScfClsvofStats()
        rc = self.L.scf_clsvof_fetch(self.ctx, C.byref(sst), C.byref(st))
        if rc != 0:
            self._err(rc)
        return vof_bc, st.as_dict()

    def uvw_liquid_field(self, vgrids, vcells) -> dict:
        """scf_clsvof_uvw_liquid_field (ComputeUVWLiquidField) from the P
        cells' device state after the last run or stage.  ``vgrids``: three
        (dx, dy, dz) interior arrays of the U, V, W grids; ``vcells``: three
        dicts of ghosted phil, nxl, nyl, nzl, vofl, updated in place."""
        I, J, K = self.shape
        cells = (capi.ScfClsvofVcell * 3)()
        keep = []
        for f in range(3):
            g = [_f64(a) for a in vgrids[f]]
            c = [_f64(vcells[f][k]) for k in ("phil", "nxl", "nyl", "nzl", "vofl")]
            for a in g:
                capi.require_shape(a, (I, J, K))
            for a in c:
                capi.require_shape(a, (I + 2, J + 2, K + 2))
            keep += g + c
            cells[f] = capi.ScfClsvofVcell(*(capi.dptr(a) for a in g + c))
        st = capi.ScfClsvofStats()
        rc = self.L.scf_clsvof_uvw_liquid_field(self.ctx, cells, C.byref(st))
        if rc != 0:
            self._err(rc)
        return st.as_dict()

    def device_fields(self):
        a, b = C.c_void_p(), C.c_void_p()
        rc = self.L.scf_clsvof_device_fields(self.ctx, C.byref(a), C.byref(b))
        if rc != 0:
            self._err(rc)
        return a.value, b.value
