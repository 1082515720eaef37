"""Host side of the cut-cell geometry preprocessing (include/scf_geometry.h).

``GridPreprocess`` is the reference-facing entry point: it takes the four
cell families (PCell, UCell, VCell, WCell, each with its grid) as Fortran
arrays with the reference's bounds and runs, on the GPU, the sequence
``GridPreprocess`` + ``DefineMomentumExchangeCell`` + ``NumberExternalCell``
x4 (src/Main.f90:203-214, src/SolidBody.f90:815-822), rewriting the arrays
in place like the reference's intent(inout) derived-type members.

``geometry_inputs`` builds seeded synthetic inputs for it: the solid level
set, normals and fluid fractions of each family on its own (staggered) grid,
as ``InitialClsvofFluidField`` (src/Clsvof.f90:74-131) defines them, plus
in/out arrays filled with seeded values so that untouched entries are
visible.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import Dict, Optional

import numpy as np

from . import capi
from . import workloads as W

FAMILIES = ("p", "u", "v", "w")
# arrays of one family: (name, dtype, kind); kind g = ghosted, i = interior,
# g3 / i3 = with a trailing component index 1..3, pn = PosNu bounds
FIELDS = (
    ("dx", np.float64, "i"), ("dy", np.float64, "i"), ("dz", np.float64, "i"),
    ("phi", np.float64, "g"), ("nx", np.float64, "g"), ("ny", np.float64, "g"), ("nz", np.float64, "g"),
    ("vof", np.float64, "g"), ("vofl", np.float64, "g"),
    ("cell_type", np.int32, "i"),
    ("eearea", np.float64, "g"), ("nearea", np.float64, "g"), ("tearea", np.float64, "g"),
    ("fce", np.float64, "g3"), ("fcn", np.float64, "g3"), ("fct", np.float64, "g3"),
    ("cell_cent", np.float64, "i3"), ("wllh", np.float64, "i"), ("delh", np.float64, "i"),
    ("moexcell", np.int32, "i"), ("posnu", np.int32, "pn"),
)
OUTPUTS = ("vof", "vofl", "cell_type", "eearea", "nearea", "tearea", "fce", "fcn", "fct", "cell_cent", "wllh",
           "delh", "moexcell", "posnu")
POSNU_CUT = {"p": (0, 0, 0), "u": (1, 0, 0), "v": (0, 1, 0), "w": (0, 0, 1)}


def field_shape(kind: str, fam: str, I: int, J: int, K: int):
    if kind == "g":
        return (I + 2, J + 2, K + 2)
    if kind == "g3":
        return (I + 2, J + 2, K + 2, 3)
    if kind == "i":
        return (I, J, K)
    if kind == "i3":
        return (I, J, K, 3)
    iu, iv, iw = POSNU_CUT[fam]
    return (I - iu, J - iv, K - iw)


@dataclasses.dataclass
class GeoFamily:
    """Arrays of one cell family, Fortran-ordered with the reference's bounds."""
    name: str
    arrays: Dict[str, Optional[np.ndarray]]
    ext_cell: int = -1

    def struct(self) -> capi.ScfGeoCells:
        s = capi.ScfGeoCells()
        for f, dt, _ in FIELDS:
            a = self.arrays.get(f)
            setattr(s, f, capi.iptr(a) if dt == np.int32 else capi.dptr(a))
        s.ext_cell = self.ext_cell
        return s

    def copy(self) -> "GeoFamily":
        return GeoFamily(self.name, {k: (None if v is None else v.copy(order="F")) for k, v in self.arrays.items()},
                         self.ext_cell)


@dataclasses.dataclass
class GeoInputs:
    imax: int
    jmax: int
    kmax: int
    fams: Dict[str, GeoFamily]
    meta: Dict[str, object] = dataclasses.field(default_factory=dict)

    def copy(self) -> "GeoInputs":
        return GeoInputs(self.imax, self.jmax, self.kmax, {k: f.copy() for k, f in self.fams.items()}, dict(self.meta))


def geometry_inputs(name: str = "c2", n: Optional[int] = None, seed: int = 20261203,
                    solid=None, extent=None, zstretch=None, shape=None) -> GeoInputs:
    """Synthetic geometry inputs.  ``name`` picks the geometry of a projection
    config: c1/c2 (unit cube, sphere r=0.15 at (0.5,0.5,0.3)), c4 (4x1x1 box,
    z-stretched toward z=0.5, vertical cylinder r=0.1 at (2,0.5)); ``n`` the
    cells per unit length (default 128 for c1, 256 for c2, c4's 512x256x256
    halved per n)."""
    if name in ("c1", "c2"):
        n = n or (128 if name == "c1" else 256)
        I = J = K = n
        solid = solid or W.SPHERE_C1
        extent = extent or ((0.0, 1.0), (0.0, 1.0), (0.0, 1.0))
    elif name == "c4":
        n = n or 256
        I, J, K = 2 * n, n, n
        solid = solid or ("zcylinder", 2.0, 0.5, 0.1)
        extent = extent or ((0.0, 4.0), (0.0, 1.0), (0.0, 1.0))
        zstretch = zstretch or 1.02
    else:
        I, J, K = shape
        extent = extent or ((0.0, 1.0), (0.0, 1.0), (0.0, 1.0))
    gx = W.Grid1D(W.uniform_nodes(I, *extent[0]))
    gy = W.Grid1D(W.uniform_nodes(J, *extent[1]))
    if zstretch:
        gz = W.Grid1D(W.stretched_nodes_about(K, extent[2][0], extent[2][1], 0.5 * sum(extent[2]), zstretch))
    else:
        gz = W.Grid1D(W.uniform_nodes(K, *extent[2]))
    shp = (I, J, K)
    b3 = W._bcast3
    X, Y, Z = b3(gx.c, 0, shp), b3(gy.c, 1, shp), b3(gz.c, 2, shp)
    DX, DY, DZ = b3(gx.d, 0, shp), b3(gy.d, 1, shp), b3(gz.d, 2, shp)
    centres = {
        "p": (X, Y, Z, DX, DY, DZ),
        "u": (b3(gx.c + 0.5 * gx.d, 0, shp), Y, Z, b3(gx.staggered_d(), 0, shp), DY, DZ),
        "v": (X, b3(gy.c + 0.5 * gy.d, 1, shp), Z, DX, b3(gy.staggered_d(), 1, shp), DZ),
        "w": (X, Y, b3(gz.c + 0.5 * gz.d, 2, shp), DX, DY, b3(gz.staggered_d(), 2, shp)),
    }
    rng = np.random.default_rng(seed)
    liquid = ("bubble", 0.5 * (extent[0][0] + extent[0][1]), 0.5, 0.65, 0.1)
    fams = {}
    F = lambda a: np.asfortranarray(np.array(a, dtype=np.float64))
    for fam in FAMILIES:
        xc, yc, zc, dx, dy, dz = centres[fam]
        phi, vof, nx, ny, nz = W._fluid_field(solid, xc, yc, zc, dx, dy, dz)
        _, vofl = W._liquid_field(liquid, xc, yc, zc, dx, dy, dz)
        arr: Dict[str, Optional[np.ndarray]] = {}
        arr["dx"], arr["dy"], arr["dz"] = F(np.broadcast_to(dx, shp)), F(np.broadcast_to(dy, shp)), F(np.broadcast_to(dz, shp))
        for key, val in (("phi", phi), ("nx", nx), ("ny", ny), ("nz", nz), ("vof", vof), ("vofl", vofl)):
            arr[key] = W._ghost_copy(np.broadcast_to(val, shp).astype(np.float64))
        for f, dt, kind in FIELDS:
            if f in arr:
                continue
            s = field_shape(kind, fam, I, J, K)
            if dt == np.int32:
                a = rng.integers(0, 2, size=s).astype(np.int32) if f == "moexcell" else np.full(s, 7, np.int32)
            else:
                a = rng.normal(0.0, 1.0, size=s)
            arr[f] = np.asfortranarray(a)
        if fam == "p":
            arr["moexcell"] = None   # PCell%MoExCell is not allocated in the reference
        fams[fam] = GeoFamily(fam, arr)
    return GeoInputs(I, J, K, fams, {"name": name, "solid": solid, "zstretch": zstretch})


class GridPreprocess:
    """The geometry sequence on the GPU for one grid size (a context)."""

    def __init__(self, imax: int, jmax: int, kmax: int, device: int = 0, lib=None):
        from .projection import load_library
        self.L = lib or load_library()
        self.shape = (imax, jmax, kmax)
        self.ctx = C.c_void_p()
        rc = self.L.scf_geo_create(C.byref(self.ctx), imax, jmax, kmax, device)
        if rc != 0:
            raise RuntimeError("scf_geo_create failed with status %d" % rc)

    def close(self):
        if self.ctx:
            self.L.scf_geo_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _err(self, rc):
        from .projection import ScfError
        buf = C.create_string_buffer(512)
        self.L.scf_geo_last_error(self.ctx, buf, 512)
        raise ScfError(rc, buf.value.decode(errors="replace"))

    def _structs(self, g: GeoInputs):
        return [g.fams[f].struct() for f in FAMILIES]

    def __call__(self, g: GeoInputs) -> dict:
        """Runs the sequence on ``g``'s arrays in place; returns the stats."""
        ss = self._structs(g)
        st = capi.ScfGeoStats()
        rc = self.L.scf_grid_preprocess(self.ctx, *(C.byref(s) for s in ss), C.byref(st))
        if rc != 0:
            self._err(rc)
        for f, s in zip(FAMILIES, ss):
            g.fams[f].ext_cell = s.ext_cell
        return {k: getattr(st, k) for k, _ in capi.ScfGeoStats._fields_}

    def stage(self, g: GeoInputs):
        ss = self._structs(g)
        rc = self.L.scf_geo_stage(self.ctx, *(C.byref(s) for s in ss))
        if rc != 0:
            self._err(rc)

    def run(self) -> dict:
        st = capi.ScfGeoStats()
        rc = self.L.scf_geo_run(self.ctx, C.byref(st))
        if rc != 0:
            self._err(rc)
        return {k: getattr(st, k) for k, _ in capi.ScfGeoStats._fields_}

    def fetch(self, g: GeoInputs):
        ss = self._structs(g)
        rc = self.L.scf_geo_fetch(self.ctx, *(C.byref(s) for s in ss))
        if rc != 0:
            self._err(rc)
        for f, s in zip(FAMILIES, ss):
            g.fams[f].ext_cell = s.ext_cell
