"""Synthetic projection workloads in SIMCOFlow's own array layout.

Every array here is laid out exactly as the Fortran host holds it: column-major
(``i`` fastest), cell arrays ghosted ``(0:I+1, 0:J+1, 0:K+1)`` where the
reference allocates them with ghosts (``src/Test/Dambreak/Dambreak.f90:228-413``)
and ``(1:I, 1:J, 1:K)`` otherwise.  In numpy that is a Fortran-ordered array of
shape ``(I+2, J+2, K+2)`` or ``(I, J, K)``.

The geometry follows the reference's own construction so the hot path sees
inputs of the kind SIMCOFlow produces:

* grids: cell-centred tensor grids (``Mesh.f90:34-158``) and the staggered
  spacings of ``InitialUVGrid`` (``Mesh.f90:160-247``);
* solid: signed distance ``phi`` (positive in fluid) and the fluid fraction
  from ``Volume_Fraction_Calc`` (``Clsvof.f90:74-131,1475-1550``);
* liquid: ``phiL`` (negative in liquid) and ``vofL`` as in
  ``Test/FlowSphere2Phases/InitialVof.f90:25-70``;
* ``DefineCell`` (``CutCell.f90:329-365``), the P-cell face apertures of
  ``CellGeoCal`` (``CutCell.f90:369-671``, via ``FaceGeoCal`` 883-981), the
  aperture override of ``GridPreprocess`` (``CutCell.f90:258-327``),
  ``DefineMomentumExchangeCell`` (673-749) and ``NumberExternalCell`` (753-786);
* ``Dp`` of the momentum predictor with no viscous terms
  (``PredictUVW.f90:907,1029-1037,1235-1246``) and its ghost copies (778-800).

Velocities are seeded N(0, 0.1^2) fields smoothed by three Jacobi passes, with
the wall-normal component zeroed on Neumann-pressure walls.

Ghost cells of the solid and liquid fields copy the adjacent interior cell
(the clamped-index construction of ``InitialVof.f90:39-45``).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, Optional, Tuple

import numpy as np

EPSI = 1.0e-3          # CutCell.f90:11
ROW = 998.3            # StateVariables.f90:9 (water density)
ROA = 1.205            # StateVariables.f90:9 (air density)
DEFAULT_SEED = 20261203

# Face order used by BC arrays and flags: W, E, S, N, B, T
# (BoundaryFunction.f90:48-59).
FACES = ("W", "E", "S", "N", "B", "T")


# ---------------------------------------------------------------------------
# geometric primitives (vectorised restatements)
# ---------------------------------------------------------------------------

def volume_fraction_calc(dx, dy, dz, nxx, nyy, nzz, s):
    """Volume of the box on the positive side of a plane.

    Restates ``Volume_Fraction_Calc`` (``Clsvof.f90:1475-1550``, the
    Griebel-Klitz formula) element-wise.  Returns the volume (not the fraction).
    Boxes entirely on one side (s <= 0 or s >= sm) take the reference's early
    returns; only cut boxes evaluate the polynomial branches.
    """
    dx, dy, dz, nxx, nyy, nzz, s = (np.ascontiguousarray(a) for a in np.broadcast_arrays(
        *(np.asarray(a, dtype=np.float64) for a in (dx, dy, dz, nxx, nyy, nzz, s))))
    shape = s.shape
    a, b, c = np.abs(nxx) * dx, np.abs(nyy) * dy, np.abs(nzz) * dz
    sm = (a + b + c)
    vbox = dx * dy * dz
    vol = np.where(s >= sm, vbox, 0.0)
    cut = (s > 0.0) & (s < sm)
    idx = np.nonzero(cut.ravel())[0]
    if idx.size:
        g = lambda v: v.ravel()[idx]
        a, b, c, S, VB = g(a), g(b), g(c), g(s), g(vbox)
        dx1 = np.maximum(np.maximum(a, b), c)
        dz1 = np.minimum(np.minimum(a, b), c)
        dy1 = (a + b + c) - dx1 - dz1
        smc = dx1 + dy1 + dz1
        sc = np.minimum(S, smc - S)
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            f1 = sc ** 3 / (6.0 * dx1 * dy1 * dz1)
            f2 = (sc ** 2 - dz1 * sc + dz1 ** 2 / 3.0) / (2.0 * dx1 * dy1)
            f3 = (2.0 * sc - dy1 - dz1) / (2.0 * dx1)
            f4 = (sc ** 3 - (sc - dz1) ** 3 - (sc - dy1) ** 3) / (6.0 * dx1 * dy1 * dz1)
            f5 = (sc ** 3 - (sc - dz1) ** 3 - (sc - dy1) ** 3 - (sc - dx1) ** 3) / (6.0 * dx1 * dy1 * dz1)
        fc = np.where(sc <= dz1, f1,
             np.where(sc <= dy1, f2,
             np.where(dx1 >= dy1 + dz1,
                      np.where(sc >= dy1 + dz1, f3, f4),
                      np.where(sc > dx1, f5, f4))))
        vcut = np.where(S <= 0.5 * smc, fc * VB, (1.0 - fc) * VB)
        vcut = np.where(S >= smc, VB, vcut)
        flat = vol.ravel().copy()
        flat[idx] = vcut
        vol = flat.reshape(shape)
    return vol


def face_geo_area(d1, d2, n1, n2, n3, d3, phi):
    """Open fraction of one rectangular cell face.

    Restates the area part of ``FaceGeoCal`` (``CutCell.f90:883-981``): the
    face polygon is clipped by the plane ``n.x + phi = 0`` (positive side open)
    and its shoelace area is divided by ``d1*d2``.  Only faces whose corners
    change sign go through the polygon; fully open faces give exactly 1 and
    fully closed faces 0, as the reference's polygon does.
    """
    d1, d2, n1, n2, n3, d3, phi = (np.ascontiguousarray(a) for a in np.broadcast_arrays(
        *(np.asarray(a, dtype=np.float64) for a in (d1, d2, n1, n2, n3, d3, phi))))
    shape = d1.shape
    d11 = d1 / 2.0
    d22 = d2 / 2.0
    t = d3 * n3
    dpt1 = d11 * n1 - d22 * n2 + t + phi
    dpt2 = -d11 * n1 - d22 * n2 + t + phi
    dpt3 = -d11 * n1 + d22 * n2 + t + phi
    dpt4 = d11 * n1 + d22 * n2 + t + phi
    anypos = (dpt1 > 0) | (dpt2 > 0) | (dpt3 > 0) | (dpt4 > 0)
    allpos = (dpt1 > 0) & (dpt2 > 0) & (dpt3 > 0) & (dpt4 > 0)
    area = np.where(allpos, 1.0, 0.0)
    cut = anypos & ~allpos
    # Sign changes without a positive corner cannot happen; nodes exist only
    # where some corner is open.
    idx = np.nonzero(cut.ravel())[0]
    if idx.size == 0:
        return area
    g = lambda a: a.ravel()[idx]
    D11, D22, N1, N2, N3, D3, PHI = (g(a) for a in (d11, d22, n1, n2, n3, d3, phi))
    P1, P2, P3, P4 = (g(a) for a in (dpt1, dpt2, dpt3, dpt4))
    T = D3 * N3
    with np.errstate(divide="ignore", invalid="ignore"):
        cand = [
            (P1 > 0, D11, -D22),
            (P1 * P2 < 0, (D22 * N2 - T - PHI) / N1, -D22),
            (P2 > 0, -D11, -D22),
            (P2 * P3 < 0, -D11, (D11 * N1 - T - PHI) / N2),
            (P3 > 0, -D11, D22),
            (P3 * P4 < 0, (-D22 * N2 - T - PHI) / N1, D22),
            (P4 > 0, D11, D22),
            (P4 * P1 < 0, D11, (-D11 * N1 - T - PHI) / N2),
        ]
    m = idx.size
    vol = np.zeros(m)
    have = np.zeros(m, dtype=bool)
    px = np.zeros(m); py = np.zeros(m)
    fx = np.zeros(m); fy = np.zeros(m)
    for valid, x, y in cand:
        x = np.where(valid, x, 0.0)
        y = np.where(valid, y, 0.0)
        add = valid & have
        vol = np.where(add, vol + 0.5 * (px * y - x * py), vol)
        first = valid & ~have
        fx = np.where(first, x, fx); fy = np.where(first, y, fy)
        px = np.where(valid, x, px); py = np.where(valid, y, py)
        have = have | valid
    vol = np.where(have, vol + 0.5 * (px * fy - fx * py), vol)
    a_cut = np.abs(vol / ((2.0 * D11) * (2.0 * D22)))
    flat = area.ravel().copy()
    flat[idx] = a_cut
    return flat.reshape(shape)


# ---------------------------------------------------------------------------
# grids
# ---------------------------------------------------------------------------

def uniform_nodes(n: int, lo: float, hi: float) -> np.ndarray:
    return lo + (hi - lo) * np.arange(n + 1, dtype=np.float64) / n


def stretched_nodes_about(n: int, lo: float, hi: float, centre: float, ratio: float) -> np.ndarray:
    """Nodes with a uniform band of n/2 cells around ``centre`` and n/4 cells
    on each side growing geometrically by ``ratio`` (a geometric stretching in
    the style of ``Mesh.f90:34-158``).  Requires the centre at mid-domain."""
    nb = n // 2
    ns = (n - nb) // 2
    assert nb + 2 * ns == n
    growth = sum(ratio ** m for m in range(1, ns + 1))
    d0 = (hi - lo) / (nb + 2.0 * growth)
    widths = [d0 * ratio ** (ns - m + 1) for m in range(1, ns + 1)]
    widths += [d0] * nb
    widths += [d0 * ratio ** m for m in range(1, ns + 1)]
    nodes = np.empty(n + 1)
    nodes[0] = lo
    nodes[1:] = lo + np.cumsum(widths)
    nodes[-1] = hi
    return nodes


@dataclasses.dataclass
class Grid1D:
    """Cell-centred 1-D grid: node coordinates and centres."""
    nodes: np.ndarray

    @property
    def n(self) -> int:
        return self.nodes.size - 1

    @property
    def d(self) -> np.ndarray:
        return self.nodes[1:] - self.nodes[:-1]

    @property
    def c(self) -> np.ndarray:
        return 0.5 * (self.nodes[1:] + self.nodes[:-1])

    def staggered_d(self) -> np.ndarray:
        """UGrid%dx of ``InitialUVGrid``: distance between neighbouring centres,
        the last cell keeps its own width (``Mesh.f90:181-185``)."""
        c = self.c
        out = self.d.copy()
        out[:-1] = c[1:] - c[:-1]
        return out


def _bcast3(a1, axis, shape):
    s = [1, 1, 1]
    s[axis] = -1
    return np.broadcast_to(np.asarray(a1).reshape(s), shape)


def _ghost_index(n):
    """Indices 0..n+1 clamped to interior 1..n, as 0-based interior positions."""
    return np.clip(np.arange(n + 2) - 1, 0, n - 1)


# ---------------------------------------------------------------------------
# workload container
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class Workload:
    """All inputs of one projection call, in the reference's array layout."""
    name: str
    imax: int
    jmax: int
    kmax: int
    dt: float
    rho_l: float
    rho_g: float
    arrays: Dict[str, np.ndarray]
    bcp_flag: Tuple[int, ...]
    bcu_flag: Tuple[int, ...]
    bcv_flag: Tuple[int, ...]
    bcw_flag: Tuple[int, ...]
    bcu_const: Tuple[float, ...]
    bcv_const: Tuple[float, ...]
    bcw_const: Tuple[float, ...]
    bcp_const: Tuple[float, ...]
    ext_cell: int
    meta: Dict[str, object] = dataclasses.field(default_factory=dict)

    @property
    def shape_g(self):
        return (self.imax + 2, self.jmax + 2, self.kmax + 2)

    @property
    def shape_i(self):
        return (self.imax, self.jmax, self.kmax)

    @property
    def ncells(self) -> int:
        return self.imax * self.jmax * self.kmax

    def copy(self) -> "Workload":
        w = dataclasses.replace(self)
        w.arrays = {k: v.copy(order="F") for k, v in self.arrays.items()}
        w.meta = dict(self.meta)
        return w


# ---------------------------------------------------------------------------
# geometry builders
# ---------------------------------------------------------------------------

def _fluid_field(solid, xc, yc, zc, dx, dy, dz):
    """phi, vof, normals of the fluid (non-solid) region on one grid.

    ``solid`` is None (no solid), ("sphere", cx, cy, cz, r) or
    ("zcylinder", cx, cy, r).  Mirrors ``InitialClsvofFluidField``
    (``Clsvof.f90:74-131``): phi = signed distance positive in fluid, normal
    pointing into the fluid, vof from ``Volume_Fraction_Calc``.
    """
    shape = np.broadcast_shapes(xc.shape, yc.shape, zc.shape)
    if solid is None:
        ones = np.ones(shape)
        return (np.full(shape, 1.0e3), ones.copy(), np.zeros(shape), np.zeros(shape), ones.copy())
    kind = solid[0]
    tiny = 1.0e-40
    if kind == "sphere":
        _, cx, cy, cz, r = solid
        ddx, ddy, ddz = xc - cx, yc - cy, zc - cz
        rr = np.sqrt(ddx ** 2 + ddy ** 2 + ddz ** 2)
        dis = rr - r
        nrm = np.sqrt(ddx ** 2 + ddy ** 2 + ddz ** 2 + tiny)
        nx, ny, nz = ddx / nrm, ddy / nrm, ddz / nrm
    elif kind == "xslab":
        # solid for x < x0 (a wall of solid cells at the west boundary)
        _, x0 = solid
        dis = np.broadcast_to(xc - x0, shape) + np.zeros(shape)
        nx, ny, nz = np.ones(shape), np.zeros(shape), np.zeros(shape)
    elif kind == "zcylinder":
        _, cx, cy, r = solid
        ddx, ddy = xc - cx, yc - cy
        ddz = np.zeros(shape)
        rr = np.sqrt(ddx ** 2 + ddy ** 2)
        dis = rr - r + np.zeros(shape)
        nrm = np.sqrt(ddx ** 2 + ddy ** 2 + tiny)
        nx, ny, nz = ddx / nrm + 0 * ddz, ddy / nrm + 0 * ddz, ddz
    else:
        raise ValueError(kind)
    nx, ny, nz, dis = (np.broadcast_to(a, shape) for a in (nx, ny, nz, dis))
    s = dis + 0.5 * (np.abs(nx) * dx + np.abs(ny) * dy + np.abs(nz) * dz)
    vol = volume_fraction_calc(dx, dy, dz, nx, ny, nz, s)
    vof = vol / (dx * dy * dz)
    return (np.array(dis), np.array(vof), np.array(nx), np.array(ny), np.array(nz))


def _liquid_field(liquid, xc, yc, zc, dx, dy, dz):
    """phiL (negative in liquid) and vofL (liquid fraction of the box)."""
    shape = np.broadcast_shapes(xc.shape, yc.shape, zc.shape)
    kind = liquid[0]
    if kind == "surface":
        # z = z0 + h(x, y); liquid below.  phiL = (z - h)/|grad|
        _, h, hx, hy = liquid
        hv, hxv, hyv = h(xc, yc), hx(xc, yc), hy(xc, yc)
        g = np.sqrt(1.0 + hxv ** 2 + hyv ** 2)
        phi = (zc - hv) / g
        nx, ny, nz = -hxv / g, -hyv / g, 1.0 / g
    elif kind == "bubble":
        # gas sphere in liquid: phiL = r - |x - c| (positive in gas)
        _, cx, cy, cz, r = liquid
        ddx, ddy, ddz = xc - cx, yc - cy, zc - cz
        rr = np.sqrt(ddx ** 2 + ddy ** 2 + ddz ** 2)
        phi = r - rr
        nrm = np.sqrt(ddx ** 2 + ddy ** 2 + ddz ** 2 + 1.0e-40)
        nx, ny, nz = -ddx / nrm, -ddy / nrm, -ddz / nrm
    else:
        raise ValueError(kind)
    phi, nx, ny, nz = (np.broadcast_to(np.asarray(a, dtype=np.float64), shape) for a in (phi, nx, ny, nz))
    s = phi + 0.5 * (np.abs(nx) * dx + np.abs(ny) * dy + np.abs(nz) * dz)
    vol = volume_fraction_calc(dx, dy, dz, nx, ny, nz, s)
    vofl = 1.0 - vol / (dx * dy * dz)
    return np.array(phi), np.array(vofl)


def _define_cell(vof, vofl):
    """``DefineCell`` (``CutCell.f90:329-365``) on interior arrays.  Returns
    (cell_type, vof, vofL) with the reference's in-place modifications."""
    vof = vof.copy()
    vofl = vofl.copy()
    ct = np.zeros(vof.shape, dtype=np.int32)
    full = vof >= 1.0 - EPSI
    ct[full] = 0
    with np.errstate(divide="ignore", invalid="ignore"):
        vofl = np.where(full, vofl / np.where(full, vof, 1.0), vofl)
    vof = np.where(full, 1.0, vof)
    gas = vof <= EPSI
    ct[gas] = 2
    vof = np.where(gas, 0.0, vof)
    vofl = np.where(gas, 0.0, vofl)
    cut = (vof >= EPSI) & (vof <= 1.0 - EPSI)
    ct[cut] = 1
    return ct, vof, vofl


def _ghost_copy(interior: np.ndarray) -> np.ndarray:
    """Ghosted Fortran array whose ghost layer copies the adjacent interior."""
    I, J, K = interior.shape
    gi, gj, gk = _ghost_index(I), _ghost_index(J), _ghost_index(K)
    out = interior[np.ix_(gi, gj, gk)]
    return np.asfortranarray(out)


def _cell_geo_areas(dx, dy, dz, nx, ny, nz, phi, ct):
    """P-cell apertures of ``CellGeoCal`` (``CutCell.f90:369-671``).

    Returns ghosted EEArea, NEArea, TEArea (initialised to 1 like the
    reference, lines 398-400)."""
    I, J, K = ct.shape
    te = face_geo_area(dx, dy, nx, ny, nz, dz / 2.0, phi)
    be = face_geo_area(dx, dy, nx, ny, nz, -dz / 2.0, phi)
    ee = face_geo_area(dy, dz, ny, nz, nx, dx / 2.0, phi)
    we = face_geo_area(dy, dz, ny, nz, nx, -dx / 2.0, phi)
    ne = face_geo_area(dz, dx, nz, nx, ny, dy / 2.0, phi)
    se = face_geo_area(dz, dx, nz, nx, ny, -dy / 2.0, phi)
    tol = 1.0e-20
    # wetted solid area of each cell (CutCell.f90:455-462), before sharing
    wllh = np.sqrt(((ee - we) * dy * dz) ** 2 + ((ne - se) * dx * dz) ** 2 + ((te - be) * dx * dy) ** 2)
    EE = np.ones((I + 2, J + 2, K + 2), order="F")
    NE = np.ones((I + 2, J + 2, K + 2), order="F")
    TE = np.ones((I + 2, J + 2, K + 2), order="F")
    EE[1:I + 1, 1:J + 1, 1:K + 1] = ee
    NE[1:I + 1, 1:J + 1, 1:K + 1] = ne
    TE[1:I + 1, 1:J + 1, 1:K + 1] = te
    # shared faces (lines 474-531): face between cells i-1 and i, i = 2..I
    a, b = we[1:, :, :], ee[:-1, :, :]
    EE[1:I, 1:J + 1, 1:K + 1] = (a ** 2 + b ** 2) / (a + b + tol)
    a, b = se[:, 1:, :], ne[:, :-1, :]
    NE[1:I + 1, 1:J, 1:K + 1] = (a ** 2 + b ** 2) / (a + b + tol)
    a, b = be[:, :, 1:], te[:, :, :-1]
    TE[1:I + 1, 1:J + 1, 1:K] = (a ** 2 + b ** 2) / (a + b + tol)
    # solid faces (lines 548-578)
    solid = np.zeros((I + 2, J + 2, K + 2), dtype=bool)
    solid[1:I + 1, 1:J + 1, 1:K + 1] = ct == 2
    s = solid[1:I + 1, 1:J + 1, 1:K + 1]
    EE[1:I + 1, 1:J + 1, 1:K + 1][s] = 0.0
    EE[0:I, 1:J + 1, 1:K + 1][s] = 0.0
    NE[1:I + 1, 1:J + 1, 1:K + 1][s] = 0.0
    NE[1:I + 1, 0:J, 1:K + 1][s] = 0.0
    TE[1:I + 1, 1:J + 1, 1:K + 1][s] = 0.0
    TE[1:I + 1, 1:J + 1, 0:K][s] = 0.0
    cut = ct == 1
    m = cut[:-1, :, :] & (ct[1:, :, :] == 2)
    EE[1:I, 1:J + 1, 1:K + 1][m] = 0.0
    m = cut[:, :-1, :] & (ct[:, 1:, :] == 2)
    NE[1:I + 1, 1:J, 1:K + 1][m] = 0.0
    m = cut[:, :, :-1] & (ct[:, :, 1:] == 2)
    TE[1:I + 1, 1:J + 1, 1:K][m] = 0.0
    return EE, NE, TE, wllh


def _staggered_vof(solid, xs, ys, zs, dxs, dys, dzs):
    if solid is None:
        return np.ones(np.broadcast_shapes(xs.shape, ys.shape, zs.shape))
    _, vof, _, _, _ = _fluid_field(solid, xs, ys, zs, dxs, dys, dzs)
    return vof


def _number_external_cell(ct):
    """``NumberExternalCell(0,0,0,PCell)`` (``CutCell.f90:753-786``): active
    cells numbered in loop order (``i`` outer, ``k`` innermost)."""
    act_loop = np.transpose(ct != 2, (0, 1, 2))  # (I,J,K), loop order = C order
    flat = act_loop.ravel(order="C")
    pos = np.cumsum(flat) - 1
    posnu = np.where(flat, pos, -1).astype(np.int32).reshape(ct.shape, order="C")
    return np.asfortranarray(posnu), int(flat.sum()) - 1


def _dp_field(ct_vel, vof_vel, dx, dy, dz, dt, axis):
    """``PUVW%Dp`` with no viscous/convective terms (``PredictUVW.f90:907,
    1029-1037,1235-1246``) plus the ghost copies of lines 778-800."""
    I, J, K = ct_vel.shape
    dp = np.zeros((I + 2, J + 2, K + 2), order="F")
    vol = dx * dy * dz
    with np.errstate(divide="ignore", invalid="ignore"):
        aP = vof_vel * vol / dt
        inner = 1.0 / aP
        val = vof_vel * dx * dy * dz * inner
    val = np.where(ct_vel != 2, val, 0.0)
    lim = [I, J, K]
    lim[axis] -= 1
    sub = np.zeros((I, J, K))
    sub[:lim[0], :lim[1], :lim[2]] = val[:lim[0], :lim[1], :lim[2]]
    dp[1:I + 1, 1:J + 1, 1:K + 1] = sub
    # ghost copies in the reference's order (PredictUVW.f90:778-800)
    if axis == 0:
        dp[0, :, :] = dp[1, :, :]
        dp[I, :, :] = dp[I - 1, :, :]
        dp[I + 1, :, :] = dp[I, :, :]
        dp[:, 0, :] = dp[:, 1, :]
        dp[:, J + 1, :] = dp[:, J, :]
        dp[:, :, 0] = dp[:, :, 1]
        dp[:, :, K + 1] = dp[:, :, K]
    elif axis == 1:
        dp[0, :, :] = dp[1, :, :]
        dp[I + 1, :, :] = dp[I, :, :]
        dp[:, 0, :] = dp[:, 1, :]
        dp[:, J, :] = dp[:, J - 1, :]
        dp[:, J + 1, :] = dp[:, J, :]
        dp[:, :, 0] = dp[:, :, 1]
        dp[:, :, K + 1] = dp[:, :, K]
    else:
        dp[0, :, :] = dp[1, :, :]
        dp[I + 1, :, :] = dp[I, :, :]
        dp[:, 0, :] = dp[:, 1, :]
        dp[:, J + 1, :] = dp[:, J, :]
        dp[:, :, 0] = dp[:, :, 1]
        dp[:, :, K] = dp[:, :, K - 1]
        dp[:, :, K + 1] = dp[:, :, K]
    return dp


def _smoothed_velocity(rng, shape_g, sigma=0.1, passes=3):
    """i.i.d. N(0, sigma^2) ghosted field, then ``passes`` Jacobi passes
    (6-neighbour average of the interior, ghosts copying the interior)."""
    f = np.asfortranarray(rng.normal(0.0, sigma, size=shape_g))
    for _ in range(passes):
        f[0, :, :] = f[1, :, :]; f[-1, :, :] = f[-2, :, :]
        f[:, 0, :] = f[:, 1, :]; f[:, -1, :] = f[:, -2, :]
        f[:, :, 0] = f[:, :, 1]; f[:, :, -1] = f[:, :, -2]
        g = f.copy(order="F")
        g[1:-1, 1:-1, 1:-1] = (f[:-2, 1:-1, 1:-1] + f[2:, 1:-1, 1:-1] + f[1:-1, :-2, 1:-1]
                               + f[1:-1, 2:, 1:-1] + f[1:-1, 1:-1, :-2] + f[1:-1, 1:-1, 2:]) / 6.0
        f = g
    f[0, :, :] = f[1, :, :]; f[-1, :, :] = f[-2, :, :]
    f[:, 0, :] = f[:, 1, :]; f[:, -1, :] = f[:, -2, :]
    f[:, :, 0] = f[:, :, 1]; f[:, :, -1] = f[:, :, -2]
    return f


def _consistent_velocity(us, vs, ws, bcp_flag, ct_u, ct_v, ct_w):
    """Wall-normal velocity zero on Neumann-pressure walls and no velocity in
    solid velocity cells (in place)."""
    I, J, K = us.shape[0] - 2, us.shape[1] - 2, us.shape[2] - 2
    if bcp_flag[0] == 1: us[0, :, :] = 0.0
    if bcp_flag[1] == 1: us[I, :, :] = 0.0; us[I + 1, :, :] = 0.0
    if bcp_flag[2] == 1: vs[:, 0, :] = 0.0
    if bcp_flag[3] == 1: vs[:, J, :] = 0.0; vs[:, J + 1, :] = 0.0
    if bcp_flag[4] == 1: ws[:, :, 0] = 0.0
    if bcp_flag[5] == 1: ws[:, :, K] = 0.0; ws[:, :, K + 1] = 0.0
    us[1:-1, 1:-1, 1:-1][ct_u == 2] = 0.0
    vs[1:-1, 1:-1, 1:-1][ct_v == 2] = 0.0
    ws[1:-1, 1:-1, 1:-1][ct_w == 2] = 0.0


def perturbed_prediction(w, seed: int, amp: float = 0.1):
    """(u*, v*, w*) of workload ``w`` plus ``amp`` times a fresh seeded field
    of the same kind (N(0, 0.1^2), three Jacobi passes), made consistent with
    the walls and the solid like the original: the next call of a sequence of
    projections on a fixed geometry."""
    rng = np.random.default_rng(seed)
    a = w.arrays
    out = []
    for key in ("u_star", "v_star", "w_star"):
        out.append(np.asfortranarray(a[key] + amp * _smoothed_velocity(rng, w.shape_g)))
    _consistent_velocity(*out, w.bcp_flag, a["ucell_cell_type"], a["vcell_cell_type"], a["wcell_cell_type"])
    return tuple(out)


class PredictionSequence:
    """Seeded predictions for a sequence of calls on one geometry, cheap at
    full size: call c gets the workload's (u*, v*, w*) plus ``amp`` times a
    combination of ``pool`` smoothed fields (generated once) with N(0, 1/pool)
    coefficients drawn from seed + c, made consistent with walls and solid."""

    def __init__(self, w, seed: int, pool: int = 4, amp: float = 0.1):
        self.w, self.seed, self.amp = w, seed, amp
        rng = np.random.default_rng(seed)
        self.fields = [[_smoothed_velocity(rng, w.shape_g) for _ in range(3)] for _ in range(pool)]

    def __call__(self, call: int):
        a = self.w.arrays
        xi = np.random.default_rng(self.seed + 1 + call).normal(0.0, 1.0 / np.sqrt(len(self.fields)),
                                                                 size=len(self.fields))
        out = []
        for comp, key in enumerate(("u_star", "v_star", "w_star")):
            f = a[key].copy(order="F")
            for m, fm in enumerate(self.fields):
                f += (self.amp * xi[m]) * fm[comp]
            out.append(f)
        _consistent_velocity(*out, self.w.bcp_flag, a["ucell_cell_type"], a["vcell_cell_type"],
                             a["wcell_cell_type"])
        return tuple(out)


def build_workload(name: str, imax: int, jmax: int, kmax: int, *,
                   extent=((0.0, 1.0), (0.0, 1.0), (0.0, 1.0)),
                   zstretch: Optional[float] = None,
                   solid=None, liquid=("surface",), rho_l=1000.0, rho_g=1.2,
                   bcp_flag=(1, 1, 1, 1, 1, 1), dt=1.0e-3, seed=DEFAULT_SEED,
                   perturb_vof_old: float = 0.0, random_tvar: bool = False) -> Workload:
    I, J, K = imax, jmax, kmax
    gx = Grid1D(uniform_nodes(I, *extent[0]))
    gy = Grid1D(uniform_nodes(J, *extent[1]))
    if zstretch:
        gz = Grid1D(stretched_nodes_about(K, extent[2][0], extent[2][1], 0.5 * sum(extent[2]), zstretch))
    else:
        gz = Grid1D(uniform_nodes(K, *extent[2]))
    shp = (I, J, K)
    X = _bcast3(gx.c, 0, shp); Y = _bcast3(gy.c, 1, shp); Z = _bcast3(gz.c, 2, shp)
    DX = _bcast3(gx.d, 0, shp); DY = _bcast3(gy.d, 1, shp); DZ = _bcast3(gz.d, 2, shp)
    udx = _bcast3(gx.staggered_d(), 0, shp)
    vdy = _bcast3(gy.staggered_d(), 1, shp)
    wdz = _bcast3(gz.staggered_d(), 2, shp)
    F = lambda a: np.asfortranarray(np.array(a, dtype=np.float64))

    # --- solid (fluid fraction) on P cells
    phi, vof, nx, ny, nz = _fluid_field(solid, X, Y, Z, DX, DY, DZ)
    # --- liquid on ghosted P cells (clamped coordinates, InitialVof.f90:39-45)
    gi, gj, gk = _ghost_index(I), _ghost_index(J), _ghost_index(K)
    shg = (I + 2, J + 2, K + 2)
    Xg = _bcast3(gx.c[gi], 0, shg); Yg = _bcast3(gy.c[gj], 1, shg); Zg = _bcast3(gz.c[gk], 2, shg)
    DXg = _bcast3(gx.d[gi], 0, shg); DYg = _bcast3(gy.d[gj], 1, shg); DZg = _bcast3(gz.d[gk], 2, shg)
    phil_g, vofl_g = _liquid_field(liquid, Xg, Yg, Zg, DXg, DYg, DZg)
    vofl_int = vofl_g[1:-1, 1:-1, 1:-1]
    ct, vof_d, vofl_d = _define_cell(vof, vofl_int)
    vofl_g = np.array(vofl_g)
    vofl_g[1:-1, 1:-1, 1:-1] = vofl_d
    vof_g = _ghost_copy(vof_d)
    EE, NE, TE, wllh = _cell_geo_areas(DX, DY, DZ, nx, ny, nz, phi, ct)

    # --- staggered velocity cells
    xs_u = _bcast3(gx.c + 0.5 * gx.d, 0, shp)
    ys_v = _bcast3(gy.c + 0.5 * gy.d, 1, shp)
    zs_w = _bcast3(gz.c + 0.5 * gz.d, 2, shp)
    vof_u = _staggered_vof(solid, xs_u, Y, Z, udx, DY, DZ)
    vof_v = _staggered_vof(solid, X, ys_v, Z, DX, vdy, DZ)
    vof_w = _staggered_vof(solid, X, Y, zs_w, DX, DY, wdz)
    zero = np.zeros(shp)
    ct_u, vof_u, _ = _define_cell(np.broadcast_to(vof_u, shp), zero)
    ct_v, vof_v, _ = _define_cell(np.broadcast_to(vof_v, shp), zero)
    ct_w, vof_w, _ = _define_cell(np.broadcast_to(vof_w, shp), zero)

    # GridPreprocess aperture override from the U/V/W fluid fractions
    # (CutCell.f90:258-327): cut velocity cell keeps CellGeoCal's value.
    for A, vv in ((EE, vof_u), (NE, vof_v), (TE, vof_w)):
        inner = A[1:-1, 1:-1, 1:-1]
        keep = (vv < 1.0) & (vv > 0.0)
        inner[...] = np.where(keep, inner, np.where(vv > 0.5, 1.0, 0.0))

    # DefineMomentumExchangeCell (CutCell.f90:673-749)
    solidP = ct == 2
    def moex(ctv, axis):
        m = np.zeros(shp, dtype=np.int32)
        nb = np.zeros(shp, dtype=bool)
        sl = [slice(None)] * 3
        sl[axis] = slice(0, shp[axis] - 1)
        sl2 = [slice(None)] * 3
        sl2[axis] = slice(1, None)
        nb[tuple(sl)] = solidP[tuple(sl2)]
        m[(ctv == 1) & (solidP | nb)] = 1
        return np.asfortranarray(m)
    moex_u, moex_v, moex_w = moex(ct_u, 0), moex(ct_v, 1), moex(ct_w, 2)

    posnu, ext_cell = _number_external_cell(ct)

    # Dp of the predictor
    dp_u = _dp_field(ct_u, vof_u, udx, DY, DZ, dt, 0)
    dp_v = _dp_field(ct_v, vof_v, DX, vdy, DZ, dt, 1)
    dp_w = _dp_field(ct_w, vof_w, DX, DY, wdz, dt, 2)

    # predicted velocity u*
    rng = np.random.default_rng(seed)
    us = _smoothed_velocity(rng, shg)
    vs = _smoothed_velocity(rng, shg)
    ws = _smoothed_velocity(rng, shg)
    _consistent_velocity(us, vs, ws, bcp_flag, ct_u, ct_v, ct_w)

    vof_old = vof_g.copy(order="F")
    if perturb_vof_old:
        pert = rng.uniform(-perturb_vof_old, perturb_vof_old, size=shg)
        mask = np.zeros(shg, dtype=bool)
        mask[1:-1, 1:-1, 1:-1] = ct == 1
        vof_old = np.asfortranarray(np.where(mask, np.clip(vof_g + pert, 0.0, 1.0), vof_g))

    if random_tvar:
        tu = np.asfortranarray(rng.normal(0, 0.1, shg)); tv = np.asfortranarray(rng.normal(0, 0.1, shg))
        tw = np.asfortranarray(rng.normal(0, 0.1, shg)); tp = np.asfortranarray(rng.normal(0, 1.0, shg))
    else:
        tu, tv, tw = us.copy(order="F"), vs.copy(order="F"), ws.copy(order="F")
        tp = np.zeros(shg, order="F")

    # BCp boundary arrays (SetConstant(0): Var* = 0)
    arrays = {
        "pgrid_dx": F(DX), "pgrid_dy": F(DY), "pgrid_dz": F(DZ),
        "ugrid_dx": F(udx), "vgrid_dy": F(vdy), "wgrid_dz": F(wdz),
        "phil": F(phil_g), "vofl": F(vofl_g), "vof": F(vof_g),
        "eearea": F(EE), "nearea": F(NE), "tearea": F(TE),
        "cell_type": np.asfortranarray(ct.astype(np.int32)), "posnu": posnu,
        "vof_old": F(vof_old),
        "u_star": F(us), "v_star": F(vs), "w_star": F(ws),
        "dp_u": dp_u, "dp_v": dp_v, "dp_w": dp_w,
        "bcp_var_w": np.zeros((J, K), order="F"), "bcp_var_e": np.zeros((J, K), order="F"),
        "bcp_var_s": np.zeros((I, K), order="F"), "bcp_var_n": np.zeros((I, K), order="F"),
        "bcp_var_b": np.zeros((I, J), order="F"), "bcp_var_t": np.zeros((I, J), order="F"),
        "ucell_moexcell": moex_u, "ucell_cell_type": np.asfortranarray(ct_u),
        "vcell_moexcell": moex_v, "vcell_cell_type": np.asfortranarray(ct_v),
        "wcell_moexcell": moex_w, "wcell_cell_type": np.asfortranarray(ct_w),
        "tvar_u": tu, "tvar_v": tv, "tvar_w": tw, "tvar_p": tp,
        # not read by the hot path; kept for the pressure-force loss of the
        # gradient harness (Solver.f90:684-706 uses the solid normal)
        "pcell_nz": F(nz), "pcell_phi": F(phi), "pcell_wllh": F(wllh),
    }
    # Velocity BCs: no-slip walls (Dirichlet 0); an open (Dirichlet-p) face
    # gets Neumann velocity, like the dam-break driver's top
    # (Test/Dambreak/Dambreak.f90:86-89).
    vflag = tuple(1 if f == 0 else 0 for f in bcp_flag)
    return Workload(name=name, imax=I, jmax=J, kmax=K, dt=dt, rho_l=rho_l, rho_g=rho_g,
                    arrays=arrays, bcp_flag=tuple(bcp_flag),
                    bcu_flag=vflag, bcv_flag=vflag, bcw_flag=vflag,
                    bcu_const=(0.0,) * 6, bcv_const=(0.0,) * 6, bcw_const=(0.0,) * 6,
                    bcp_const=(0.0,) * 6, ext_cell=ext_cell,
                    meta={"seed": seed, "solid": solid, "liquid": liquid[0]})


def _surface(z0, amp, kx, ky=None, kind="sinsin"):
    two_pi = 2.0 * math.pi
    if kind == "sinsin":
        h = lambda x, y: z0 + amp * np.sin(two_pi * x) * np.sin(two_pi * y)
        hx = lambda x, y: amp * two_pi * np.cos(two_pi * x) * np.sin(two_pi * y)
        hy = lambda x, y: amp * two_pi * np.sin(two_pi * x) * np.cos(two_pi * y)
    else:  # cosx wave of wavelength kx
        w = two_pi / kx
        h = lambda x, y: z0 + amp * np.cos(w * x) + 0.0 * y
        hx = lambda x, y: -amp * w * np.sin(w * x) + 0.0 * y
        hy = lambda x, y: 0.0 * x + 0.0 * y
    return ("surface", h, hx, hy)


# Named workloads -------------------------------------------------------------

SPHERE_C1 = ("sphere", 0.5, 0.5, 0.3, 0.15)


def pressure_force_weights(w) -> np.ndarray:
    """Weights g of the vertical pressure force on the solid: the sum over
    cut cells of p * (-nz) * WlLh (the Clpz1 sum of PrintDragLiftCoef,
    Solver.f90:684-706); interior (I,J,K) array."""
    a = w.arrays
    g = -a["pcell_nz"] * a["pcell_wllh"]
    return np.asfortranarray(np.where(a["cell_type"] == 1, g, 0.0))


def config(name: str, n: Optional[int] = None, seed: int = DEFAULT_SEED, **kw) -> Workload:
    """Named synthetic configurations.

    * ``c0``: 64^3 two-phase, no solid, interface z=0.5+0.02 sin2πx sin2πy,
      ρ=1000/1.2, all-Neumann pressure (singular, mean pinned).
    * ``c1``: 128^3, c0 plus a cut-cell sphere r=0.15 at (0.5,0.5,0.3).
    * ``c2``: 256^3, the c1 sphere in a water column with a gas bubble
      r=0.1 at (0.5,0.5,0.65), ρ_l/ρ_g = 1000.
    * ``c3``: c1 geometry at 128^3 (gradient harness).
    * ``c4``: 512x256x256 wave tank on [0,4]x[0,1]x[0,1], z stretched about
      z=0.5 with ratio 1.02, vertical cylinder r=0.1 at (2,0.5), free surface
      z=0.5+0.03 cos(2πx/0.8), ρ_l/ρ_g = 833, Dirichlet-p top (open).

    ``n`` overrides the cell count of the (cubic) configs for small test cases.
    """
    surf0 = _surface(0.5, 0.02, None)
    if name == "c0":
        n = n or 64
        return build_workload("c0", n, n, n, liquid=surf0, rho_l=1000.0, rho_g=1.2, seed=seed, **kw)
    if name in ("c1", "c3"):
        n = n or 128
        return build_workload(name, n, n, n, solid=SPHERE_C1, liquid=surf0, rho_l=1000.0, rho_g=1.2,
                              seed=seed, **kw)
    if name == "c2":
        n = n or 256
        return build_workload("c2", n, n, n, solid=SPHERE_C1, liquid=("bubble", 0.5, 0.5, 0.65, 0.1),
                              rho_l=1000.0, rho_g=1.0, seed=seed, **kw)
    if name == "c4":
        if n is None:
            I, J, K = 512, 256, 256
        else:
            I, J, K = 2 * n, n, n
        return build_workload("c4", I, J, K, extent=((0.0, 4.0), (0.0, 1.0), (0.0, 1.0)), zstretch=1.02,
                              solid=("zcylinder", 2.0, 0.5, 0.1), liquid=_surface(0.5, 0.03, 0.8, kind="cosx"),
                              rho_l=833.0, rho_g=1.0, bcp_flag=(1, 1, 1, 1, 1, 0), seed=seed, **kw)
    raise KeyError(name)
