"""The oracle of the CLSVOF module (oracle/clsvof.c): ComputeUVWLiquidField,
Interface_Reconstruct, the directional sweeps, Redistance_Levelset,
BoundaryConditionLvsVof and Clsvof_Scheme, against closed forms, an
independent vectorised Volume_Fraction_Calc, the reference's index shift of
the velocity cells' direction averages, exact translation of a plane,
conservation along each swept line and in a shear, and independent
restatements of the redistancing (as a gather) and of the boundary planes,
matched bit for bit.  CPU only (no GPU counterpart yet)."""
import math

import numpy as np
import pytest

from simcoflow3d_gb300 import workloads as W
from oracle import oracle as O


def test_volume_fraction_calc_matches_vectorised():
    """The C restatement and the numpy one (simcoflow3d_gb300/workloads.py)
    agree to rounding: the numpy one multiplies fc by (dx*dy*dz) where the
    reference multiplies (fc*dx)*dy*dz."""
    rng = np.random.default_rng(3)
    n = 4000
    dx, dy, dz = (rng.uniform(0.2, 2.0, n) for _ in range(3))
    nv = rng.normal(size=(3, n))
    nv /= np.linalg.norm(nv, axis=0)
    sm = np.abs(nv[0]) * dx + np.abs(nv[1]) * dy + np.abs(nv[2]) * dz
    s = rng.uniform(-0.1, 1.1, n) * sm
    ref = W.volume_fraction_calc(dx, dy, dz, nv[0], nv[1], nv[2], s)
    got = np.array([O.volume_fraction_calc(*(float(a[q]) for a in (dx, dy, dz, nv[0], nv[1], nv[2], s)))
                    for q in range(n)])
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-15)


def test_volume_fraction_closed_forms():
    # a plane normal to x at distance s from the corner cuts s*dy*dz off
    assert O.volume_fraction_calc(2.0, 3.0, 5.0, 1.0, 0.0, 0.0, 0.5) == pytest.approx(0.5 * 3.0 * 5.0, rel=1e-15)
    # fully on one side
    assert O.volume_fraction_calc(1.0, 1.0, 1.0, 0.0, 0.0, 1.0, -0.2) == 0.0
    assert O.volume_fraction_calc(1.0, 2.0, 3.0, 0.0, 0.0, 1.0, 3.5) == 6.0
    # the diagonal plane through the box centre halves the cube
    n = 1.0 / np.sqrt(3.0)
    assert O.volume_fraction_calc(1.0, 1.0, 1.0, n, n, n, 1.5 * n) == pytest.approx(0.5, rel=1e-12)


def _fields(I, J, K, zc, seed=1):
    """P cells of a uniform unit box with a horizontal interface at z = zc
    (liquid below): phiL = z - zc, normal +z, vofL the exact fractions."""
    h = (1.0 / I, 1.0 / J, 1.0 / K)
    shp_i, shp_g = (I, J, K), (I + 2, J + 2, K + 2)
    pgrid = tuple(np.full(shp_i, hq, order="F") for hq in h)
    zcent = (np.arange(K + 2) - 0.5) * h[2]
    phil = np.asfortranarray(np.broadcast_to(zcent - zc, shp_g).copy())
    vofl = np.asfortranarray(np.clip((zc - (zcent - 0.5 * h[2])) / h[2], 0.0, 1.0) * np.ones(shp_g))
    pcell = {"phil": phil, "nxl": np.zeros(shp_g, order="F"), "nyl": np.zeros(shp_g, order="F"),
             "nzl": np.ones(shp_g, order="F"), "vofl": vofl}
    rng = np.random.default_rng(seed)
    vgrids = [pgrid, pgrid, pgrid]
    vcells = [{k: np.asfortranarray(rng.normal(size=shp_g)) for k in ("phil", "nxl", "nyl", "nzl")}
              for _ in range(3)]
    for c in vcells:
        c["vofl"] = np.asfortranarray(rng.uniform(0.0, 1.0, size=shp_g))
        c["vof"] = np.ones(shp_g, order="F")
    return pgrid, pcell, vgrids, vcells


def test_u_cells_see_a_horizontal_interface_like_the_p_cells():
    """A horizontal interface: each U cell spans the right half of P cell i
    and the left half of P cell i+1 at the same height, so its liquid
    fraction is the P cells' (and the last plane copies PCell's)."""
    I, J, K = 6, 5, 8
    pgrid, pcell, vgrids, vcells = _fields(I, J, K, zc=0.43)
    O.uvw_liquid_field(pgrid, pcell, vgrids, vcells)
    u = vcells[0]["vofl"][1:-1, 1:-1, 1:-1]
    p = pcell["vofl"][1:-1, 1:-1, 1:-1]
    np.testing.assert_allclose(u, p, rtol=0, atol=1e-14)


def test_direction_averages_land_one_cell_lower():
    """DirectionAverageArray writes through a dummy numbered from 1 into
    arrays allocated from 0: the average of P cells (i, i+1) is stored at
    U cell (i-1, j-1, k-1), the last written plane repeats the one before,
    and the rest keeps the caller's values."""
    I, J, K = 5, 4, 6
    pgrid, pcell, vgrids, vcells = _fields(I, J, K, zc=0.5)
    rng = np.random.default_rng(9)
    pcell["phil"] = np.asfortranarray(rng.normal(size=pcell["phil"].shape))
    before = vcells[0]["phil"].copy(order="F")
    O.uvw_liquid_field(pgrid, pcell, vgrids, vcells)
    out = vcells[0]["phil"]
    ph = pcell["phil"]
    for i in range(1, I):
        for j in range(1, J + 1):
            for k in range(1, K + 1):
                want = 0.5 * ph[i, j, k] + (1.0 - 0.5) * ph[i + 1, j, k]
                assert out[i - 1, j - 1, k - 1] == want
    assert np.array_equal(out[I - 1, 0:J, 0:K], out[I - 2, 0:J, 0:K])
    # the planes never written: i = I, I+1, and j, k = J, K and beyond
    assert np.array_equal(out[I:, :, :], before[I:, :, :])
    assert np.array_equal(out[:, J:, :], before[:, J:, :])


def _conv(dx, dy, dz, nx, ny, nz, phi):
    return phi + 0.5 * (abs(nx) * dx + abs(ny) * dy + abs(nz) * dz)


@pytest.mark.parametrize("fam", [1, 2])
def test_v_and_w_cells_follow_the_reference_lines(fam):
    """The V and W loops as the reference writes them, cell by cell: the V
    cells' left half takes the whole dy and phiL itself, their right half
    phiL(i,j,k) with the (i,j+1,k) normal and a plus sign; the W cells'
    right half shifts by +dz/2 (Clsvof.f90:225-291)."""
    I, J, K = 4, 5, 6
    pgrid, pcell, vgrids, vcells = _fields(I, J, K, zc=0.37)
    rng = np.random.default_rng(17)
    nv = rng.normal(size=(3,) + pcell["phil"].shape)
    nv /= np.linalg.norm(nv, axis=0)
    for q, key in enumerate(("nxl", "nyl", "nzl")):
        pcell[key] = np.asfortranarray(nv[q])
    O.uvw_liquid_field(pgrid, pcell, vgrids, vcells)
    ph, nx, ny, nz = pcell["phil"], pcell["nxl"], pcell["nyl"], pcell["nzl"]
    dx, dy, dz = (g[0, 0, 0] for g in pgrid)
    vf = O.volume_fraction_calc
    got = vcells[fam]["vofl"]
    for (i, j, k) in [(1, 1, 1), (2, 3, 4), (4, 4, 5), (3, 2, 2)]:
        n0 = (nx[i, j, k], ny[i, j, k], nz[i, j, k])
        if fam == 1:
            if j > J - 1:
                continue
            n1 = (nx[i, j + 1, k], ny[i, j + 1, k], nz[i, j + 1, k])
            dc = dy / 2.0
            left = dx * dc * dz - vf(dx, dc, dz, *n0, _conv(dx, dy, dz, *n0, ph[i, j, k]))
            phn = ph[i, j, k] + dc * ny[i, j + 1, k]
            right = dx * dc * dz - vf(dx, dc, dz, *n1, _conv(dx, dc, dz, *n1, phn))
        else:
            if k > K - 1:
                continue
            n1 = (nx[i, j, k + 1], ny[i, j, k + 1], nz[i, j, k + 1])
            dc = dz / 2.0
            phn = ph[i, j, k] + dc * nz[i, j, k]
            left = dx * dy * dc - vf(dx, dy, dc, *n0, _conv(dx, dy, dc, *n0, phn))
            phn = ph[i, j, k + 1] + dc * nz[i, j, k + 1]
            right = dx * dy * dc - vf(dx, dy, dc, *n1, _conv(dx, dy, dc, *n1, phn))
        want = (left + right) / dx / dy / dz
        assert got[i, j, k] == want, (fam, i, j, k)


def test_find_distance_inverts_volume_fraction():
    """Find_Distance (with its cube root and Newton steps) returns the
    corner distance at which Volume_Fraction_Calc gives back the fraction."""
    rng = np.random.default_rng(5)
    worst = 0.0
    for _ in range(3000):
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        d = rng.uniform(0.5, 2.0, 3)
        f = rng.uniform(0.001, 0.999)
        s = O.find_distance(*d, *n, f)
        worst = max(worst, abs(O.volume_fraction_calc(*d, *n, s) / np.prod(d) - f))
    assert worst < 1e-10


def test_interface_reconstruct_recovers_a_plane():
    """A planar liquid surface: every interface cell gets the plane's unit
    normal (phi is linear, so every difference Normal_Vector_Irre may pick
    is exact to rounding) and a distance whose cut volume is its liquid
    fraction; the other cells get zeros."""
    I = J = K = 10
    h = 1.0 / I
    c = (np.arange(I) + 0.5) * h
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    centres = tuple(np.asfortranarray(a) for a in (X, Y, Z))
    spacings = tuple(np.full((I, J, K), h, order="F") for _ in range(3))
    n = np.array([0.3, -0.5, 0.81])
    n /= np.linalg.norm(n)
    cg = (np.arange(I + 2) - 0.5) * h
    Xg, Yg, Zg = np.meshgrid(cg, cg, cg, indexing="ij")
    phi = np.asfortranarray(n[0] * (Xg - 0.52) + n[1] * (Yg - 0.47) + n[2] * (Zg - 0.55))
    # liquid (phi < 0) fraction of each cell, from the corner distance
    s = phi + 0.5 * h * np.abs(n).sum()
    vfl = np.asfortranarray(1.0 - W.volume_fraction_calc(h, h, h, n[0], n[1], n[2], s) / h ** 3)
    nx, ny, nz, dis = O.interface_reconstruct(centres, spacings, vfl, phi)
    part = (vfl > 1e-14) & (vfl < 1.0 - 1e-14)
    inner = np.zeros_like(part)
    inner[1:-1, 1:-1, 1:-1] = part[1:-1, 1:-1, 1:-1]
    assert inner.sum() > 50
    for q, a in enumerate((nx, ny, nz)):
        np.testing.assert_allclose(a[inner], n[q], atol=1e-12)
    for (i, j, k) in np.argwhere(inner)[:40]:
        got = O.volume_fraction_calc(h, h, h, nx[i, j, k], ny[i, j, k], nz[i, j, k], dis[i, j, k]) / h ** 3
        assert abs(got - vfl[i, j, k]) < 1e-10
    far = np.zeros_like(part)
    far[1:-1, 1:-1, 1:-1] = (vfl[1:-1, 1:-1, 1:-1] == 0.0) & (np.abs(phi[1:-1, 1:-1, 1:-1]) > 3 * h)
    assert (nx[far] == 0).all() and (dis[far] == 0).all()


# ---- the directional sweeps (X_Sweep / Y_Sweep / Z_Sweep) ----------------

_SHAPE = (12, 9, 10)


def _plane_case(axis, n, x0, shape=_SHAPE):
    """Cells of the unit box (spacing 1/I, 1/J, 1/K) cut by the plane
    n.(x - x0 e_axis) = 0, liquid on the phi < 0 side: centres, spacings,
    the ghosted phi and the exact liquid fractions."""
    I, J, K = shape
    h = np.array([1.0 / I, 1.0 / J, 1.0 / K])
    n = np.asarray(n, float) / np.linalg.norm(n)
    cs = [(np.arange(m) + 0.5) * hq for m, hq in zip(shape, h)]
    cg = [(np.arange(m + 2) - 0.5) * hq for m, hq in zip(shape, h)]
    centres = tuple(np.asfortranarray(a) for a in np.meshgrid(*cs, indexing="ij"))
    spacings = tuple(np.full(shape, hq, order="F") for hq in h)
    Xg = np.meshgrid(*cg, indexing="ij")
    off = np.zeros(3)
    off[axis] = x0

    def phi_at(shift):
        return np.asfortranarray(sum(n[q] * (Xg[q] - off[q] - (shift if q == axis else 0.0)) for q in range(3)))

    def fractions(phi):
        s = phi + 0.5 * (np.abs(n) * h).sum()
        return np.asfortranarray(1.0 - W.volume_fraction_calc(h[0], h[1], h[2], n[0], n[1], n[2], s) / h.prod())

    return centres, spacings, h, n, phi_at, fractions


def _wall(a, axis):
    """The ghost plane at the low wall of ``axis``, interior in the others."""
    idx = [slice(1, -1)] * 3
    idx[axis] = 0
    return np.asfortranarray(a[tuple(idx)])


@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("tilt", [False, True])
def test_sweep_translates_a_plane(axis, tilt):
    """A uniform velocity along the axis carries a plane exactly: the
    geometric fluxes cut the upstream cells by the reconstructed plane, so
    each new liquid fraction is the fraction of the plane moved by u dt;
    the level set, linear, drops by u dt times its slope in every cell when
    the wall value is the level set at the wall half a step upstream."""
    n = [0.0, 0.0, 0.0]
    n[axis] = 1.0
    if tilt:
        n[(axis + 1) % 3], n[(axis + 2) % 3] = 0.15, -0.1
    centres, spacings, h, nu, phi_at, fractions = _plane_case(axis, n, 0.57)
    u, dt = 0.7, 0.35 * h[axis] / 0.7
    phi = phi_at(0.0)
    vfl = fractions(phi)
    vel = np.full(phi.shape, u, order="F")
    bc_vel = _wall(vel, axis)
    wall_phi = _wall(phi, axis) + 0.5 * h[axis] * nu[axis]
    bc_lvs = np.asfortranarray(wall_phi - nu[axis] * u * dt / 2.0)
    temvf, temls, _ = O.clsvof_sweep(axis, centres, spacings, vfl, phi, vel, bc_vel, bc_lvs, dt)
    moved = phi_at(u * dt)
    inner = (slice(1, -1),) * 3
    part = (vfl[inner] > 0.0) & (vfl[inner] < 1.0)
    assert part.sum() > 20
    np.testing.assert_allclose(temvf[inner], fractions(moved)[inner], atol=1e-12)
    np.testing.assert_allclose(temls[inner], moved[inner], atol=1e-13)


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_sweep_conserves_liquid_along_each_line(axis):
    """Every interior face's VOF flux leaves one cell and enters the next,
    so along a line the liquid changes only by the two wall fluxes
    vfl(1) u(0) dt and vfl(n) u(n) dt, whatever the velocities (both signs
    here, so the east and the west cuts both run)."""
    centres, spacings, h, _, phi_at, fractions = _plane_case(axis, [0.45, -0.6, 0.66], 0.5)
    phi = phi_at(0.0)
    vfl = fractions(phi)
    rng = np.random.default_rng(5 + axis)
    vel = np.asfortranarray(rng.uniform(-1.0, 1.0, phi.shape))
    dt = 0.4 * h.min()
    wall = np.zeros(_wall(vel, axis).shape, order="F")
    temvf, _, _ = O.clsvof_sweep(axis, centres, spacings, vfl, phi, vel, wall, wall, dt)
    inner = (slice(1, -1),) * 3
    gained = np.moveaxis((temvf - vfl)[inner], axis, 0).sum(axis=0) * h[axis]
    vm = np.moveaxis(vel, axis, 0)
    fm = np.moveaxis(vfl, axis, 0)
    # the other two axes keep their interior order after moveaxis
    lo = fm[1, 1:-1, 1:-1] * vm[0, 1:-1, 1:-1] * dt
    hi = fm[-2, 1:-1, 1:-1] * vm[-2, 1:-1, 1:-1] * dt
    np.testing.assert_allclose(gained, lo - hi, atol=1e-14)
    assert ((vfl[inner] > 0) & (vfl[inner] < 1)).sum() > 20


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_sweep_backward_level_set_keeps_the_reference_faces(axis):
    """u < 0 on a level set of unit slope along the axis: the faces between
    cells 2..n take the upwind value exactly, the first face takes the
    reference's x / y / z forms (x divides by 2 and multiplies by dx(2), y
    is the exact upwind value, z adds the correction), and the last face
    extrapolates from the face below, which leaves cell n as it was when
    its spacings are all equal (x, y) and scales by dy for z."""
    n = [0.0, 0.0, 0.0]
    n[axis] = 1.0
    centres, spacings, h, _, phi_at, fractions = _plane_case(axis, n, 0.57)
    u = -0.8
    dt = 0.3 * h.min() / 0.8
    phi = phi_at(0.0)
    vfl = fractions(phi)
    vel = np.full(phi.shape, u, order="F")
    bc_lvs = np.asfortranarray(_wall(phi, axis) * 0.0 + 0.25)
    _, temls, _ = O.clsvof_sweep(axis, centres, spacings, vfl, phi, vel, _wall(vel, axis), bc_lvs, dt)
    hd = h[axis]
    p = np.moveaxis(phi, axis, 0)[1:-1, 1:-1, 1:-1]
    t = np.moveaxis(temls, axis, 0)[1:-1, 1:-1, 1:-1]
    m = p.shape[0]
    a = hd / 2.0 * (1.0 + u * dt / hd)
    face = {q: p[q + 1] - a for q in range(1, m - 1)}   # 0-based: the face between cells q and q+1
    first = {0: p[1] - a * hd * hd, 1: p[1] - a, 2: p[1] + a}[axis]
    scale = h[1] if axis == 2 else hd
    last = p[m - 1] - hd / 2.0 * (1.0 + u * dt / scale)
    f = lambda ls: u * ls * dt / hd
    np.testing.assert_allclose(t[0], p[0] - f(first) + u * 0.25 * dt / hd, atol=1e-13)
    np.testing.assert_allclose(t[1], p[1] + f(first) - f(face[1]), atol=1e-13)
    for q in range(2, m - 1):
        np.testing.assert_allclose(t[q], p[q] - u * dt, atol=1e-13)
    np.testing.assert_allclose(t[m - 1], p[m - 1] + f(face[m - 2]) - f(last), atol=1e-13)
    if axis != 2:
        np.testing.assert_allclose(t[m - 1], p[m - 1], atol=1e-13)


# ---- redistancing (Redistance_Levelset) -----------------------------------

def _sg(a):
    return math.copysign(1.0, a)


def _shortest_point_2d(n, d1, off, cas, h, s):
    """Shortest_Point_2d (Clsvof.f90:1961-2060) on the face normal to axis
    ``cas`` (0, 1, 2): writes the two other coordinates of ``s``.  The y
    face solves for x by dividing by |nz| (the reference's)."""
    a, b = [q for q in range(3) if q != cas]
    t = math.sqrt(n[a] * n[a] + n[b] * n[b] + 1e-30 * 1e-30)
    na, nb, d = n[a] / t, n[b] / t, d1 / t
    dij = na * h[a] * off[a] + nb * h[b] * off[b] + d
    pa, pb = h[a] * off[a] - dij * na, h[b] * off[b] - dij * nb
    if -0.5 * h[a] <= pa <= 0.5 * h[a] and -0.5 * h[b] <= pb <= 0.5 * h[b]:
        s[a], s[b] = pa, pb
        return
    oa, ob = max(abs(pa) - 0.5 * h[a], 0.0), max(abs(pb) - 0.5 * h[b], 0.0)
    if oa * abs(na) > ob * abs(nb):
        s[a] = _sg(pa) * 0.5 * h[a]
        s[b] = (d + na * s[a]) / (_sg(-nb) * max(abs(nb), 1e-14))
    else:
        s[b] = _sg(pb) * 0.5 * h[b]
        div = abs(nb) if cas == 1 else abs(na)
        s[a] = (d + nb * s[b]) / (_sg(-na) * max(div, 1e-14))


def _band_distance(n, dc, off, h, side):
    """The distance Redistance_Levelset (Clsvof.f90:1740-1861) measures from
    the centre ``off`` cells away to an interface cell's plane n.x + dc = 0."""
    X = [h[q] * off[q] for q in range(3)]
    xv = [h[q] * max(-1, min(1, off[q])) / 2.0 for q in range(3)]
    dv = n[0] * xv[0] + n[1] * xv[1] + n[2] * xv[2] + dc
    dist = lambda p: math.sqrt((X[0] - p[0]) * (X[0] - p[0]) + (X[1] - p[1]) * (X[1] - p[1]) +
                               (X[2] - p[2]) * (X[2] - p[2]))
    if dv * _sg(side) <= 0.0:
        return dist(xv)
    dij = n[0] * h[0] * off[0] + n[1] * h[1] * off[1] + n[2] * h[2] * off[2] + dc
    p = [X[q] - dij * n[q] for q in range(3)]
    if all(-0.5 * h[q] <= p[q] <= 0.5 * h[q] for q in range(3)):
        return dist(p)
    w = [max(abs(p[q]) - 0.5 * h[q], 0.0) * abs(n[q]) for q in range(3)]
    fc = [_sg(p[q]) * 0.5 * h[q] for q in range(3)]
    s = [0.0, 0.0, 0.0]
    for c in range(3):
        o1, o2 = [q for q in range(3) if q != c]
        if not (w[c] >= w[o1] and w[c] >= w[o2]):
            continue
        corners = []      # Iscutface's point1..point4, around the face
        for sa, sb in ((-0.5, -0.5), (-0.5, 0.5), (0.5, 0.5), (0.5, -0.5)):
            v = [0.0, 0.0, 0.0]
            v[c], v[o1], v[o2] = fc[c], sa * h[o1], sb * h[o2]
            corners.append(n[0] * v[0] + n[1] * v[1] + n[2] * v[2] + dc)
        cut = not all(corners[q] * corners[(q + 1) % 4] >= 0.0 for q in range(4))
        if cut:
            cas = c
        else:
            cas = o1 if w[o1] > w[o2] else o2
        s[cas] = fc[cas]
        _shortest_point_2d(n, n[cas] * s[cas] + dc, off, cas, h, s)
    return dist(s)


def _redistance_gather(h, vfl, phi, nx, ny, nz, dis):
    """Redistance_Levelset restated as a gather: each full or empty cell
    takes the least band distance over the interface cells around it."""
    I, J, K = (m - 2 for m in vfl.shape)
    inner = (slice(1, -1),) * 3
    part = (vfl[inner] > 1e-15) & (vfl[inner] < 1.0 - 1e-15)
    iface = [tuple(int(v) + 1 for v in c) for c in np.argwhere(part)]
    out = np.array(phi, copy=True)

    def centre_distance(a, b, c):
        n = (nx[a, b, c], ny[a, b, c], nz[a, b, c])
        return n, (0.5 * h[0] * abs(n[0]) + 0.5 * h[1] * abs(n[1]) + 0.5 * h[2] * abs(n[2])) - dis[a, b, c]

    for i in range(1, I + 1):
        for j in range(1, J + 1):
            for k in range(1, K + 1):
                f = vfl[i, j, k]
                if part[i - 1, j - 1, k - 1]:
                    out[i, j, k] = _sg(0.5 - f) * abs(centre_distance(i, j, k)[1])
                    continue
                best = None
                if f < 1e-15 or f > 1.0 - 1e-15:
                    for (a, b, c) in iface:
                        off = (i - a, j - b, k - c)
                        if max(abs(q) for q in off) > 4:
                            continue
                        n, dc = centre_distance(a, b, c)
                        d = _band_distance(n, dc, off, h, phi[i, j, k])
                        best = d if best is None or d < best else best
                out[i, j, k] = _sg(0.5 - f) * (min(best, 1.0e4) if best is not None else 5 * h[0] * math.sqrt(3.0))
    return out


@pytest.mark.parametrize("n", [[1.0, 0.0, 0.0], [1.0, 0.15, 0.0], [1.0, 0.15, -0.1]])
def test_redistance_matches_a_gather_restatement(n):
    """The oracle's Redistance_Levelset (a scatter of running minima over
    the band of each interface cell, as the reference loops) equals, bit for
    bit, an independent gather over the interface cells around each cell.
    An axis-normal plane comes back as its exact signed distance; a tilted
    one is never under the true distance where the reference's y-face
    division by |nz| cannot act (nz = 0), and with nz != 0 that division
    puts some band cells well under it."""
    centres, spacings, h, nu, phi_at, fractions = _plane_case(0, n, 0.53, (12, 9, 10))
    phi = phi_at(0.0)
    vfl = fractions(phi)
    got, nl = O.clsvof_redistance(centres, spacings, vfl, 2.5 * phi)
    nx, ny, nz, dis = O.interface_reconstruct(centres, spacings, vfl, 2.5 * phi)
    ref = _redistance_gather(h, vfl, 2.5 * phi, nx, ny, nz, dis)
    np.testing.assert_array_equal(got, ref)
    for q, a in enumerate(nl):
        np.testing.assert_array_equal(a[1:-1, 1:-1, 1:-1], (nx, ny, nz)[q][1:-1, 1:-1, 1:-1])
    inner = (slice(1, -1),) * 3
    assert (np.sign(got[inner]) == np.where(vfl[inner] > 0.5, -1.0, 1.0)).all()
    far = np.abs(got[inner]) == 5 * h[0] * math.sqrt(3.0)
    under = np.abs(got[inner][~far]) - np.abs(phi[inner][~far])
    if n[1] == 0.0 and n[2] == 0.0:
        assert np.abs(under).max() < 1e-14
    elif n[2] == 0.0:
        assert under.min() > -1e-14 and (np.abs(under) < 1e-13).mean() > 0.6
    else:
        assert under.min() < -h[0]


# ---- one Clsvof_Scheme step ---------------------------------------------

def _clip(v):
    return np.where(v <= 1e-14, 0.0, np.where(v >= 1.0 - 1e-14, 1.0, v))


def _bc_lvs_vof(phi, vof, nxl, nf, h, lvs, vof_bc):
    """BoundaryConditionLvsVof restated on numpy planes: ``lvs`` and
    ``vof_bc`` are (flags, consts) pairs; fills the ghosts of phi and vof
    and returns the 12 wall planes W, E, S, N, B, T of each."""
    def typical(flag, cst, var, d):
        return np.full(var.shape, cst) if flag == 0 else var - cst * d / 2.0
    out = []
    for f, (flags, consts) in ((phi, lvs), (vof, vof_bc)):
        lvl = f is phi
        planes = []
        for ax in range(3):
            for hi in (False, True):
                q = 2 * ax + hi
                cell = [slice(1, -1)] * 3
                ghost = [slice(1, -1)] * 3
                cell[ax] = -2 if hi else 1
                ghost[ax] = -1 if hi else 0
                var = f[tuple(cell)].copy()
                d = -h[ax] if hi else h[ax]
                plane = typical(flags[q], consts[q], var, np.full(var.shape, d))
                if lvl and ax == 0:
                    plane = var - nxl[tuple(cell)] * d / 2.0
                planes.append(np.asfortranarray(plane))
                if lvl:
                    step = nf[ax][tuple(cell)] * h[ax]
                    f[tuple(ghost)] = var + step if hi and ax != 1 else var - step
                else:
                    f[tuple(ghost)] = var
        out.append(planes)
    return out


def _scheme_inputs(n, x0, shape=(12, 9, 10)):
    centres, spacings, h, nu, phi_at, fractions = _plane_case(0, n, x0, shape)
    g = (shape[0] + 2, shape[1] + 2, shape[2] + 2)
    state = {"phil": phi_at(0.0), "vofl": np.asfortranarray(_clip(fractions(phi_at(0.0))))}
    for key in ("nxl", "nyl", "nzl"):
        state[key] = np.zeros(g, order="F")
    nf = [np.full(g, nu[q], order="F") for q in range(3)]
    lvs_bc = [np.zeros(sh, order="F") for sh in [shape[1:]] * 2 + [(shape[0], shape[2])] * 2 + [shape[:2]] * 2]
    return centres, spacings, h, nu, phi_at, fractions, state, nf, lvs_bc


def test_scheme_at_rest_is_six_redistancings():
    """With no velocity the sweeps move nothing, so a step is six rounds of
    the boundary planes and ghosts (W/E planes from the liquid normals, the
    others TypicalBC; ghost level set from the fluid normals, the north one
    subtracting like the south) followed by the redistancing; the liquid
    fractions stay as they are, bit for bit."""
    centres, spacings, h, nu, phi_at, fractions, state, nf, lvs_bc = _scheme_inputs([1.0, 0.15, -0.1], 0.53)
    state["phil"] = np.asfortranarray(2.5 * state["phil"])
    lvs = ((1, 1, 0, 1, 1, 1), (0.0, 0.0, 0.7, 0.3, 0.0, 0.0))
    vofb = ((1, 1, 1, 1, 0, 1), (0.0, 0.0, 0.0, 0.0, 0.25, 0.1))
    vel = [np.zeros_like(state["phil"]) for _ in range(3)]
    bc_vel = [np.zeros(a.shape, order="F") for a in (lvs_bc[0], lvs_bc[2], lvs_bc[4])]
    phi = state["phil"].copy(order="F")
    vof = state["vofl"].copy(order="F")
    nxl = state["nxl"].copy(order="F")
    for _ in range(6):
        planes = _bc_lvs_vof(phi, vof, nxl, nf, h, lvs, vofb)
        phi, nl = O.clsvof_redistance(centres, spacings, vof, phi)
        nxl = nl[0]
    vof_bc = O.clsvof_scheme(centres, spacings, state, vel, nf, bc_vel, lvs_bc, 0.01, lvs_flag=lvs[0],
                             lvs_const=lvs[1], vof_flag=vofb[0], vof_const=vofb[1])
    np.testing.assert_array_equal(state["phil"], phi)
    np.testing.assert_array_equal(state["vofl"], vof)
    np.testing.assert_array_equal(state["nxl"][1:-1, 1:-1, 1:-1], nl[0][1:-1, 1:-1, 1:-1])
    np.testing.assert_array_equal(state["nyl"][1:-1, 1:-1, 1:-1], nl[1][1:-1, 1:-1, 1:-1])
    for q in range(6):
        np.testing.assert_array_equal(lvs_bc[q], planes[0][q])
        np.testing.assert_array_equal(vof_bc[q], planes[1][q])
    assert (lvs_bc[2] == 0.7).all() and (vof_bc[4] == 0.25).all()


def test_scheme_carries_a_plane_one_step():
    """A uniform velocity along x carries a tilted plane through the six
    sub-steps: the liquid fractions are those of the moved plane, and the
    interface cells' level set and normals are the moved plane's."""
    n = [1.0, 0.0, 0.15]
    centres, spacings, h, nu, phi_at, fractions, state, nf, lvs_bc = _scheme_inputs(n, 0.47)
    u, dt = 0.9, 0.45 * h[0] / 0.9
    g = state["phil"].shape
    vel = [np.full(g, u, order="F"), np.zeros(g, order="F"), np.zeros(g, order="F")]
    bc_vel = [np.full(lvs_bc[0].shape, u, order="F"), np.zeros(lvs_bc[2].shape, order="F"),
              np.zeros(lvs_bc[4].shape, order="F")]
    O.clsvof_scheme(centres, spacings, state, vel, nf, bc_vel, lvs_bc, dt)
    moved = phi_at(u * dt)
    inner = (slice(1, -1),) * 3
    want = _clip(fractions(moved))[inner]
    part = (want > 0) & (want < 1)
    assert part.sum() > 50
    np.testing.assert_allclose(state["vofl"][inner], want, atol=1e-12)
    np.testing.assert_allclose(state["phil"][inner][part], moved[inner][part], atol=1e-12)
    for q, key in enumerate(("nxl", "nyl", "nzl")):
        np.testing.assert_allclose(state[key][inner][part], nu[q], atol=1e-12)


def test_scheme_keeps_the_liquid_volume_in_a_shear():
    """u = u(y), v = w = 0 is divergence-free along every x line, so the
    first sweep's division and the later corrections are exact no-ops and a
    drop away from the walls keeps its liquid volume to rounding."""
    I = J = K = 14
    h = 1.0 / I
    c = (np.arange(I) + 0.5) * h
    cg = (np.arange(I + 2) - 0.5) * h
    centres = tuple(np.asfortranarray(a) for a in np.meshgrid(c, c, c, indexing="ij"))
    spacings = tuple(np.full((I, J, K), h, order="F") for _ in range(3))
    Xg, Yg, Zg = np.meshgrid(cg, cg, cg, indexing="ij")
    r = np.sqrt((Xg - 0.48) ** 2 + (Yg - 0.52) ** 2 + (Zg - 0.5) ** 2)
    phi = np.asfortranarray(r - 0.23)
    sub = (np.arange(6) + 0.5) / 6 - 0.5
    vof = np.zeros_like(phi)
    for a in sub:
        for b in sub:
            for d in sub:
                vof += (np.sqrt((Xg + a * h - 0.48) ** 2 + (Yg + b * h - 0.52) ** 2 + (Zg + d * h - 0.5) ** 2)
                        < 0.23)
    vof = np.asfortranarray(_clip(vof / 216.0))
    g = phi.shape
    state = {"phil": phi, "vofl": vof}
    for key in ("nxl", "nyl", "nzl"):
        state[key] = np.zeros(g, order="F")
    nf = [np.zeros(g, order="F") for _ in range(3)]
    vel = [np.asfortranarray(0.6 * np.sin(2 * np.pi * Yg) + np.zeros(g)), np.zeros(g, order="F"),
           np.zeros(g, order="F")]
    lvs_bc = [np.zeros(sh, order="F") for sh in [(J, K)] * 2 + [(I, K)] * 2 + [(I, J)] * 2]
    bc_vel = [np.asfortranarray(vel[0][0, 1:-1, 1:-1]), np.zeros((I, K), order="F"), np.zeros((I, J), order="F")]
    vof0 = vof[1:-1, 1:-1, 1:-1].copy()
    before = vof0.sum()
    O.clsvof_scheme(centres, spacings, state, vel, nf, bc_vel, lvs_bc, 0.4 * h / 0.6)
    after = state["vofl"][1:-1, 1:-1, 1:-1]
    assert ((after > 0) & (after < 1)).sum() > 100
    assert abs(after.sum() - before) < 1e-11 * before
    assert np.abs(after - vof0).max() > 0.05


def test_powers_are_correctly_rounded():
    """x**3.d0 and x**(1.d0/3.d0) in the oracle are the exact powers rounded
    once to nearest, against 300-bit arithmetic, on random arguments and on
    arguments where the C library's pow lands on the wrong side of a
    near-tie (0.501 against 0.499 ulp)."""
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 300
    L = O.lib()
    third = mp.mpf(1.0 / 3.0)   # fl(1/3), the exponent Fortran's 1.d0/3.d0 holds
    rng = np.random.default_rng(11)
    xs = list(np.exp(rng.uniform(np.log(1e-30), np.log(1e3), 3000)))
    ties_cube = ["0x1.29b7c7f567ad7p-4", "0x1.1ea6bb697d9dap-29", "0x1.ccf39d3c80638p-2"]
    ties_third = ["0x1.e9f8dceb7595ep-8", "0x1.4406cfa26b09p-3", "0x1.f0dc3db8102p-15", "0x1.326eef373a70ap-7"]
    for x in xs + [float.fromhex(h) for h in ties_cube]:
        assert L.oracle_cube_rn(x) == float(mp.mpf(x) ** 3), x.hex()
    for x in xs + [float.fromhex(h) for h in ties_third]:
        assert L.oracle_pow_third(x) == float(mp.mpf(x) ** third), x.hex()
    assert L.oracle_pow_third(0.0) == 0.0
