"""The oracle of ComputeUVWLiquidField (oracle/clsvof.c), the first piece of
the CLSVOF module, against closed forms, an independent vectorised
Volume_Fraction_Calc, and the reference's index shift of the velocity cells'
direction averages.  CPU only (no GPU counterpart yet)."""
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
