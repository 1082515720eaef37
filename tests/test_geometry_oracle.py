"""The geometry oracle (oracle/geometry.c: GridPreprocess, DefineCell,
CellGeoCal, FaceGeoCal, DefineMomentumExchangeCell, NumberExternalCell of
src/CutCell.f90) against known answers: exact apertures of planar cuts,
an independent vectorised restatement of the aperture, numbering and
exchange-cell invariants, the wetted area of a sphere, and idempotence of
the whole sequence.  CPU only."""
import math

import numpy as np
import pytest

from simcoflow3d_gb300 import geometry as GM, workloads as W
from oracle import oracle as O


@pytest.mark.parametrize("phi,area,c2", [(0.25, 0.75, 0.125), (-0.25, 0.25, 0.375), (0.75, 1.0, 0.0),
                                         (-0.5, 0.0, 0.0), (0.0, 0.5, 0.25), (0.5, 0.0, 0.0)])
def test_face_planar_cut(phi, area, c2):
    """Unit face, plane normal along the face's second axis: open where
    s2 > -phi, so the open fraction is 0.5 + phi and the centroid is the
    middle of [-phi, 0.5].  A plane through two corners (phi = 0.5) gives the
    reference's degenerate result 0: corner values of exactly 0 count as
    neither open nor as a sign change, leaving a two-vertex polygon."""
    a, c = O.face_geo_cal(1.0, 1.0, 0.0, 1.0, 0.0, 0.3, phi)
    assert a == area
    if area > 0:
        assert abs(c[1] - c2) <= 1e-15
        assert c[0] == 0.0
    assert c[2] == 0.3


def test_face_open_depends_on_edges_only():
    """An open face: area exactly 1 and the same centroid whatever the
    normal, offset or level set (the kernels memoise it on d1, d2)."""
    rng = np.random.default_rng(1)
    ref = O.face_geo_cal(0.3, 0.7, 0.0, 0.0, 0.0, 0.0, 1.0)
    assert ref[0] == 1.0
    for _ in range(50):
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        a, c = O.face_geo_cal(0.3, 0.7, *n, 0.1, 10.0 + rng.uniform())
        assert a == ref[0] and c[0] == ref[1][0] and c[1] == ref[1][1]


def test_face_matches_vectorised_restatement():
    """workloads.face_geo_area restates the aperture independently (numpy,
    vectorised); the two agree bit for bit on random faces."""
    rng = np.random.default_rng(3)
    m = 4000
    d1, d2 = rng.uniform(0.5, 2, m), rng.uniform(0.5, 2, m)
    n = rng.normal(size=(m, 3))
    n /= np.linalg.norm(n, axis=1)[:, None]
    d3, phi = rng.uniform(-1, 1, m), rng.uniform(-1.5, 1.5, m)
    ref = W.face_geo_area(d1, d2, n[:, 0], n[:, 1], n[:, 2], d3, phi)
    got = np.array([O.face_geo_cal(d1[q], d2[q], *n[q], d3[q], phi[q])[0] for q in range(m)])
    assert np.array_equal(ref, got)


def test_diagonal_cut():
    """Unit face, normal (1,1)/sqrt2, phi = 0.1: the closed part is the
    corner triangle s1 + s2 < -0.1 sqrt2 with legs 1 - 0.1 sqrt2; the open
    part's centroid lies on the diagonal."""
    r = 1 / math.sqrt(2)
    a, c = O.face_geo_cal(1.0, 1.0, r, r, 0.0, 0.0, 0.1)
    leg = 1.0 - 0.1 * math.sqrt(2)
    assert abs(a - (1.0 - leg * leg / 2)) <= 1e-14
    # centroid: open square minus the triangle (centroid at -0.5 + leg/3 per axis)
    ct = -0.5 + leg / 3
    want = (0.0 - (leg * leg / 2) * ct) / a
    assert abs(c[0] - want) <= 1e-14 and abs(c[1] - want) <= 1e-14


@pytest.fixture(scope="module")
def sphere():
    g = GM.geometry_inputs("c1", n=48)
    return g, O.grid_preprocess(g)


def test_numbering_and_types(sphere):
    g, r = sphere
    I, J, K = g.imax, g.jmax, g.kmax
    for f in GM.FAMILIES:
        F = r.fams[f].arrays
        ct = F["cell_type"]
        assert set(np.unique(ct)) <= {0, 1, 2}
        iu, iv, iw = GM.POSNU_CUT[f]
        pos = F["posnu"]
        sub = ct[:I - iu, :J - iv, :K - iw]
        assert np.array_equal(pos < 0, sub == 2)
        # numbered 0..ext in loop order (i outer, k fastest)
        order = np.transpose(pos, (0, 1, 2)).ravel(order="C")
        act = order[order >= 0]
        assert np.array_equal(act, np.arange(act.size))
        assert r.fams[f].ext_cell == act.size - 1
        # DefineCell: full cells have vof = 1, empty cells vof = vofL = 0
        vof = F["vof"][1:-1, 1:-1, 1:-1]
        assert (vof[ct == 0] == 1.0).all()
        # CellGeoCal closes every face of a solid cell; GridPreprocess then
        # rewrites PCell's E/N/T apertures and UCell's E, VCell's N, WCell's T
        # from the other families, so check the apertures it keeps
        keep = {"p": (), "u": ("nearea", "tearea"), "v": ("eearea", "tearea"), "w": ("eearea", "nearea")}[f]
        s = np.argwhere(ct == 2)
        for key in keep:
            ax = {"eearea": 0, "nearea": 1, "tearea": 2}[key]
            a = F[key]
            for i, j, k in s[:300]:
                lo = [i + 1, j + 1, k + 1]
                lo[ax] -= 1
                assert a[i + 1, j + 1, k + 1] == 0.0 and a[tuple(lo)] == 0.0


def test_momentum_exchange_cells(sphere):
    g, r = sphere
    P = r.fams["p"].arrays["cell_type"]
    for f, ax in (("u", 0), ("v", 1), ("w", 2)):
        a0 = g.fams[f].arrays["moexcell"]
        a = r.fams[f].arrays["moexcell"]
        ct = r.fams[f].arrays["cell_type"]
        nb = np.roll(P, -1, axis=ax) == 2
        sl = [slice(None)] * 3
        sl[ax] = -1
        nb[tuple(sl)] = False
        want = (ct == 1) & ((P == 2) | nb)
        assert np.array_equal(a, np.where(want, 1, a0))


def test_wetted_area_of_the_sphere(sphere):
    """Sum of WlLh over the pressure cells approximates 4 pi r^2."""
    g, r = sphere
    wl = r.fams["p"].arrays["wllh"]
    ct = r.fams["p"].arrays["cell_type"]
    est = wl[ct == 1].sum()
    assert abs(est / (4 * math.pi * 0.15 ** 2) - 1) < 0.05


def test_sequence_is_idempotent(sphere):
    """Running the sequence again on its own results changes nothing (the
    device path reruns in place on that basis)."""
    _, r = sphere
    r2 = O.grid_preprocess(r)
    for f in GM.FAMILIES:
        for k in GM.OUTPUTS:
            a, b = r.fams[f].arrays.get(k), r2.fams[f].arrays.get(k)
            if a is None:
                continue
            assert a.tobytes(order="F") == b.tobytes(order="F"), (f, k)


def test_untouched_entries_keep_their_values(sphere):
    """Face centres on the i = I+1 ghost plane are written only by the
    boundary-plane copies along j and k; elsewhere on it they keep the
    caller's values."""
    g, r = sphere
    for f in GM.FAMILIES:
        for key in ("fce", "fcn", "fct"):
            a0, a = g.fams[f].arrays[key], r.fams[f].arrays[key]
            assert np.array_equal(a0[-1, 1:-2, 1:-2], a[-1, 1:-2, 1:-2])
            assert not np.array_equal(a0[-1, 0], a[-1, 0])
