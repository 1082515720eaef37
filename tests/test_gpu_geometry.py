"""GPU parity of the cut-cell geometry preprocessing (include/scf_geometry.h)
against the oracle (oracle/geometry.c): every array the sequence writes,
and the ExtCell counts, are bit-identical, on a sphere, a z-stretched box
with a cylinder (the stretched-grid face-centre branch), a solid slab on an
odd-sized box, and grids whose k extent spans several thread segments.
Also: the split stage/run/fetch API, reruns in place, and error paths."""
import ctypes as C

import numpy as np
import pytest

from simcoflow3d_gb300 import capi, geometry as GM
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = [
    ("sphere", lambda: GM.geometry_inputs("c1", n=32)),
    ("sphere40", lambda: GM.geometry_inputs("c1", n=40, solid=("sphere", 0.43, 0.55, 0.51, 0.23))),
    ("cylinder_stretched", lambda: GM.geometry_inputs("c4", n=16)),
    ("slab_odd", lambda: GM.geometry_inputs("box", shape=(19, 13, 37), solid=("xslab", 0.23))),
    ("no_solid", lambda: GM.geometry_inputs("box", shape=(8, 9, 10), solid=None)),
]


def _same(a, b):
    return a.tobytes(order="F") == b.tobytes(order="F")


def _compare(got, ref):
    for f in GM.FAMILIES:
        assert got.fams[f].ext_cell == ref.fams[f].ext_cell, f
        for k in GM.OUTPUTS:
            a, b = got.fams[f].arrays.get(k), ref.fams[f].arrays.get(k)
            if a is None:
                assert b is None
                continue
            if not _same(a, b):
                bad = np.argwhere(a.view(np.int64 if a.dtype == np.float64 else np.int32) !=
                                  b.view(np.int64 if b.dtype == np.float64 else np.int32))
                raise AssertionError("%s.%s differs at %d entries, first %s: %r vs %r" % (
                    f, k, len(bad), bad[0], a[tuple(bad[0])], b[tuple(bad[0])]))


@pytest.fixture(scope="module")
def lib(gpu_lib):
    return gpu_lib


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_grid_preprocess_bit_exact(lib, name, make):
    g = make()
    ref = O.grid_preprocess(g)
    got = g.copy()
    gp = GM.GridPreprocess(g.imax, g.jmax, g.kmax)
    st = gp(got)
    _compare(got, ref)
    assert st["gpu_launches"] > 0
    if name != "no_solid":
        assert 0 < st["exact_faces"] < 9 * g.imax * g.jmax * g.kmax


def test_split_api_and_rerun_in_place(lib):
    """stage, run twice (the sequence is idempotent), fetch: the same arrays
    as the one-shot call and the oracle."""
    g = GM.geometry_inputs("c1", n=24)
    ref = O.grid_preprocess(g)
    gp = GM.GridPreprocess(g.imax, g.jmax, g.kmax)
    gp.stage(g)
    gp.run()
    gp.run()
    got = g.copy()
    gp.fetch(got)
    _compare(got, ref)


def test_pressure_cells_feed_the_projection(lib):
    """The sequence's PCell outputs are what the projection reads: PosNu is
    -1 exactly on Cell_Type 2 and ExtCell counts the rest."""
    g = GM.geometry_inputs("c1", n=32)
    got = g.copy()
    GM.GridPreprocess(g.imax, g.jmax, g.kmax)(got)
    P = got.fams["p"]
    ct, pos = P.arrays["cell_type"], P.arrays["posnu"]
    assert np.array_equal(pos == -1, ct == 2)
    assert P.ext_cell == int((ct != 2).sum()) - 1


def test_error_paths(lib):
    from simcoflow3d_gb300.projection import ScfError
    g = GM.geometry_inputs("c1", n=8)
    gp = GM.GridPreprocess(g.imax, g.jmax, g.kmax)
    with pytest.raises(ScfError) as e:
        gp.run()
    assert e.value.status == capi.SCF_ERR_NO_SOLVE
    bad = g.copy()
    bad.fams["u"].arrays["moexcell"] = None
    with pytest.raises(ScfError) as e:
        gp(bad)
    assert e.value.status == capi.SCF_ERR_BAD_ARG
    bad = g.copy()
    bad.fams["v"].arrays["phi"] = None
    with pytest.raises(ScfError) as e:
        gp(bad)
    assert e.value.status == capi.SCF_ERR_BAD_ARG
    L = gp.L
    ctx = C.c_void_p()
    assert L.scf_geo_create(C.byref(ctx), 1, 8, 8, 0) == capi.SCF_ERR_BAD_ARG
