"""The synthetic workloads follow the reference's conventions."""
import numpy as np
import pytest

from simcoflow3d_gb300 import workloads as W


@pytest.mark.parametrize("name,n", [("c0", 12), ("c1", 16), ("c2", 16), ("c4", 8)])
def test_workload_invariants(name, n):
    w = W.config(name, n=n)
    a = w.arrays
    ct, pos = a["cell_type"], a["posnu"]
    # NumberExternalCell numbering: loop order, k innermost
    act = (ct != 2)
    order = np.transpose(act, (0, 1, 2)).ravel(order="C")
    expect = np.where(order, np.cumsum(order) - 1, -1).reshape(act.shape, order="C")
    assert np.array_equal(pos, expect)
    assert w.ext_cell == act.sum() - 1
    # DefineCell: vof in {0} U (eps,1-eps] U {1}, solid <=> vof == 0
    vof = a["vof"][1:-1, 1:-1, 1:-1]
    assert ((vof == 0) == (ct == 2)).all()
    assert ((vof == 1) | (vof == 0) | ((vof > 1e-3) & (vof < 1 - 1e-3))).all()
    for k in ("eearea", "nearea", "tearea"):
        assert (a[k] >= 0).all() and (a[k] <= 1).all()
    # faces of solid cells are closed (CellGeoCal)
    EE = a["eearea"]
    s = ct == 2
    assert (EE[1:-1, 1:-1, 1:-1][s] == 0).all() and (EE[:-2, 1:-1, 1:-1][s] == 0).all()
    # Dp = dt on open velocity cells, 0 on solid ones (PredictUVW.f90:907,1235)
    dpu = a["dp_u"][1:-1, 1:-1, 1:-1][: w.imax - 1]
    ctu = a["ucell_cell_type"][: w.imax - 1]
    assert np.allclose(dpu[ctu != 2], w.dt, rtol=1e-13) and (dpu[ctu == 2] == 0).all()
    # wall-normal predicted velocity vanishes on Neumann-pressure walls
    if w.bcp_flag[0] == 1:
        assert (a["u_star"][0] == 0).all()
    if w.bcp_flag[5] == 1:
        assert (a["w_star"][:, :, w.kmax] == 0).all()


def test_volume_fraction_limits():
    # full box, empty box and a half-space through the centre
    one = np.ones(4)
    v = W.volume_fraction_calc(one, one, one, np.array([1.0, 0.0, 0.6, 0.0]), np.array([0.0, 1.0, 0.8, 0.0]),
                               np.array([0.0, 0.0, 0.0, 1.0]), np.array([2.0, -1.0, 0.7, 0.5]))
    assert v[0] == 1.0 and v[1] == 0.0 and abs(v[2] - 0.5) < 1e-15 and abs(v[3] - 0.5) < 1e-15


def test_face_area_limits():
    # open, closed and half-cut faces
    a = W.face_geo_area(np.ones(3), np.ones(3), np.array([1.0, 1.0, 1.0]), np.zeros(3), np.zeros(3), np.zeros(3),
                        np.array([5.0, -5.0, 0.0]))
    assert a[0] == 1.0 and a[1] == 0.0 and abs(a[2] - 0.5) < 1e-15
