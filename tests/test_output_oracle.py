"""The output oracle (oracle/vtr.py) and the reader
(simcoflow3d_gb300/output.py): the file of PrintResultVTK's layout round
trips -- node coordinates as Float32 of the centres -+ half widths, cell data
rounded to Float32, i fastest, fields in the reference's order.  CPU only."""
import numpy as np

from simcoflow3d_gb300 import output as OUT, workloads as W
from oracle import vtr as V


def _axes(w):
    a = w.arrays
    return (np.cumsum(a["pgrid_dx"][:, 0, 0]) - a["pgrid_dx"][:, 0, 0] / 2,
            a["pgrid_dx"][:, 0, 0],
            np.cumsum(a["pgrid_dy"][0, :, 0]) - a["pgrid_dy"][0, :, 0] / 2, a["pgrid_dy"][0, :, 0],
            np.cumsum(a["pgrid_dz"][0, 0, :]) - a["pgrid_dz"][0, 0, :] / 2, a["pgrid_dz"][0, 0, :])


def test_oracle_file_round_trips(tmp_path):
    w = W.config("c1", n=12, random_tvar=True)
    a = w.arrays
    fields = list(zip(OUT.PRINT_RESULT_VTK_FIELDS[:4], (a["tvar_p"], a["tvar_u"], a["tvar_v"], a["tvar_w"])))
    fields += [("LiquidLvs", a["phil"]), ("LiquidVof", a["vofl"]), ("FluidVof", a["vof"])]
    axes = _axes(w)
    path = str(tmp_path / "f.vtr")
    V.write_vtr(path, (w.imax, w.jmax, w.kmax), axes, fields)
    got = OUT.read_vtr(path)
    assert list(got)[:3] == ["X_COORDINATES", "Y_COORDINATES", "Z_COORDINATES"]
    assert np.array_equal(got["X_COORDINATES"], V.nodes(axes[0], axes[1]))
    assert got["X_COORDINATES"].size == w.imax + 1
    for name, arr in fields:
        want = arr[1:-1, 1:-1, 1:-1].astype(np.float32)
        assert got[name].dtype == np.float32 and np.array_equal(got[name], want), name
    # uniform unit cube: nodes 0, 1/12, ..., 1
    assert abs(got["X_COORDINATES"][-1] - 1.0) < 1e-6 and got["X_COORDINATES"][0] == 0.0
