"""GPU field output (include/scf_output.h): the projection context's
device-resident fields (corrected u, v, w, p and the staged phiL, vofL, vof)
and a host field (the solid level set) written by scf_write_vtr (appended
raw) and scf_write_vtr_binary (VTKFortran's inline base64, the reference's
own file) give files byte-identical to the oracle's (oracle/vtr.py) from the
same values on the host, in PrintResultVTK's field order."""
import numpy as np
import pytest

from simcoflow3d_gb300 import output as OUT, workloads as W
from oracle import vtr as V

pytestmark = pytest.mark.gpu


def _axes(w):
    a = w.arrays
    dx, dy, dz = a["pgrid_dx"][:, 0, 0], a["pgrid_dy"][0, :, 0], a["pgrid_dz"][0, 0, :]
    return (np.cumsum(dx) - dx / 2, dx, np.cumsum(dy) - dy / 2, dy, np.cumsum(dz) - dz / 2, dz)


@pytest.mark.parametrize("encoding", ["appended", "binary"])
@pytest.mark.parametrize("name,n", [("c1", 24), ("c4", 12), ("c1", 17)])
def test_device_fields_to_vtr(gpu_lib, tmp_path, name, n, encoding):
    from simcoflow3d_gb300.projection import Projection
    w = W.config(name, n=n)
    p = Projection.for_workload(w, rel_tol=1e-10)
    u, v, ww, pp, _, _ = p.update_puvw(w)
    dev = p.device_fields()
    phi = np.zeros(w.shape_g, order="F")
    phi[1:-1, 1:-1, 1:-1] = w.arrays["pcell_phi"]
    names = OUT.PRINT_RESULT_VTK_FIELDS
    gpu_fields = [(names[0], dev["p"]), (names[1], dev["u"]), (names[2], dev["v"]), (names[3], dev["w"]),
                  (names[4], dev["phil"]), (names[5], phi), (names[6], dev["vofl"]), (names[7], dev["vof"])]
    host_fields = [(names[0], pp), (names[1], u), (names[2], v), (names[3], ww), (names[4], w.arrays["phil"]),
                   (names[5], phi), (names[6], w.arrays["vofl"]), (names[7], w.arrays["vof"])]
    axes = _axes(w)
    shape = (w.imax, w.jmax, w.kmax)
    f_gpu, f_ref = str(tmp_path / "gpu.vtr"), str(tmp_path / "ref.vtr")
    st = OUT.write_vtr(f_gpu, shape, axes, gpu_fields, encoding=encoding)
    (V.write_vtr if encoding == "appended" else V.write_vtr_binary)(f_ref, shape, axes, host_fields)
    assert open(f_gpu, "rb").read() == open(f_ref, "rb").read()
    launches = 8 if encoding == "appended" else 16
    assert st["gpu_launches"] == launches and st["bytes_file"] == len(open(f_gpu, "rb").read())
    got = OUT.read_vtr(f_gpu)
    assert np.array_equal(got["u"], u[1:-1, 1:-1, 1:-1].astype(np.float32))
    p.close()


def test_bad_arguments(gpu_lib, tmp_path):
    from simcoflow3d_gb300.projection import ScfError
    w = W.config("c1", n=8)
    with pytest.raises(ScfError):
        OUT.write_vtr(str(tmp_path / "x.vtr"), (8, 8, 8), _axes(w), [('bad"name', w.arrays["vof"])])
    with pytest.raises(ScfError):
        OUT.write_vtr(str(tmp_path / "nodir" / "x.vtr"), (8, 8, 8), _axes(w), [("vof", w.arrays["vof"])])
