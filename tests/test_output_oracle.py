"""The output oracle (oracle/vtr.py) and the reader
(simcoflow3d_gb300/output.py): the file of PrintResultVTK's layout round
trips -- node coordinates as Float32 of the centres -+ half widths, cell data
rounded to Float32, i fastest, fields in the reference's order -- in both
layouts.  The inline (VTKFortran "BINARY") layout's base64 is pinned to
BeFoR64's own documented examples, and its text to a file written out by
hand from VTKFortran's tag routines.  CPU only."""
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


def test_base64_matches_befor64_examples():
    """The encodings BeFoR64 documents for its b64_encode calls
    (src/VTKFortran/src/third_party/BeFoR64/src/lib/befor64.F90: the
    examples of b64_encode_up / b64_encode on R4P, I1P, R8P and a string)."""
    assert V.b64(np.array([0.0, -32.12], dtype="<f4").tobytes()) == "AAAAAOF6AMI="
    assert V.b64(np.array([120, -1], dtype=np.int8).tobytes()) == "eP8="
    assert V.b64(np.array([120], dtype=np.int8).tobytes()) == "eA=="
    assert V.b64(np.array([1.0], dtype="<f8").tobytes()) == "AAAAAAAA8D8="
    assert V.b64(np.array([1.0, 2.0], dtype="<f8").tobytes()) == "AAAAAAAA8D8AAAAAAAAAQA=="
    assert V.b64(b"hello") == "aGVsbG8="


def test_binary_layout_is_vtkfortrans_text(tmp_path):
    """A 1x1x2 grid with one field, against the text VTKFortran's
    xml_writer_binary_local produces for PrintResultVTK, written out here by
    hand: XML declaration, VTKFile without a header_type, extents with
    PENF's '+' signs, tags indented 2 per level, each array's base64 on its
    own line 2 deeper, closing tags indented like their opening ones."""
    axes = (np.array([0.5]), np.array([1.0]), np.array([0.5]), np.array([1.0]), np.array([0.25, 0.75]),
            np.array([0.5, 0.5]))
    f = np.zeros((3, 3, 4), order="F")
    f[1, 1, 1], f[1, 1, 2] = 1.5, -2.0
    path = str(tmp_path / "t.vtr")
    V.write_vtr_binary(path, (1, 1, 2), axes, [("p", f)])
    b = lambda *v: V.b64_dataarray(np.array(v, dtype=np.float32))
    want = ('<?xml version="1.0"?>\n'
            '<VTKFile type="RectilinearGrid" version="1.0" byte_order="LittleEndian">\n'
            '  <RectilinearGrid WholeExtent="+1 +2 +1 +2 +1 +3">\n'
            '    <Piece Extent="+1 +2 +1 +2 +1 +3">\n'
            '      <Coordinates>\n'
            '        <DataArray type="Float32" NumberOfComponents="1" Name="X" format="binary">\n'
            '          ' + b(0.0, 1.0) + '\n'
            '        </DataArray>\n'
            '        <DataArray type="Float32" NumberOfComponents="1" Name="Y" format="binary">\n'
            '          ' + b(0.0, 1.0) + '\n'
            '        </DataArray>\n'
            '        <DataArray type="Float32" NumberOfComponents="1" Name="Z" format="binary">\n'
            '          ' + b(0.0, 0.5, 1.0) + '\n'
            '        </DataArray>\n'
            '      </Coordinates>\n'
            '      <CellData>\n'
            '        <DataArray type="Float32" NumberOfComponents="1" Name="p" format="binary">\n'
            '          ' + b(1.5, -2.0) + '\n'
            '        </DataArray>\n'
            '      </CellData>\n'
            '    </Piece>\n'
            '  </RectilinearGrid>\n'
            '</VTKFile>\n')
    assert open(path).read() == want
    # the header of X: Int32 8 (two Float32) in front of the data
    assert b(0.0, 1.0) == V.b64(np.int32(8).tobytes() + np.array([0.0, 1.0], dtype="<f4").tobytes())


def test_binary_oracle_file_round_trips(tmp_path):
    w = W.config("c1", n=10, random_tvar=True)
    a = w.arrays
    fields = list(zip(OUT.PRINT_RESULT_VTK_FIELDS[:4], (a["tvar_p"], a["tvar_u"], a["tvar_v"], a["tvar_w"])))
    axes = _axes(w)
    path = str(tmp_path / "b.vtr")
    V.write_vtr_binary(path, (w.imax, w.jmax, w.kmax), axes, fields)
    got = OUT.read_vtr(path)
    assert np.array_equal(got["X"], V.nodes(axes[0], axes[1]))
    for name, arr in fields:
        assert np.array_equal(got[name], arr[1:-1, 1:-1, 1:-1].astype(np.float32)), name
