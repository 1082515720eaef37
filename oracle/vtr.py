"""Oracle of the field output (test infrastructure only): the files that
scf_write_vtr and scf_write_vtr_binary write, restated with numpy from host
FP64 fields -- node coordinates as Float32 of c - w/2 (and c + w/2 past the
last cell), cell data as the interior values rounded to Float32, i fastest,
as PrintResultVTK and WriteDataArrayVTK form them
(src/PrintResult.f90:328-421).

``write_vtr_binary`` restates the file VTKFortran writes for
PrintResultVTK's initialize(format='BINARY') (src/VTKFortran/src/lib/):
- vtk_fortran_vtk_file_xml_writer_abstract.f90: write_header_tag (the XML
  declaration and VTKFile line, 776-794), write_topology_tag (WholeExtent,
  845-900), write_piece_start_tag (Extent, 1084-1106), write_geo_rect (X, Y,
  Z arrays inside Coordinates, 1162-1181), write_dataarray_location_tag
  (CellData, 968-1029), write_dataarray_tag (type, NumberOfComponents, Name,
  format, 903-933), write_start_tag / write_end_tag / write_tag (indent 2
  per level, the content on its own line indented 2 deeper, 761-843);
- FoXy's xml_tag stringify (third_party/FoXy/src/lib/foxy_xml_tag.F90);
- PENF's str(n=...) for the extents: an explicit '+' sign
  (third_party/PENF/src/lib/penf_stringify.F90:424-446);
- encode_binary_dataarray (vtk_fortran_dataarray_encoder.f90:1047-1062):
  base64 (BeFoR64's b64_encode, RFC 4648 with '=' padding) of the Int32 byte
  count followed by the Float32 data.
"""
from __future__ import annotations

import numpy as np


def nodes(c, w):
    c = np.asarray(c, dtype=np.float64)
    w = np.asarray(w, dtype=np.float64)
    return np.concatenate([(c - w / 2.0).astype(np.float32), [np.float32(c[-1] + w[-1] / 2.0)]])


def write_vtr(path, shape, axes, fields):
    I, J, K = shape
    X, Y, Z = nodes(axes[0], axes[1]), nodes(axes[2], axes[3]), nodes(axes[4], axes[5])
    ext = "1 %d 1 %d 1 %d" % (I + 1, J + 1, K + 1)
    arrays = [("X_COORDINATES", X), ("Y_COORDINATES", Y), ("Z_COORDINATES", Z)]
    for name, a in fields:
        arrays.append((name, np.asarray(a)[1:-1, 1:-1, 1:-1].astype(np.float32).ravel(order="F")))
    h = ['<?xml version="1.0"?>\n',
         '<VTKFile type="RectilinearGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n',
         '  <RectilinearGrid WholeExtent="%s">\n' % ext, '    <Piece Extent="%s">\n' % ext]
    off = 0
    lines = []
    for name, a in arrays:
        lines.append('        <DataArray type="Float32" Name="%s" NumberOfComponents="1" format="appended" '
                     'offset="%d"/>\n' % (name, off))
        off += 8 + a.nbytes
    h += ["      <Coordinates>\n"] + lines[:3] + ["      </Coordinates>\n", "      <CellData>\n"] + lines[3:]
    h += ["      </CellData>\n", "    </Piece>\n", "  </RectilinearGrid>\n", '  <AppendedData encoding="raw">\n_']
    with open(path, "wb") as f:
        f.write("".join(h).encode())
        for _, a in arrays:
            f.write(np.uint64(a.nbytes).tobytes())
            f.write(a.astype("<f4").tobytes())
        f.write(b"\n  </AppendedData>\n</VTKFile>\n")


def b64(data: bytes) -> str:
    """BeFoR64's b64_encode of a byte stream: RFC 4648 base64, '=' padding,
    no line breaks (third_party/BeFoR64/src/lib/befor64.F90:187-233)."""
    import base64
    return base64.b64encode(bytes(data)).decode()


def b64_dataarray(a) -> str:
    """VTKFortran's encode_binary_dataarray of a Float32 array: base64 of its
    Int32 byte count followed by the data, little endian."""
    a = np.ascontiguousarray(a, dtype="<f4")
    return b64(np.int32(a.nbytes).astype("<i4").tobytes() + a.tobytes())


def write_vtr_binary(path, shape, axes, fields):
    I, J, K = shape
    X, Y, Z = nodes(axes[0], axes[1]), nodes(axes[2], axes[3]), nodes(axes[4], axes[5])
    ext = "+1 +%d +1 +%d +1 +%d" % (I + 1, J + 1, K + 1)

    def array(name, a):
        return ('        <DataArray type="Float32" NumberOfComponents="1" Name="%s" format="binary">\n'
                '          %s\n        </DataArray>\n' % (name, b64_dataarray(a)))

    out = ['<?xml version="1.0"?>\n',
           '<VTKFile type="RectilinearGrid" version="1.0" byte_order="LittleEndian">\n',
           '  <RectilinearGrid WholeExtent="%s">\n' % ext, '    <Piece Extent="%s">\n' % ext,
           "      <Coordinates>\n", array("X", X), array("Y", Y), array("Z", Z), "      </Coordinates>\n",
           "      <CellData>\n"]
    for name, a in fields:
        out.append(array(name, np.asarray(a)[1:-1, 1:-1, 1:-1].astype(np.float32).ravel(order="F")))
    out += ["      </CellData>\n", "    </Piece>\n", "  </RectilinearGrid>\n", "</VTKFile>\n"]
    with open(path, "wb") as f:
        f.write("".join(out).encode())
