"""Oracle of the field output (test infrastructure only): the file that
scf_write_vtr writes, restated with numpy from host FP64 fields -- node
coordinates as Float32 of c - w/2 (and c + w/2 past the last cell), cell
data as the interior values rounded to Float32, i fastest, as
PrintResultVTK and WriteDataArrayVTK form them (src/PrintResult.f90:328-421).
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
