"""Field output (include/scf_output.h): the VTK XML RectilinearGrid that
PrintResultVTK writes (src/PrintResult.f90:328-421), from device-resident
or host FP64 fields, and a reader for it.

``PRINT_RESULT_VTK_FIELDS`` is the reference's field list and order: p, u,
v, w of TVar, then phiL, phi, vofL and vof of PCell.
"""
from __future__ import annotations

import ctypes as C
import re
from typing import Dict, Iterable, Optional, Sequence, Tuple

import numpy as np

from . import capi

PRINT_RESULT_VTK_FIELDS = ("p", "u", "v", "w", "LiquidLvs", "FluidLvs", "LiquidVof", "FluidVof")


def write_vtr(path: str, shape: Tuple[int, int, int], axes: Sequence[np.ndarray],
              fields: Iterable[Tuple[str, object]], device: int = 0, lib=None, encoding: str = "appended") -> dict:
    """Writes ``fields`` to ``path``.  ``axes`` = (xc, dx, yc, dy, zc, dz), the
    cell centres and widths of each axis (host, FP64).  Each field is
    (name, array) with a ghosted Fortran-ordered FP64 host array, or
    (name, int) with a device pointer to one.  ``encoding``: "appended"
    (raw arrays in an appended section, scf_write_vtr) or "binary"
    (VTKFortran's inline base64, the reference's own file,
    scf_write_vtr_binary).  Returns the call's stats."""
    from .projection import load_library, ScfError
    L = lib or load_library()
    I, J, K = shape
    ax = [np.ascontiguousarray(a, dtype=np.float64) for a in axes]
    capi.require([a.size for a in ax] == [I, I, J, J, K, K], "axes must hold I, I, J, J, K, K values")
    fl = list(fields)
    arr = (capi.ScfVtrField * max(1, len(fl)))()
    keep = []
    for q, (name, data) in enumerate(fl):
        if isinstance(data, np.ndarray):
            capi.require(data.dtype == np.float64 and data.flags.f_contiguous and data.shape == (I + 2, J + 2, K + 2),
                         f"field {name}: a ghosted Fortran-ordered FP64 array of shape {(I + 2, J + 2, K + 2)} is required")
            keep.append(data)
            arr[q].data = data.ctypes.data
            arr[q].on_device = 0
        else:
            arr[q].data = int(data)
            arr[q].on_device = 1
        arr[q].name = name.encode()
    st = capi.ScfVtrStats()
    capi.require(encoding in ("appended", "binary"), "encoding must be 'appended' or 'binary'")
    fn = L.scf_write_vtr if encoding == "appended" else L.scf_write_vtr_binary
    rc = fn(path.encode(), I, J, K, *(capi.dptr(a) for a in ax), len(fl), arr, device, C.byref(st))
    if rc != 0:
        raise ScfError(rc, "scf_write_vtr failed for %s" % path)
    return {k: getattr(st, k) for k, _ in capi.ScfVtrStats._fields_}


def read_vtr(path: str) -> Dict[str, np.ndarray]:
    """The arrays of a file written by write_vtr, in either layout:
    the coordinates (X_COORDINATES ... in the appended layout, X, Y, Z in
    the inline one) as 1-D Float32, cell fields as (I, J, K) Float32 arrays
    in Fortran order."""
    raw = open(path, "rb").read()
    if b'format="binary"' in raw:
        return _read_vtr_binary(raw)
    head_end = raw.index(b'<AppendedData encoding="raw">') + len(b'<AppendedData encoding="raw">')
    head = raw[:head_end].decode()
    base = raw.index(b"_", head_end) + 1
    ext = [int(v) for v in re.search(r'WholeExtent="([^"]+)"', head).group(1).split()]
    I, J, K = ext[1] - 1, ext[3] - 1, ext[5] - 1
    out = {}
    for name, off in re.findall(r'Name="([^"]+)" NumberOfComponents="1" format="appended" offset="(\d+)"', head):
        p = base + int(off)
        nb = int(np.frombuffer(raw, dtype="<u8", count=1, offset=p)[0])
        a = np.frombuffer(raw, dtype="<f4", count=nb // 4, offset=p + 8).copy()
        if name.endswith("_COORDINATES"):
            out[name] = a
        else:
            out[name] = a.reshape((I, J, K), order="F")
    return out


def _read_vtr_binary(raw: bytes) -> Dict[str, np.ndarray]:
    import base64
    text = raw.decode()
    ext = [int(v) for v in re.search(r'WholeExtent="([^"]+)"', text).group(1).split()]
    I, J, K = ext[1] - 1, ext[3] - 1, ext[5] - 1
    out = {}
    for name, code in re.findall(r'Name="([^"]+)" format="binary">\s*([A-Za-z0-9+/=]+)\s*</DataArray>', text):
        b = base64.b64decode(code)
        nb = int(np.frombuffer(b, dtype="<i4", count=1)[0])
        a = np.frombuffer(b, dtype="<f4", count=nb // 4, offset=4).copy()
        out[name] = a if name in ("X", "Y", "Z") else a.reshape((I, J, K), order="F")
    return out
