"""VTK XML rectilinear-grid (.vtr) writer for level fields.

The reference writes its results with pyevtk's ``gridToVTK``
(go_melt/computeFunctions.py:1945-2057); pyevtk is not available here, so
this module writes the same file type itself: an ``<ImageData>``-free
``RectilinearGrid`` with the three coordinate arrays and point data arrays,
raw little-endian binary in an appended section (the layout pyevtk uses),
node order x fastest — the order of the device arrays, so no transpose.
"""

from __future__ import annotations

import numpy as np

_TYPES = {np.dtype(np.float32): "Float32", np.dtype(np.float64): "Float64", np.dtype(np.uint8): "UInt8",
          np.dtype(np.int32): "Int32", np.dtype(np.int64): "Int64"}


def write_vtr(path, x, y, z, point_data):
    """Write ``path + '.vtr'``; x, y, z: node coordinates per axis;
    point_data: {name: array of nx*ny*nz values, x fastest}.  Returns the
    file name."""
    x, y, z = (np.ascontiguousarray(np.asarray(a, dtype=np.float64)) for a in (x, y, z))
    nx, ny, nz = x.size, y.size, z.size
    arrays = []
    for name, v in point_data.items():
        a = np.ascontiguousarray(np.asarray(v).reshape(-1))
        if a.dtype == np.bool_:
            a = a.astype(np.uint8)
        if a.dtype not in _TYPES:
            a = a.astype(np.float64)
        if a.size != nx * ny * nz:
            raise ValueError(f"point data {name!r} has {a.size} values, grid has {nx * ny * nz}")
        arrays.append((name, a))
    blocks = []
    offset = 0
    coord_xml = []
    for name, a in (("x_coordinates", x), ("y_coordinates", y), ("z_coordinates", z)):
        coord_xml.append(f'<DataArray type="Float64" Name="{name}" NumberOfComponents="1" format="appended" '
                         f'offset="{offset}"/>')
        blocks.append(a)
        offset += 8 + a.nbytes
    pd_xml = []
    for name, a in arrays:
        pd_xml.append(f'<DataArray type="{_TYPES[a.dtype]}" Name="{name}" NumberOfComponents="1" '
                      f'format="appended" offset="{offset}"/>')
        blocks.append(a)
        offset += 8 + a.nbytes
    ext = f"0 {nx - 1} 0 {ny - 1} 0 {nz - 1}"
    head = ('<?xml version="1.0"?>\n'
            '<VTKFile type="RectilinearGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n'
            f'<RectilinearGrid WholeExtent="{ext}">\n<Piece Extent="{ext}">\n'
            '<Coordinates>\n' + "\n".join(coord_xml) + '\n</Coordinates>\n'
            '<PointData>\n' + "\n".join(pd_xml) + '\n</PointData>\n'
            '</Piece>\n</RectilinearGrid>\n<AppendedData encoding="raw">\n_')
    fname = str(path) + ".vtr"
    with open(fname, "wb") as f:
        f.write(head.encode("ascii"))
        for a in blocks:
            le = a.astype(a.dtype.newbyteorder("<"), copy=False)
            f.write(np.uint64(le.nbytes).tobytes())
            f.write(le.tobytes())
        f.write(b"\n</AppendedData>\n</VTKFile>\n")
    return fname


def read_vtr(fname):
    """Read a file written by write_vtr: (x, y, z, {name: array})."""
    import re

    with open(fname, "rb") as f:
        data = f.read()
    start = data.index(b"<AppendedData encoding=\"raw\">\n_") + len(b"<AppendedData encoding=\"raw\">\n_")
    head = data[:start].decode("ascii")
    inv = {v: k for k, v in _TYPES.items()}
    out = {}
    coords = {}
    for typ, name, off in re.findall(r'<DataArray type="(\w+)" Name="([^"]+)" NumberOfComponents="1" '
                                     r'format="appended" offset="(\d+)"/>', head):
        o = start + int(off)
        n = int(np.frombuffer(data[o:o + 8], dtype="<u8")[0])
        a = np.frombuffer(data[o + 8:o + 8 + n], dtype=inv[typ].newbyteorder("<"))
        if name.endswith("_coordinates"):
            coords[name[0]] = a
        else:
            out[name] = a
    return coords["x"], coords["y"], coords["z"], out
