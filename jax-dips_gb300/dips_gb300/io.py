"""Solution output on the evaluation grid as VTK XML structured-grid files (.vts), the format the
reference writes through ``structuredToVTK`` (utils/io.py:80-88, write_vtk_manual; :62-78,
write_vtk_solution).

The writer follows the public VTK XML file-format specification: a ``StructuredGrid`` whose
point coordinates and point fields are stored as raw little-endian binary in one
``AppendedData`` block, each array preceded by its byte count (UInt64 header).  Grids are
meshgrid(x, y, z, indexing='ij') with x varying fastest in the file (VTK's point order), which
is the Fortran-order flattening of the 'ij' arrays.
"""

from __future__ import annotations

import os

import numpy as np

_VTK_TYPES = {np.dtype(np.float32): "Float32", np.dtype(np.float64): "Float64", np.dtype(np.int32): "Int32",
              np.dtype(np.int64): "Int64", np.dtype(np.uint8): "UInt8"}


def _host(a):
    try:
        import torch

        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy()
    except Exception:  # pragma: no cover
        pass
    return np.asarray(a)


def write_structured_vts(path: str, X, Y, Z, point_data: dict) -> str:
    """Write a structured grid with point fields; ``path`` without extension, returns the file name.

    X, Y, Z and every field are arrays of the grid's shape (nx, ny, nz) ('ij' indexing); a field
    of shape (nx, ny, nz, 3) is written as a 3-component vector.
    """
    X, Y, Z = (np.asarray(_host(a)) for a in (X, Y, Z))
    shape = X.shape
    if len(shape) != 3 or Y.shape != shape or Z.shape != shape:
        raise ValueError("X, Y, Z must be 3-D arrays of one shape")
    nx, ny, nz = shape
    arrays = []  # (name, components, flat little-endian array)
    pts = np.stack([X, Y, Z], axis=-1)
    pts = np.ascontiguousarray(pts.transpose(2, 1, 0, 3).reshape(-1, 3))  # x fastest
    arrays.append(("Points", 3, pts.astype(pts.dtype.newbyteorder("<"))))
    for name, val in point_data.items():
        a = np.asarray(_host(val))
        if a.dtype not in _VTK_TYPES:
            a = a.astype(np.float32)
        if a.shape == shape:
            arrays.append((name, 1, np.ascontiguousarray(a.transpose(2, 1, 0).reshape(-1))))
        elif a.shape == shape + (3,):
            arrays.append((name, 3, np.ascontiguousarray(a.transpose(2, 1, 0, 3).reshape(-1, 3))))
        elif a.size == nx * ny * nz:  # flat field in the grid's C order ('ij')
            arrays.append((name, 1, np.ascontiguousarray(a.reshape(shape).transpose(2, 1, 0).reshape(-1))))
        else:
            raise ValueError(f"field {name!r} has shape {a.shape}, grid is {shape}")
    extent = f"0 {nx - 1} 0 {ny - 1} 0 {nz - 1}"
    offsets, off = [], 0
    for _, _, a in arrays:
        offsets.append(off)
        off += 8 + a.nbytes
    lines = ['<?xml version="1.0"?>',
             '<VTKFile type="StructuredGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">',
             f'<StructuredGrid WholeExtent="{extent}">', f'<Piece Extent="{extent}">']
    names = [n for n, _, _ in arrays[1:]]
    lines.append(f'<PointData Scalars="{names[0]}">' if names else "<PointData>")
    for (name, comp, a), o in zip(arrays[1:], offsets[1:]):
        lines.append(f'<DataArray type="{_VTK_TYPES[a.dtype]}" Name="{name}" NumberOfComponents="{comp}" '
                     f'format="appended" offset="{o}"/>')
    lines.append("</PointData>")
    lines.append("<Points>")
    a0 = arrays[0][2]
    lines.append(f'<DataArray type="{_VTK_TYPES[a0.dtype]}" NumberOfComponents="3" format="appended" offset="0"/>')
    lines += ["</Points>", "</Piece>", "</StructuredGrid>", '<AppendedData encoding="raw">']
    fname = path + ".vts"
    d = os.path.dirname(fname)
    if d:
        os.makedirs(d, exist_ok=True)
    with open(fname, "wb") as f:
        f.write(("\n".join(lines) + "\n_").encode())
        for _, _, a in arrays:
            b = a.astype(a.dtype.newbyteorder("<"), copy=False).tobytes()
            f.write(np.uint64(len(b)).astype("<u8").tobytes())
            f.write(b)
        f.write(b"\n</AppendedData>\n</VTKFile>\n")
    return fname


def _mesh(gstate):
    return np.meshgrid(np.asarray(gstate.x), np.asarray(gstate.y), np.asarray(gstate.z), indexing="ij")


def write_vtk_manual(gstate, field_dict: dict, filename: str = "results/manual_dump") -> str:
    """``write_vtk_manual`` (utils/io.py:80-88): point fields on the grid of ``gstate``."""
    X, Y, Z = _mesh(gstate)
    return write_structured_vts(filename, X, Y, Z, {k: _host(v) for k, v in field_dict.items()})


def write_vtk_solution(gstate, log, address: str = "results/", maxsteps=None):
    """``write_vtk_solution`` (utils/io.py:62-78): one file ``solutionNNNN.vts`` per entry of
    ``log["U"]``."""
    X, Y, Z = _mesh(gstate)
    out = []
    for i, sol in enumerate(log["U"]):
        out.append(write_structured_vts(os.path.join(address, "solution" + str(i).zfill(4)), X, Y, Z,
                                        {"sol": np.asarray(_host(sol)).reshape(X.shape)}))
        if maxsteps and i >= maxsteps - 1:
            break
    return out


def read_vts(fname: str) -> dict:
    """Read back a file written by ``write_structured_vts`` (the point coordinates under
    "Points", each field by name, all in VTK point order)."""
    import re

    data = open(fname, "rb").read()
    head, _, rest = data.partition(b'<AppendedData encoding="raw">')
    blob = rest[rest.index(b"_") + 1 :]
    out = {}
    inv = {v: k for k, v in _VTK_TYPES.items()}
    for m in re.finditer(rb'<DataArray type="(\w+)"(?: Name="([^"]+)")? NumberOfComponents="(\d+)" '
                         rb'format="appended" offset="(\d+)"/>', head):
        typ, name, comp, off = m.group(1).decode(), m.group(2), int(m.group(3)), int(m.group(4))
        n = int(np.frombuffer(blob[off : off + 8], "<u8")[0])
        arr = np.frombuffer(blob[off + 8 : off + 8 + n], inv[typ].newbyteorder("<"))
        out[name.decode() if name else "Points"] = arr.reshape(-1, comp) if comp > 1 else arr
    return out
