"""VTK XML unstructured-grid (``.vtu``) output of a phase-field solution,
written headless from device buffers.

The reference writes its solution files with meshio (``allen_cahn.py:
182-210``: cell data ``T``, ``ori_inds`` and the IPF colours ``ipf_x/y/z`` on
the polycrystal's hexahedral mesh).  meshio is not a dependency here, so this
module writes the same file format itself: the structured grid as hexahedra
(VTK cell type 12), points in float32 or float64, connectivity and offsets in
int32 or int64 as the size needs, cell data arrays as they are given, all as
raw little-endian binary appended after the XML header (``encoding="raw"``,
``header_type="UInt64"``), which ParaView and meshio read.  The IPF colour
arrays are written when the polycrystal supplies its orientations' colours
(computing them needs orix's colour key, which is plotting only and not
reproduced here).

``read_vtu`` reads back what ``write_vtu`` writes (used by the tests).
"""
import os
import re
import xml.etree.ElementTree as ET

import numpy as np
import torch

_VTK_TYPES = {np.dtype("float32"): "Float32", np.dtype("float64"): "Float64",
              np.dtype("int32"): "Int32", np.dtype("int64"): "Int64",
              np.dtype("uint8"): "UInt8", np.dtype("int8"): "Int8"}
_NP_TYPES = {v: k for k, v in _VTK_TYPES.items()}
HEXAHEDRON = 12


def _host(a):
    if torch.is_tensor(a):
        a = a.detach().cpu().numpy()
    a = np.asarray(a)
    if a.dtype == np.bool_:
        a = a.astype(np.uint8)
    return np.ascontiguousarray(a)


def grid_points(shape_xyz, h, origin=(0.0, 0.0, 0.0), dtype=np.float32):
    """(Nx+1)(Ny+1)(Nz+1) corner points, x fastest."""
    Nx, Ny, Nz = shape_xyz
    xs = origin[0] + h[0] * np.arange(Nx + 1)
    ys = origin[1] + h[1] * np.arange(Ny + 1)
    zs = origin[2] + h[2] * np.arange(Nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    return np.stack((X.ravel(), Y.ravel(), Z.ravel()), axis=1).astype(dtype)


def grid_hexahedra(shape_xyz, dtype=np.int64):
    """(N, 8) corner indices of the cells in z-major order (x fastest), in
    VTK's hexahedron order: the bottom face counter-clockwise, then the top."""
    Nx, Ny, Nz = shape_xyz
    px, pxy = Nx + 1, (Nx + 1) * (Ny + 1)
    z, y, x = np.meshgrid(np.arange(Nz, dtype=dtype), np.arange(Ny, dtype=dtype),
                          np.arange(Nx, dtype=dtype), indexing="ij")
    p0 = (z * pxy + y * px + x).ravel()
    return np.stack((p0, p0 + 1, p0 + 1 + px, p0 + px,
                     p0 + pxy, p0 + pxy + 1, p0 + pxy + 1 + px, p0 + pxy + px), axis=1)


def write_vtu(path, shape_xyz, h, cell_data, origin=(0.0, 0.0, 0.0)):
    """Write the grid ``shape_xyz`` (cells) of cell size ``h`` with the given
    cell data (name -> array of N or (N, k) values; CUDA tensors are copied to
    the host) to ``path``."""
    Nx, Ny, Nz = (int(v) for v in shape_xyz)
    N = Nx * Ny * Nz
    npts = (Nx + 1) * (Ny + 1) * (Nz + 1)
    idx_t = np.int32 if npts < 2 ** 31 and 8 * N < 2 ** 31 else np.int64
    pts = grid_points((Nx, Ny, Nz), h, origin)
    conn = grid_hexahedra((Nx, Ny, Nz), idx_t)
    offsets = (8 * np.arange(1, N + 1, dtype=np.int64)).astype(idx_t)
    types = np.full(N, HEXAHEDRON, dtype=np.uint8)
    blocks, xml_arrays = [], []
    offset = 0

    def add(name, arr, ncomp):
        nonlocal offset
        arr = _host(arr)
        xml_arrays.append((name, _VTK_TYPES[arr.dtype], ncomp, offset))
        blocks.append(arr)
        offset += 8 + arr.nbytes
        return len(xml_arrays) - 1

    data_xml = []
    for name, arr in cell_data.items():
        arr = _host(arr)
        if arr.shape[0] != N:
            raise ValueError(f"cell data {name!r} has {arr.shape[0]} rows, expected {N}")
        ncomp = 1 if arr.ndim == 1 else int(np.prod(arr.shape[1:]))
        data_xml.append(add(name, arr.reshape(N, -1) if ncomp > 1 else arr.reshape(N), ncomp))
    p_i = add("Points", pts, 3)
    c_i = add("connectivity", conn, 1)
    o_i = add("offsets", offsets, 1)
    t_i = add("types", types, 1)

    def da(i):
        name, typ, ncomp, off = xml_arrays[i]
        comp = f' NumberOfComponents="{ncomp}"' if ncomp > 1 else ""
        return (f'<DataArray type="{typ}" Name="{name}"{comp} format="appended" '
                f'offset="{off}"/>')

    head = ['<?xml version="1.0"?>',
            '<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" '
            'header_type="UInt64">',
            '<UnstructuredGrid>',
            f'<Piece NumberOfPoints="{npts}" NumberOfCells="{N}">',
            '<Points>', da(p_i), '</Points>',
            '<Cells>', da(c_i), da(o_i), da(t_i), '</Cells>',
            '<CellData>', *[da(i) for i in data_xml], '</CellData>',
            '</Piece>', '</UnstructuredGrid>',
            '<AppendedData encoding="raw">']
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n_").encode("ascii"))
        for arr in blocks:
            f.write(np.uint64(arr.nbytes).tobytes())
            f.write(arr.astype(arr.dtype.newbyteorder("<"), copy=False).tobytes())
        f.write(b"\n</AppendedData>\n</VTKFile>\n")
    return path


def read_vtu(path):
    """Points, connectivity, offsets, types and cell data of a file written by
    ``write_vtu``: a dict of NumPy arrays keyed by DataArray name."""
    raw = open(path, "rb").read()
    start = raw.index(b"<AppendedData")
    mark = raw.index(b"_", start) + 1
    head = raw[:start].decode("ascii") + "</VTKFile>"
    head = re.sub(r"<\?xml[^>]*\?>", "", head)
    root = ET.fromstring(head)
    out = {}
    for el in root.iter("DataArray"):
        off = mark + int(el.get("offset"))
        nbytes = int(np.frombuffer(raw[off:off + 8], dtype="<u8")[0])
        arr = np.frombuffer(raw[off + 8:off + 8 + nbytes], dtype=_NP_TYPES[el.get("type")])
        ncomp = int(el.get("NumberOfComponents", "1"))
        out[el.get("Name")] = arr.reshape(-1, ncomp) if ncomp > 1 else arr
    return out
