"""Mesh file ingestion: ``Mesh(filename)`` of src/MFEM/MUtils.jl:33-50.

The reference reads ``.mat`` files with MAT.jl (``nodes``, ``elems`` variables, 1-based
elements) and every other format with the Python package meshio, then keeps the first
cell block (which must hold triangles) and the x, y columns of the points.  meshio is
not a dependency here; this module reads the formats AdFem's own mesh data uses
(deps/MFEM/MeshData: STL, Gmsh .msh, legacy VTK, MATLAB .mat):

  * ``.mat``   scipy.io.loadmat (MATLAB v5/v7 files), variables ``nodes`` (n x 2) and
               ``elems`` (m x 3, 1-based);
  * ``.stl``   ASCII or binary; the facets' corner points are merged into unique points
               in the order of their first appearance (meshio's STL reader does the same);
  * ``.msh``   Gmsh ASCII format 2.2 or 4.1; node tags are renumbered in the order the
               nodes are listed; the triangles (element type 2) of the first element block
               that has any;
  * ``.vtk``   legacy ASCII unstructured grid (POINTS, CELLS, CELL_TYPES); the cells of type
               5 (triangle) of the first run of triangles.
Binary VTK/Gmsh files and MATLAB v7.3 (HDF5) files raise MeshFileError.

``read_mesh_file`` returns ``(coords (n, 2) float64, elems (m, 3) int64 1-based)``.
"""
from __future__ import annotations

import os
import struct

import numpy as np


class MeshFileError(ValueError):
    pass


def _unique_first(points):
    """Unique rows in order of first appearance, and the index of each input row."""
    _, idx, inv = np.unique(points, axis=0, return_index=True, return_inverse=True)
    order = np.argsort(idx)
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    return points[idx[order]], rank[inv.ravel()]


def _read_stl(path):
    with open(path, "rb") as f:
        data = f.read()
    facets = None
    if len(data) >= 84:
        n = struct.unpack("<I", data[80:84])[0]
        if 84 + 50 * n == len(data):
            rec = np.frombuffer(data, dtype=np.dtype([("normal", "<f4", 3), ("v", "<f4", (3, 3)), ("attr", "<u2")]),
                                count=n, offset=84)
            facets = rec["v"].astype(np.float64)
    if facets is None:
        try:
            text = data.decode("ascii")
        except UnicodeDecodeError as e:
            raise MeshFileError("%s: neither binary nor ASCII STL" % path) from e
        verts = [line.split()[1:4] for line in text.splitlines() if line.strip().startswith("vertex")]
        if len(verts) % 3:
            raise MeshFileError("%s: ASCII STL with a facet that is not a triangle" % path)
        facets = np.array(verts, dtype=np.float64).reshape(-1, 3, 3)
    pts, inv = _unique_first(facets.reshape(-1, 3))
    return pts, inv.reshape(-1, 3)


def _sections(lines, name):
    out = []
    for i, line in enumerate(lines):
        if line.strip() == "$" + name:
            j = i + 1
            while lines[j].strip() != "$End" + name:
                j += 1
            out.append(lines[i + 1:j])
    return out


def _read_msh(path):
    with open(path) as f:
        lines = f.read().splitlines()
    fmt = _sections(lines, "MeshFormat")
    if not fmt:
        raise MeshFileError("%s: no $MeshFormat section (binary or unknown Gmsh file)" % path)
    version, ftype = fmt[0][0].split()[:2]
    if ftype != "0":
        raise MeshFileError("%s: binary Gmsh files are not supported" % path)
    nodes = _sections(lines, "Nodes")[0]
    elems = _sections(lines, "Elements")[0]
    tags, xyz = [], []
    blocks = []  # per element block: list of triangles (node tags)
    if version.startswith("2"):
        n = int(nodes[0])
        for line in nodes[1:1 + n]:
            t = line.split()
            tags.append(int(t[0]))
            xyz.append([float(v) for v in t[1:4]])
        cur_type, cur = None, None
        for line in elems[1:1 + int(elems[0])]:
            t = [int(v) for v in line.split()]
            etype, ntag = t[1], t[2]
            if etype != cur_type:
                cur_type, cur = etype, []
                blocks.append((etype, cur))
            cur.append(t[3 + ntag:])
    elif version.startswith("4"):
        nb = int(nodes[0].split()[0])
        k = 1
        for _ in range(nb):
            nn = int(nodes[k].split()[3])
            tags.extend(int(v) for v in nodes[k + 1:k + 1 + nn])
            xyz.extend([float(v) for v in line.split()[:3]] for line in nodes[k + 1 + nn:k + 1 + 2 * nn])
            k += 1 + 2 * nn
        nb = int(elems[0].split()[0])
        k = 1
        for _ in range(nb):
            _, _, etype, ne = (int(v) for v in elems[k].split()[:4])
            blocks.append((etype, [[int(v) for v in line.split()[1:]] for line in elems[k + 1:k + 1 + ne]]))
            k += 1 + ne
    else:
        raise MeshFileError("%s: Gmsh format %s is not supported (2.2 and 4.1 are)" % (path, version))
    tri = next((b for t, b in blocks if t == 2 and b), None)
    if tri is None:
        raise MeshFileError("No triangles found in the mesh file.")
    pos = {t: i for i, t in enumerate(tags)}
    el = np.array([[pos[v] for v in row[:3]] for row in tri], dtype=np.int64)
    return np.array(xyz, dtype=np.float64), el


def _read_vtk(path):
    with open(path, "rb") as f:
        head = f.read(512).split(b"\n")[:4]
        if any(h.strip().upper() == b"BINARY" for h in head):
            raise MeshFileError("%s: binary VTK files are not supported (legacy ASCII is)" % path)
        f.seek(0)
        tok = f.read().decode("ascii", errors="replace").split()
    up = [t.upper() for t in tok]
    i = up.index("POINTS")
    n = int(tok[i + 1])
    pts = np.array(tok[i + 3:i + 3 + 3 * n], dtype=np.float64).reshape(n, 3)
    i = up.index("CELLS")
    nc, size = int(tok[i + 1]), int(tok[i + 2])
    conn = np.array(tok[i + 3:i + 3 + size], dtype=np.int64)
    i = up.index("CELL_TYPES")
    types = np.array(tok[i + 2:i + 2 + nc], dtype=np.int64)
    cells, k = [], 0
    for c in range(nc):
        m = conn[k]
        cells.append(conn[k + 1:k + 1 + m])
        k += 1 + m
    start = next((c for c in range(nc) if types[c] == 5), None)
    if start is None:
        raise MeshFileError("No triangles found in the mesh file.")
    stop = start
    while stop < nc and types[stop] == 5:
        stop += 1
    return pts, np.array(cells[start:stop], dtype=np.int64)


def read_mesh_file(path, file_format: str | None = None):
    """(coords (n, 2), elems (m, 3) 1-based) of a mesh file (src/MFEM/MUtils.jl:33-50)."""
    ext = (file_format or os.path.splitext(path)[1].lstrip(".")).lower()
    if ext == "mat":
        from scipy.io import loadmat

        try:
            d = loadmat(path)
        except NotImplementedError as e:  # MATLAB v7.3 files are HDF5 containers
            raise MeshFileError("%s: MATLAB v7.3 (HDF5) files are not supported; save with -v7" % path) from e
        return np.asarray(d["nodes"], dtype=np.float64)[:, :2].copy(), np.asarray(d["elems"], dtype=np.int64)
    readers = {"stl": _read_stl, "msh": _read_msh, "gmsh": _read_msh, "vtk": _read_vtk}
    if ext not in readers:
        raise MeshFileError("%s: unsupported mesh format %r (mat, stl, msh, vtk are)" % (path, ext))
    pts, el = readers[ext](path)
    if el.size == 0:
        raise MeshFileError("No triangles found in the mesh file.")
    return np.ascontiguousarray(pts[:, :2]), el + 1
