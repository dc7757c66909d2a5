"""Mesh file ingestion (Mesh(filename), src/MFEM/MUtils.jl:33-50) on CPU: files written
here in every supported format for one small triangulation read back to the same
coordinates and 1-based elements (STL: points in order of first appearance)."""
import struct

import numpy as np
import pytest

from adfem_gpu import synth
from adfem_gpu.meshfile import MeshFileError, read_mesh_file


def small():
    coords, elems = synth.jittered_square(3, seed=1)
    return coords, elems


def first_appearance(coords, elems):
    order, seen = [], {}
    for v in elems.ravel() - 1:
        if v not in seen:
            seen[v] = len(order)
            order.append(v)
    ren = np.array([seen[v] for v in elems.ravel() - 1]).reshape(-1, 3) + 1
    return coords[order], ren


def test_stl_ascii_and_binary(tmp_path):
    coords, elems = small()
    tri = np.concatenate([coords, np.zeros((coords.shape[0], 1))], 1)[elems - 1]
    a = tmp_path / "m_ascii.stl"
    with open(a, "w") as f:
        f.write("solid m\n")
        for t in tri:
            f.write("facet normal 0 0 1\n outer loop\n")
            for v in t:
                f.write("  vertex %.17g %.17g %.17g\n" % tuple(v))
            f.write(" endloop\nendfacet\n")
        f.write("endsolid m\n")
    want_c, want_e = first_appearance(coords, elems)
    c, e = read_mesh_file(str(a))
    np.testing.assert_array_equal(c, want_c)
    np.testing.assert_array_equal(e, want_e)
    b = tmp_path / "m_bin.stl"
    with open(b, "wb") as f:
        f.write(b"\0" * 80 + struct.pack("<I", len(tri)))
        for t in tri:
            f.write(struct.pack("<3f", 0, 0, 1) + t.astype("<f4").tobytes() + b"\0\0")
    c, e = read_mesh_file(str(b))
    np.testing.assert_array_equal(c, want_c.astype(np.float32).astype(np.float64))
    np.testing.assert_array_equal(e, want_e)


@pytest.mark.parametrize("version", ["2.2", "4.1"])
def test_gmsh_ascii(tmp_path, version):
    coords, elems = small()
    n, m = coords.shape[0], elems.shape[0]
    tags = 10 + 3 * np.arange(n)  # non-contiguous node tags
    p = tmp_path / ("m%s.msh" % version)
    with open(p, "w") as f:
        f.write("$MeshFormat\n%s 0 8\n$EndMeshFormat\n" % version)
        if version == "2.2":
            f.write("$Nodes\n%d\n" % n)
            for t, (x, y) in zip(tags, coords):
                f.write("%d %.17g %.17g 0\n" % (t, x, y))
            f.write("$EndNodes\n$Elements\n%d\n" % (m + 2))
            f.write("1 1 2 0 1 %d %d\n" % (tags[0], tags[1]))  # a boundary line first
            f.write("2 15 2 0 1 %d\n" % tags[2])
            for k, el in enumerate(elems):
                f.write("%d 2 2 0 1 %d %d %d\n" % ((k + 3,) + tuple(tags[el - 1])))
            f.write("$EndElements\n")
        else:
            f.write("$Nodes\n1 %d %d %d\n2 1 0 %d\n" % (n, tags.min(), tags.max(), n))
            f.write("".join("%d\n" % t for t in tags))
            f.write("".join("%.17g %.17g 0\n" % (x, y) for x, y in coords))
            f.write("$EndNodes\n$Elements\n2 %d 1 %d\n" % (m + 1, m + 1))
            f.write("1 1 1 1\n1 %d %d\n" % (tags[0], tags[1]))
            f.write("2 1 2 %d\n" % m)
            for k, el in enumerate(elems):
                f.write("%d %d %d %d\n" % ((k + 2,) + tuple(tags[el - 1])))
            f.write("$EndElements\n")
    c, e = read_mesh_file(str(p))
    np.testing.assert_array_equal(c, coords)
    np.testing.assert_array_equal(e, elems)


def test_vtk_ascii_and_mat(tmp_path):
    coords, elems = small()
    n, m = coords.shape[0], elems.shape[0]
    p = tmp_path / "m.vtk"
    with open(p, "w") as f:
        f.write("# vtk DataFile Version 4.2\nmesh\nASCII\nDATASET UNSTRUCTURED_GRID\n")
        f.write("POINTS %d double\n" % n)
        f.write("".join("%.17g %.17g 0\n" % (x, y) for x, y in coords))
        f.write("CELLS %d %d\n" % (m + 1, 4 * m + 2))
        f.write("1 0\n")  # a vertex cell first
        f.write("".join("3 %d %d %d\n" % tuple(el - 1) for el in elems))
        f.write("CELL_TYPES %d\n1\n" % (m + 1) + "5\n" * m)
    c, e = read_mesh_file(str(p))
    np.testing.assert_array_equal(c, coords)
    np.testing.assert_array_equal(e, elems)
    from scipy.io import savemat

    q = tmp_path / "m.mat"
    savemat(str(q), {"nodes": coords, "elems": elems.astype(np.float64)})
    c, e = read_mesh_file(str(q))
    np.testing.assert_array_equal(c, coords)
    np.testing.assert_array_equal(e, elems)


def test_errors(tmp_path):
    p = tmp_path / "x.obj"
    p.write_text("v 0 0 0\n")
    with pytest.raises(MeshFileError):
        read_mesh_file(str(p))
    q = tmp_path / "lines.msh"
    q.write_text("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n2\n1 0 0 0\n2 1 0 0\n$EndNodes\n"
                 "$Elements\n1\n1 1 2 0 1 1 2\n$EndElements\n")
    with pytest.raises(MeshFileError, match="No triangles"):
        read_mesh_file(str(q))
