"""Gmsh input (no GPU): MSH 2.2 parsing (ASCII, binary, both byte orders), tet4 -> tet10 / tet35
elevation and Dirichlet masks bit for bit against the reference's loader (fixture ``mesh_io.npz``),
and the elevated meshes through the host pattern builder."""

from __future__ import annotations

import os
import struct
from pathlib import Path

import numpy as np
import pytest

from conftest import golden

# a reference checkout named by SSP_REFERENCE_ROOT (the tests that read its mesh skip without one)
_REF = os.environ.get("SSP_REFERENCE_ROOT")
REF_MESH = Path(_REF) / "meshes/3d_hetero_ssr/SSR_hetero_ada_L1.msh" if _REF else Path("/nonexistent")


def _write_msh(path, coord, tet, tri, tet_tags, tri_tags, names, *, binary, big_endian=False, id_offset=0):
    """A minimal MSH 2.2 writer (node ids 1 + id_offset + index)."""
    n = coord.shape[1]
    ids = np.arange(n) + 1 + id_offset
    head = "$MeshFormat\n2.2 {} 8\n".format(1 if binary else 0)
    phys = "$PhysicalNames\n{}\n".format(len(names)) + "".join(f'{d} {t} "{nm}"\n' for nm, (t, d) in names.items())
    phys += "$EndPhysicalNames\n"
    e = "<" if not big_endian else ">"
    with open(path, "wb") as f:
        f.write(head.encode())
        if binary:
            f.write(struct.pack(e + "i", 1) + b"\n")
        f.write(b"$EndMeshFormat\n" + phys.encode() + f"$Nodes\n{n}\n".encode())
        if binary:
            for k in range(n):
                f.write(struct.pack(e + "iddd", int(ids[k]), *coord[:, k]))
            f.write(b"\n")
        else:
            for k in range(n):
                f.write(("%d %.17g %.17g %.17g\n" % (ids[k], *coord[:, k])).encode())
        n_el = tri.shape[1] + tet.shape[1] + 1
        f.write(f"$EndNodes\n$Elements\n{n_el}\n".encode())
        num = 1
        blocks = [(15, np.array([[0]]), np.array([0])), (2, tri, tri_tags), (4, tet, tet_tags)]
        for etype, conn, tags in blocks:
            if binary:
                f.write(struct.pack(e + "iii", etype, conn.shape[1], 2))
            for k in range(conn.shape[1]):
                nodes = ids[conn[:, k]]
                if binary:
                    f.write(struct.pack(e + "i" * (3 + conn.shape[0]), num, int(tags[k]), 1, *map(int, nodes)))
                else:
                    f.write((f"{num} {etype} 2 {int(tags[k])} 1 " + " ".join(map(str, nodes)) + "\n").encode())
                num += 1
        f.write(b"\n$EndElements\n" if binary else b"$EndElements\n")


@pytest.fixture(scope="module")
def g():
    return golden("mesh_io.npz")


@pytest.mark.parametrize("binary,big_endian,id_offset", [(False, False, 0), (True, False, 0), (True, True, 0),
                                                          (False, False, 100), (True, False, 7)])
def test_read_gmsh_round_trip(tmp_path, g, binary, big_endian, id_offset):
    from slope_stability_petsc4py_gb300 import mesh_io

    # physical tag 10 + N is named "boundary_N", tag 21 + N "material_N"
    names = {**{f"boundary_{k}": (10 + k, 2) for k in range(1, 7)}, **{f"material_{k}": (21 + k, 3) for k in range(3)}}
    tri_tags = g["boundary"] + 10
    tet_tags = g["material"] + 21
    p = tmp_path / "m.msh"
    _write_msh(p, g["coord"], g["tet4"], g["tri3"], tet_tags, tri_tags, names, binary=binary, big_endian=big_endian,
               id_offset=id_offset)
    m = mesh_io.read_gmsh(p)
    assert np.array_equal(m.points.T, g["coord"])
    conn, tags = m.cells["tetra"]
    assert np.array_equal(conn.T, g["tet4"]) and np.array_equal(tags, tet_tags)
    conn, tags = m.cells["triangle"]
    assert np.array_equal(conn.T, g["tri3"]) and np.array_equal(tags, tri_tags)
    assert m.cells["vertex"][0].shape == (1, 1)
    data = mesh_io.load_mesh_file(p, elem_type="P2")
    assert np.array_equal(data.material, g["material"])
    assert np.array_equal(data.boundary, g["boundary"])
    assert np.array_equal(data.q_mask, g["q_mask_p2_bt0"])
    assert np.array_equal(data.coord, g["coord_p2"]) and np.array_equal(data.elem, g["elem_p2"])


@pytest.mark.parametrize("order", [2, 4])
def test_elevation_bit_exact_with_reference(g, order):
    from slope_stability_petsc4py_gb300 import mesh_io

    c, e, s = mesh_io.elevate_tet4_mesh(g["coord"], g["tet4"], g["tri3"], order)
    assert np.array_equal(e, g[f"elem_p{order}"]) and np.array_equal(s, g[f"surf_p{order}"])
    assert c.shape == g[f"coord_p{order}"].shape
    assert np.array_equal(c.view(np.uint64), g[f"coord_p{order}"].view(np.uint64))  # bitwise
    for bt in (0, 1):
        q = mesh_io.dirichlet_mask(3, c.shape[1], s, g["boundary"], boundary_type=bt)
        assert np.array_equal(q, g[f"q_mask_p{order}_bt{bt}"])


def test_elevated_node_order_matches_the_basis(g):
    """Local node k of an elevated tet sits at the barycentric point tet_node_tuples(p)[k] / p."""
    from slope_stability_petsc4py_gb300 import mesh_io, synthetic

    for order in (2, 4):
        c, e, _ = mesh_io.elevate_tet4_mesh(g["coord"], g["tet4"], g["tri3"], order)
        tup = np.asarray(synthetic.tet_node_tuples(order), dtype=np.float64) / order
        X = c[:, e]
        assert np.max(np.abs(np.einsum("dve,kv->dke", X[:, :4], tup) - X)) <= 1e-12 * np.abs(c).max()


def test_physical_names_and_p1_mask(g):
    from slope_stability_petsc4py_gb300 import mesh_io

    field = {"boundary_0": np.array([11, 2]), "boundary_1": np.array([12, 2]), "material_0": np.array([7, 3]),
             "material_1": np.array([8, 3]), "other": np.array([9, 3])}
    assert np.array_equal(mesh_io.map_physical_ids(g["physical_tags"], field, 2, "boundary"), g["physical_mapped"])
    with pytest.raises(ValueError):
        mesh_io.map_physical_ids(np.array([11, 99]), field, 2, "boundary")
    assert np.array_equal(mesh_io.map_physical_ids(np.array([5, 6]), {}, 2, "boundary"), [5, 6])
    q = mesh_io.dirichlet_mask(3, g["coord"].shape[1], g["tri3"], g["boundary"])
    assert np.array_equal(q, g["q_mask_p1_bt0"])


def test_elevated_mesh_through_the_pattern_builder(g):
    """An elevated file mesh gives a valid owned pattern (host builder): every element's map entries
    land on its own rows, and the constrained rows hold their diagonal only."""
    from slope_stability_petsc4py_gb300 import mesh_io
    from slope_stability_petsc4py_gb300.distributed_tangent import _PatternBuild

    c, e, s = mesh_io.elevate_tet4_mesh(g["coord"], g["tet4"], g["tri3"], 4)
    q = mesh_io.dirichlet_mask(3, c.shape[1], s, g["boundary"])
    pb = _PatternBuild(e, q, (0, c.shape[1]))
    indptr, indices, cdiag = pb.get("indptr"), pb.get("indices"), pb.get("constrained_diag_positions")
    pb.close()
    fixed = np.flatnonzero(~q.reshape(-1, order="F"))
    assert np.array_equal(np.diff(indptr)[fixed], np.ones(fixed.size)) and np.array_equal(indices[cdiag], fixed)


@pytest.mark.skipif(not REF_MESH.exists(), reason="the reference checkout with its meshes is not mounted")
def test_reads_a_reference_mesh_file():
    """The reference's binary MSH 2.2 mesh (18,419 tets): counts, labels, elevation consistency."""
    from slope_stability_petsc4py_gb300 import mesh_io

    m = mesh_io.load_mesh_file(REF_MESH, elem_type="P2")
    assert m.elem.shape == (10, 18419) and m.coord.shape[0] == 3
    assert set(np.unique(m.material)) == {0, 1, 2, 3} and set(np.unique(m.boundary)) <= set(range(7))
    assert (~m.q_mask).any(axis=1).all()
    X = m.coord[:, m.elem]
    mid = 0.5 * (X[:, 0] + X[:, 1])
    assert np.max(np.abs(mid - X[:, 4])) <= 1e-12 * np.abs(m.coord).max()
