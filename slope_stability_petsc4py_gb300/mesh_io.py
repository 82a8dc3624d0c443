"""Gmsh mesh input without meshio: the reference's ``.msh`` loader (``src/slope_stability/io.py``).

* ``read_gmsh`` parses MSH 2.2 files, ASCII and binary (either byte order): points, cells per gmsh
  element type with their physical tags, and the physical names -- what the reference reads through
  ``meshio.read`` (``io.py:401-413``).
* ``elevate_tet4_mesh`` raises a tet4 mesh (and its boundary triangles) to P2 (tet10/tri6) or P4
  (tet35/tri15) with the reference's global numbering and coordinates (``io.py:216-398``): new nodes
  are numbered in order of creation, element by element -- the element's new edges in the order
  (0,1),(1,2),(0,2),(1,3),(2,3),(0,3) (an edge's P4 nodes from its lower to its higher vertex id),
  then (P4) its new face interiors in the order (0,1,2),(0,1,3),(0,2,3),(1,2,3) (laid out on the face's
  sorted vertices), then its centroid; boundary triangles come after the tetrahedra.  The
  creation order is found for the whole mesh at once (first occurrences of sorted keys) instead of
  with per-element dictionaries.
* ``load_mesh_file`` returns the reference's ``MeshData`` (``io.py:17-25, 464-476``) for ``.msh``
  files: material and boundary labels through the ``material_N`` / ``boundary_N`` physical names
  (``io.py:165-189``) and the Dirichlet mask from boundary labels per axis (``io.py:61-93``).

The reference takes the per-axis Dirichlet labels from the mesh family's ``definition.py``; here
they are an argument (default: the reference's defaults, ``io.py:34-40``).
"""

from __future__ import annotations

import re
from dataclasses import dataclass
from pathlib import Path

import numpy as np

# nodes per gmsh element type (MSH 2.2 element type codes)
GMSH_NODES = {1: 2, 2: 3, 3: 4, 4: 4, 5: 8, 6: 6, 7: 5, 8: 3, 9: 6, 10: 9, 11: 10, 12: 27, 13: 18, 14: 14, 15: 1,
              16: 8, 17: 20, 18: 15, 19: 13, 20: 9, 21: 10, 22: 12, 23: 15, 24: 15, 25: 21, 26: 4, 27: 5, 28: 6,
              29: 20, 30: 35, 31: 56}
GMSH_TYPE_NAMES = {1: "line", 2: "triangle", 3: "quad", 4: "tetra", 5: "hexahedron", 6: "wedge", 7: "pyramid",
                   8: "line3", 9: "triangle6", 11: "tetra10", 15: "vertex"}

DEFAULT_DIRICHLET_LABELS = {2: {"x": (1, 2), "y": (3,)}, 3: {"x": (1, 2), "y": (5,), "z": (3, 4)}}


@dataclass
class GmshMesh:
    points: np.ndarray  # (n_points, 3)
    cells: dict  # gmsh type name -> (connectivity (n_cells, k) 0-based int64, physical tags (n_cells,))
    field_data: dict  # physical name -> array([tag, dim])


@dataclass
class MeshData:
    coord: np.ndarray
    elem: np.ndarray
    surf: np.ndarray
    q_mask: np.ndarray
    material: np.ndarray
    boundary: np.ndarray
    elem_type: str | None = None


def _section(data: bytes, name: str, start: int = 0) -> tuple[int, int]:
    """(offset just after the '$name' line, offset of '$Endname') or (-1, -1)."""
    head = data.find(b"$" + name.encode(), start)
    if head < 0:
        return -1, -1
    body = data.index(b"\n", head) + 1
    end = data.find(b"$End" + name.encode(), body)
    if end < 0:
        raise ValueError(f"section ${name} is not closed")
    return body, end


def _next_line(data: bytes, pos: int) -> tuple[bytes, int]:
    nl = data.index(b"\n", pos)
    return data[pos:nl].strip(), nl + 1


def read_gmsh(path) -> GmshMesh:
    """Parse a gmsh MSH 2.2 file (ASCII or binary)."""
    data = Path(path).read_bytes()
    b0, _ = _section(data, "MeshFormat")
    if b0 < 0:
        raise ValueError(f"{path}: no $MeshFormat section")
    fmt, pos = _next_line(data, b0)
    parts = fmt.split()
    version, binary, dsize = parts[0].decode(), int(parts[1]), int(parts[2])
    if not version.startswith("2."):
        raise ValueError(f"{path}: MSH {version} is not supported (save the mesh as MSH 2.2)")
    if binary and dsize != 8:
        raise ValueError(f"{path}: binary MSH with {dsize}-byte reals is not supported")
    order = "<"
    if binary:
        one = np.frombuffer(data, dtype="<i4", count=1, offset=pos)[0]
        if one != 1:
            order = ">"
            if np.frombuffer(data, dtype=">i4", count=1, offset=pos)[0] != 1:
                raise ValueError(f"{path}: bad binary MSH endianness marker")
    i4, f8 = np.dtype(order + "i4"), np.dtype(order + "f8")

    field_data: dict[str, np.ndarray] = {}
    p0, p1 = _section(data, "PhysicalNames")
    if p0 >= 0:
        lines = data[p0:p1].decode().splitlines()
        for line in lines[1 : 1 + int(lines[0])]:
            m = re.match(r"\s*(\d+)\s+(\d+)\s+\"(.*)\"\s*$", line)
            if m is None:
                raise ValueError(f"{path}: bad physical name line {line!r}")
            field_data[m.group(3)] = np.array([int(m.group(2)), int(m.group(1))], dtype=np.int64)

    n0, n1 = _section(data, "Nodes")
    if n0 < 0:
        raise ValueError(f"{path}: no $Nodes section")
    cnt, pos = _next_line(data, n0)
    n_nodes = int(cnt)
    if binary:
        rec = np.dtype([("id", i4), ("xyz", f8, (3,))])
        nodes = np.frombuffer(data, dtype=rec, count=n_nodes, offset=pos)
        node_ids, points = nodes["id"].astype(np.int64), nodes["xyz"].astype(np.float64)
    else:
        arr = np.array(data[pos:n1].split(), dtype=np.float64).reshape(n_nodes, 4) if n_nodes else np.empty((0, 4))
        node_ids, points = arr[:, 0].astype(np.int64), np.ascontiguousarray(arr[:, 1:4])
    if n_nodes and np.array_equal(node_ids, np.arange(1, n_nodes + 1)):
        to_index = None
    else:
        to_index = np.full(int(node_ids.max(initial=0)) + 1, -1, dtype=np.int64)
        to_index[node_ids] = np.arange(n_nodes)

    e0, e1 = _section(data, "Elements")
    if e0 < 0:
        raise ValueError(f"{path}: no $Elements section")
    cnt, pos = _next_line(data, e0)
    n_elem = int(cnt)
    blocks: dict[int, list[tuple[np.ndarray, np.ndarray]]] = {}
    if binary:
        seen = 0
        while seen < n_elem:
            etype, count, ntags = (int(v) for v in np.frombuffer(data, dtype=i4, count=3, offset=pos))
            pos += 12
            if etype not in GMSH_NODES:
                raise ValueError(f"{path}: unknown gmsh element type {etype}")
            width = 1 + ntags + GMSH_NODES[etype]
            block = np.frombuffer(data, dtype=i4, count=count * width, offset=pos).reshape(count, width)
            pos += 4 * count * width
            phys = block[:, 1] if ntags else np.zeros(count, dtype=np.int64)
            blocks.setdefault(etype, []).append((block[:, 1 + ntags :].astype(np.int64), phys.astype(np.int64)))
            seen += count
    else:
        for line in data[pos:e1].decode().splitlines()[:n_elem]:
            v = [int(x) for x in line.split()]
            etype, ntags = v[1], v[2]
            if etype not in GMSH_NODES:
                raise ValueError(f"{path}: unknown gmsh element type {etype}")
            conn = np.asarray(v[3 + ntags : 3 + ntags + GMSH_NODES[etype]], dtype=np.int64)[None, :]
            blocks.setdefault(etype, []).append((conn, np.asarray([v[3] if ntags else 0], dtype=np.int64)))
    cells = {}
    for etype, parts in blocks.items():
        conn = np.concatenate([c for c, _ in parts])
        phys = np.concatenate([p for _, p in parts])
        if to_index is None:
            conn = conn - 1
        else:
            conn = np.where((conn >= 0) & (conn < to_index.size), to_index[np.clip(conn, 0, to_index.size - 1)], -1)
        if (conn < 0).any() or (conn >= n_nodes).any():
            raise ValueError(f"{path}: element refers to a missing node")
        cells[GMSH_TYPE_NAMES.get(etype, f"type{etype}")] = (conn, phys)
    return GmshMesh(points=points, cells=cells, field_data=field_data)


TET_EDGES = ((0, 1), (1, 2), (0, 2), (1, 3), (2, 3), (0, 3))
TET_FACES = ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3))
TRI_EDGES = ((0, 1), (1, 2), (0, 2))
# face-interior nodes of a P4 triangle: barycentric counts on the face's sorted vertices, in order
P4_FACE_COUNTS = ((2, 1, 1), (1, 2, 1), (1, 1, 2))
_EDGE, _FACE, _CENTROID = 0, 1, 2


def elevate_tet4_mesh(coord, tet4, tri3, order: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Raise tet4 (4, n_t) and boundary tri3 (3, n_s) to order 2 (tet10, tri6) or 4 (tet35, tri15).
    Returns (coord, elem, surf) with the reference loader's numbering and coordinates."""
    coord = np.asarray(coord, dtype=np.float64)
    tet4 = np.asarray(tet4, dtype=np.int64)
    tri3 = np.asarray(tri3, dtype=np.int64).reshape(3, -1)
    if order not in (2, 4):
        raise ValueError("elevation order must be 2 or 4")
    if tet4.shape[0] != 4:
        raise ValueError(f"elevation expects 4-node tetrahedra, got shape {tet4.shape}")
    n_v, n_t, n_s = coord.shape[1], tet4.shape[1], tri3.shape[1]
    p4 = order == 4
    # the entities in creation order: per tet its edges (+ faces, centroid), then per triangle its
    # edges (+ face); key = (kind, sorted vertex ids | tet index)
    per_tet, per_tri = [], []
    for i, j in TET_EDGES:
        a, b = tet4[i], tet4[j]
        per_tet.append(np.stack((np.full(n_t, _EDGE), np.minimum(a, b), np.maximum(a, b), np.full(n_t, -1)), axis=1))
    if p4:
        for f in TET_FACES:
            s = np.sort(tet4[list(f)], axis=0)
            per_tet.append(np.stack((np.full(n_t, _FACE), s[0], s[1], s[2]), axis=1))
        per_tet.append(np.stack((np.full(n_t, _CENTROID), np.arange(n_t), np.full(n_t, -1), np.full(n_t, -1)), axis=1))
    for i, j in TRI_EDGES:
        a, b = tri3[i], tri3[j]
        per_tri.append(np.stack((np.full(n_s, _EDGE), np.minimum(a, b), np.maximum(a, b), np.full(n_s, -1)), axis=1))
    if p4:
        s = np.sort(tri3, axis=0)
        per_tri.append(np.stack((np.full(n_s, _FACE), s[0], s[1], s[2]), axis=1))
    k_tet, k_tri = len(per_tet), len(per_tri)
    seq = np.concatenate((np.stack(per_tet, axis=1).reshape(-1, 4), np.stack(per_tri, axis=1).reshape(-1, 4)))
    if seq.shape[0] == 0:
        return coord.copy(), np.empty((10 if not p4 else 35, 0), np.int64), np.empty((6 if not p4 else 15, 0), np.int64)
    uniq, first, inv = np.unique(seq, axis=0, return_index=True, return_inverse=True)
    inv = inv.reshape(-1)
    created = np.argsort(first, kind="stable")  # unique entities in creation order
    sizes = np.where(uniq[created, 0] == _EDGE, order - 1, np.where(uniq[created, 0] == _FACE, 3, 1))
    base_created = n_v + np.concatenate(([0], np.cumsum(sizes)[:-1]))
    base_u = np.empty(uniq.shape[0], dtype=np.int64)
    base_u[created] = base_created
    base = base_u[inv]
    base_tet = base[: n_t * k_tet].reshape(n_t, k_tet)
    base_tri = base[n_t * k_tet :].reshape(n_s, k_tri)

    # coordinates of the new nodes, in creation order
    ent = uniq[created]
    new = np.empty((coord.shape[0], int(sizes.sum())), dtype=np.float64)
    off = base_created - n_v
    edge = ent[:, 0] == _EDGE
    lo, hi = ent[edge, 1], ent[edge, 2]
    if not p4:
        new[:, off[edge]] = 0.5 * (coord[:, lo] + coord[:, hi])
    else:
        for step in range(1, order):
            alpha, beta = float(order - step) / float(order), float(step) / float(order)
            new[:, off[edge] + step - 1] = alpha * coord[:, lo] + beta * coord[:, hi]
        face = ent[:, 0] == _FACE
        fv = ent[face, 1:4]
        for k, counts in enumerate(P4_FACE_COUNTS):
            point = np.zeros((coord.shape[0], fv.shape[0]))
            for c, col in zip(counts, range(3)):
                point += (float(c) / float(order)) * coord[:, fv[:, col]]
            new[:, off[face] + k] = point
        cen = ent[:, 0] == _CENTROID
        t = tet4[:, ent[cen, 1]]
        new[:, off[cen]] = 0.25 * (coord[:, t[0]] + coord[:, t[1]] + coord[:, t[2]] + coord[:, t[3]])
    coord_out = np.concatenate((coord, new), axis=1)

    if not p4:
        elem = np.concatenate((tet4, base_tet.T))
        surf = np.concatenate((tri3, base_tri.T))
        return coord_out, elem, surf

    def edge_nodes(verts, i, j, b):
        # an edge's nodes from vertex i to vertex j (stored from the lower id to the higher)
        fwd = (verts[i] < verts[j])[None, :]
        steps = np.arange(order - 1)[:, None]
        return np.where(fwd, b[None, :] + steps, b[None, :] + (order - 2 - steps))

    def face_nodes(verts, f, b):
        # local interior node k sits nearest local vertex f[k]: its id is the rank of that vertex
        # among the face's sorted vertices
        v = verts[list(f)]
        rank = np.argsort(np.argsort(v, axis=0, kind="stable"), axis=0, kind="stable")
        return b[None, :] + rank

    elem = np.empty((35, n_t), dtype=np.int64)
    elem[:4] = tet4
    row = 4
    for k, (i, j) in enumerate(TET_EDGES):
        elem[row : row + 3] = edge_nodes(tet4, i, j, base_tet[:, k])
        row += 3
    for k, f in enumerate(TET_FACES):
        elem[row : row + 3] = face_nodes(tet4, f, base_tet[:, len(TET_EDGES) + k])
        row += 3
    elem[34] = base_tet[:, -1]
    surf = np.empty((15, n_s), dtype=np.int64)
    surf[:3] = tri3
    row = 3
    for k, (i, j) in enumerate(TRI_EDGES):
        surf[row : row + 3] = edge_nodes(tri3, i, j, base_tri[:, k])
        row += 3
    surf[12:15] = face_nodes(tri3, (0, 1, 2), base_tri[:, 3])
    return coord_out, elem, surf


def _physical_map(field_data: dict, dim: int, prefix: str) -> dict[int, int]:
    pattern = re.compile(rf"^{re.escape(prefix)}_(\d+)$")
    out = {}
    for name, meta in field_data.items():
        arr = np.asarray(meta, dtype=np.int64).ravel()
        if arr.size < 2 or int(arr[1]) != dim:
            continue
        m = pattern.match(str(name).strip().lower())
        if m is not None:
            out[int(arr[0])] = int(m.group(1))
    return out


def map_physical_ids(ids, field_data: dict, dim: int, prefix: str) -> np.ndarray:
    """Physical tags -> the N of their ``<prefix>_N`` names (unchanged when no name matches)."""
    ids = np.asarray(ids, dtype=np.int64).ravel()
    mapping = _physical_map(field_data, dim, prefix)
    if not mapping:
        return ids
    missing = sorted(int(v) for v in np.unique(ids) if int(v) not in mapping)
    if missing:
        raise ValueError(f"Physical group mapping for prefix {prefix!r} is incomplete; missing logical ids for "
                         f"physical tags {missing}.")
    return np.asarray([mapping[int(v)] for v in ids], dtype=np.int64)


def dirichlet_mask(dim: int, n_nodes: int, surf, boundary, *, dirichlet_labels=None, boundary_type: int = 0):
    """q_mask (dim, n_nodes): False on every node of a boundary face whose label constrains that
    axis; with boundary_type, the 'y' labels (the bottom of the 3D slope families) fix every axis."""
    labels = DEFAULT_DIRICHLET_LABELS[int(dim)] if dirichlet_labels is None else dirichlet_labels
    face = np.asarray(surf, dtype=np.int64)
    lab = np.asarray(boundary, dtype=np.int64).ravel()
    q = np.ones((int(dim), int(n_nodes)), dtype=bool)
    for axis, name in enumerate(("x", "y", "z")[:dim]):
        fixed = tuple(int(v) for v in labels.get(name, ()))
        if fixed and face.size:
            sel = np.isin(lab, np.asarray(fixed, dtype=np.int64))
            q[axis, face[:, sel].ravel()] = False
    if int(dim) == 3 and int(boundary_type) and face.size:
        glued = tuple(int(v) for v in labels.get("y", ()))
        if glued:
            sel = np.isin(lab, np.asarray(glued, dtype=np.int64))
            q[:, face[:, sel].ravel()] = False
    return q


def load_mesh_file(mesh_file, *, elem_type: str | None = None, boundary_type: int = 0,
                   dirichlet_labels=None) -> MeshData:
    """A gmsh tet4 mesh with physical groups as ``MeshData``, elevated to ``elem_type`` (P1, P2, P4)."""
    path = Path(mesh_file)
    if path.suffix.lower() != ".msh":
        raise ValueError(f"Unsupported mesh format for {path} (gmsh .msh files are read here)")
    msh = read_gmsh(path)
    if msh.points.ndim != 2 or msh.points.shape[1] < 3:
        raise ValueError(f"Expected 3D point coordinates in {path}, got shape {msh.points.shape}.")
    if "tetra" not in msh.cells:
        raise ValueError(f"No tetrahedral cells found in {path}.")
    tets, tet_tags = msh.cells["tetra"]
    tris, tri_tags = msh.cells.get("triangle", (np.empty((0, 3), np.int64), np.empty(0, np.int64)))
    coord = np.ascontiguousarray(msh.points[:, :3].T)
    material = map_physical_ids(tet_tags, msh.field_data, 3, "material")
    boundary = map_physical_ids(tri_tags, msh.field_data, 2, "boundary")
    elem, surf = np.ascontiguousarray(tets.T), np.ascontiguousarray(tris.T)
    target = None if elem_type is None else str(elem_type).strip().upper()
    if target in (None, "", "P1"):
        et = "P1"
    elif target in ("P2", "P4"):
        et = target
        coord, elem, surf = elevate_tet4_mesh(coord, elem, surf, 2 if target == "P2" else 4)
    else:
        raise NotImplementedError(f"Gmsh simplex loader supports P1 source meshes elevated to P2/P4; requested {target!r}.")
    q = dirichlet_mask(3, coord.shape[1], surf, boundary, dirichlet_labels=dirichlet_labels, boundary_type=boundary_type)
    return MeshData(coord=coord, elem=elem, surf=surf, q_mask=q, material=material, boundary=boundary, elem_type=et)
