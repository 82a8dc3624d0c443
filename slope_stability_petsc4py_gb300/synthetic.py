"""Seeded synthetic slope problems with the shapes of the reference's benchmark cases.

The reference runs its SSR benchmarks on gmsh meshes of a 2:1 slope (height 10 m, toe and
crest benches 15 m, 10 m of foundation below the toe).  Those meshes are not part of this
package, so the workloads here are structured stand-ins with the same geometry:

* 2D: a structured quad grid mapped onto the slope profile, each quad split into two
  triangles, elevated to 6-node P2 triangles (node order of
  ``src/slope_stability/fem/basis.py:21-56``: vertices, then edges (1,2), (0,2), (0,1)) or
  15-node P4 triangles (node order of ``src/slope_stability/mesh/textmesh_2d.py:116-184``).
* 3D: the same profile extruded ``depth`` metres in z, each hexahedral cell split into six
  tetrahedra along its main diagonal (a conforming Freudenthal split), elevated to P2
  (edge order of ``src/slope_stability/core/simplex_lagrange.py:11``) or P4 (node tuples of
  ``simplex_lagrange.py:50-83``).

A gmsh tet4 file (the reference's own slope meshes, for instance) becomes a workload through
``register_mesh_file`` (read and elevated by ``mesh_io``).

Displacements are a gravity-loaded, elastic-like settlement field plus a ``tanh`` shear
band of width ``band_width`` along a 30 degree plane through the toe, with an amplitude
chosen by the caller (``calibrate_amplitude`` picks one for a target yield fraction).
"""

from __future__ import annotations

from dataclasses import dataclass, field
from functools import lru_cache
from itertools import permutations
from pathlib import Path

import numpy as np

X1, X2, X3 = 15.0, 20.0, 15.0  # toe bench, slope run (2:1 for 10 m rise), crest bench
Y1, Y2 = 10.0, 10.0  # foundation thickness below the toe, slope height
TOE = np.array([X1, Y1])


@dataclass
class MaterialSet:
    """Per-material Mohr-Coulomb and elastic constants (angles in degrees, moduli in kPa)."""

    c0: np.ndarray
    phi: np.ndarray
    psi: np.ndarray
    young: np.ndarray
    poisson: np.ndarray
    gamma: np.ndarray

    @classmethod
    def homogeneous(cls, c0=6.0, phi=45.0, psi=0.0, young=2.0e4, poisson=0.49, gamma=20.0):
        arr = lambda v: np.array([float(v)], dtype=np.float64)  # noqa: E731
        return cls(arr(c0), arr(phi), arr(psi), arr(young), arr(poisson), arr(gamma))

    @classmethod
    def layered(cls, n_layers: int = 4, seed: int = 0):
        rng = np.random.default_rng(seed)
        return cls(
            c0=rng.uniform(5.0, 15.0, n_layers),
            phi=rng.uniform(25.0, 40.0, n_layers),
            psi=np.zeros(n_layers),
            young=rng.uniform(1.0e4, 6.0e4, n_layers),
            poisson=rng.uniform(0.30, 0.45, n_layers),
            gamma=np.full(n_layers, 20.0),
        )

    @property
    def shear(self):
        return self.young / (2.0 * (1.0 + self.poisson))

    @property
    def bulk(self):
        return self.young / (3.0 * (1.0 - 2.0 * self.poisson))

    @property
    def lame(self):
        return self.bulk - 2.0 * self.shear / 3.0


@dataclass
class SlopeMesh:
    dim: int
    elem_type: str
    coord: np.ndarray  # (dim, n_nodes)
    elem: np.ndarray  # (n_p, n_elem) int64
    q_mask: np.ndarray  # (dim, n_nodes) bool, True = free dof
    material_id: np.ndarray  # (n_elem,) int64
    extra: dict = field(default_factory=dict)

    @property
    def n_nodes(self) -> int:
        return int(self.coord.shape[1])

    @property
    def n_elem(self) -> int:
        return int(self.elem.shape[1])


def surface_height(x: np.ndarray) -> np.ndarray:
    x = np.asarray(x, dtype=np.float64)
    return np.where(x <= X1, Y1, np.where(x >= X1 + X2, Y1 + Y2, Y1 + (x - X1) * (Y2 / X2)))


def _grid_x(nx: int) -> np.ndarray:
    # split the columns between benches and slope proportionally, with a node at both kinks
    n1 = max(1, int(round(nx * X1 / (X1 + X2 + X3))))
    n3 = max(1, int(round(nx * X3 / (X1 + X2 + X3))))
    n2 = max(1, nx - n1 - n3)
    return np.concatenate(
        (
            np.linspace(0.0, X1, n1 + 1),
            np.linspace(X1, X1 + X2, n2 + 1)[1:],
            np.linspace(X1 + X2, X1 + X2 + X3, n3 + 1)[1:],
        )
    )


def _vertex_grid_2d(nx: int, ny: int) -> np.ndarray:
    xs = _grid_x(nx)
    frac = np.linspace(0.0, 1.0, ny + 1)
    X = np.repeat(xs[:, None], ny + 1, axis=1)
    Y = frac[None, :] * surface_height(xs)[:, None]
    return np.stack((X, Y))  # (2, nx+1, ny+1)


@lru_cache(maxsize=None)
def tet_node_tuples(order: int) -> tuple[tuple[int, int, int, int], ...]:
    """Barycentric count tuples of the order-p tetrahedron, in the reference's node order.

    Vertices, then edges in the order (0,1),(1,2),(0,2),(1,3),(2,3),(0,3) with nodes walking
    from the first to the second vertex, then face interiors for faces (0,1,2),(0,1,3),(0,2,3),
    (1,2,3), then the cell interior (``simplex_lagrange.py:15-83``).
    """
    p = int(order)
    out: list[tuple[int, ...]] = []
    for v in range(4):
        t = [0, 0, 0, 0]
        t[v] = p
        out.append(tuple(t))
    for i, j in ((0, 1), (1, 2), (0, 2), (1, 3), (2, 3), (0, 3)):
        for k in range(1, p):
            t = [0, 0, 0, 0]
            t[i], t[j] = p - k, k
            out.append(tuple(t))
    tri_interior = [
        (a, b, p - a - b) for a in range(p - 2, 0, -1) for b in range(p - a - 1, 0, -1) if p - a - b > 0
    ]
    for face in ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)):
        for tri in tri_interior:
            t = [0, 0, 0, 0]
            for local, vtx in enumerate(face):
                t[vtx] = tri[local]
            out.append(tuple(t))
    for a in range(p - 3, 0, -1):
        for b in range(p - a - 2, 0, -1):
            for c in range(p - a - b - 1, 0, -1):
                d = p - a - b - c
                if d > 0:
                    out.append((a, b, c, d))
    return tuple(out)


@lru_cache(maxsize=None)
def tri_node_tuples(order: int) -> tuple[tuple[int, int, int], ...]:
    """Barycentric count tuples (v0, v1, v2) of the order-p triangle, in the reference's node order.

    P1: the vertices.  P2: vertices, then the midpoints of edges (1,2), (0,2), (0,1)
    (``src/slope_stability/fem/basis.py:22-33``).  P4: vertices, the midpoints of edges (0,1),
    (1,2), (2,0), the quarter points of those edges in the same edge order, each edge walked from
    its first vertex, then the three interior nodes nearest v0, v1, v2
    (``src/slope_stability/mesh/textmesh_2d.py:116-184``, ``fem/basis.py:57-75``).
    """
    p = int(order)
    verts = ((p, 0, 0), (0, p, 0), (0, 0, p))
    if p == 1:
        return verts
    if p == 2:
        return verts + ((0, 1, 1), (1, 0, 1), (1, 1, 0))
    if p == 4:
        mids = ((2, 2, 0), (0, 2, 2), (2, 0, 2))
        quarters = ((3, 1, 0), (1, 3, 0), (0, 3, 1), (0, 1, 3), (1, 0, 3), (3, 0, 1))
        interior = ((2, 1, 1), (1, 2, 1), (1, 1, 2))
        return verts + mids + quarters + interior
    raise ValueError(f"unsupported triangle order {order}")


def elevate_simplices(vcoord: np.ndarray, cells: np.ndarray, tuples) -> tuple[np.ndarray, np.ndarray]:
    """Elevate a linear simplex mesh (cells: (dim+1, n_e) vertex ids) to the Lagrange nodes
    ``tuples`` (barycentric counts, vertices first) with shared higher-order nodes.

    A higher-order node is identified by the vertices it lies on and its barycentric counts,
    so nodes on shared edges and faces are created once.  New nodes are numbered after all
    vertices, in order of first appearance (element-major, then local node).
    """
    n_vert = cells.shape[0]
    order = int(sum(tuples[0]))
    n_v = vcoord.shape[1]
    n_e = cells.shape[1]
    elem = np.empty((len(tuples), n_e), dtype=np.int64)
    elem[:n_vert] = cells
    if len(tuples) == n_vert:
        return vcoord.copy(), elem
    # key of a higher-order node: its (vertex, count) pairs sorted by vertex, padded with (-1, 0)
    hi = np.asarray(tuples[n_vert:], dtype=np.int64)  # (n_hi, n_vert) barycentric counts
    width = int((hi > 0).sum(axis=1).max())
    verts = cells.T  # (n_e, n_vert)
    key_v = np.full((n_e, hi.shape[0], width), -1, dtype=np.int64)
    key_c = np.zeros((n_e, hi.shape[0], width), dtype=np.int64)
    for li, t in enumerate(hi):
        nz = np.flatnonzero(t > 0)
        vv = verts[:, nz]
        order_ = np.argsort(vv, axis=1, kind="stable")
        key_v[:, li, : nz.size] = np.take_along_axis(vv, order_, axis=1)
        key_c[:, li, : nz.size] = t[nz][order_]
    keys = np.concatenate((key_v, key_c), axis=2).reshape(n_e * hi.shape[0], 2 * width)
    uniq, first, inverse = np.unique(keys, axis=0, return_index=True, return_inverse=True)
    # number new nodes in order of first appearance (element-major, then local node)
    rank = np.empty(uniq.shape[0], dtype=np.int64)
    rank[np.argsort(first, kind="stable")] = np.arange(uniq.shape[0])
    gid = n_v + rank[inverse.reshape(-1)]
    elem[n_vert:] = gid.reshape(n_e, hi.shape[0]).T
    # coordinates of the new nodes from their first element
    occ = np.sort(first)
    e_of, li_of = occ // hi.shape[0], occ % hi.shape[0]
    bary = hi[li_of].astype(np.float64) / order  # (n_new, n_vert)
    new_pts = np.einsum("dkn,nk->dn", vcoord[:, cells[:, e_of]], bary)
    coord = np.concatenate((vcoord, new_pts), axis=1)
    return coord, elem


def elevate_tets(vcoord: np.ndarray, tet4: np.ndarray, order: int) -> tuple[np.ndarray, np.ndarray]:
    """Elevate a linear tet mesh to Lagrange order 1, 2 or 4 (reference node order)."""
    return elevate_simplices(vcoord, tet4, tet_node_tuples(order))


def elevate_triangles(vcoord: np.ndarray, tri3: np.ndarray, order: int) -> tuple[np.ndarray, np.ndarray]:
    """Elevate a linear triangle mesh to Lagrange order 1, 2 or 4 (reference node order)."""
    return elevate_simplices(vcoord, tri3, tri_node_tuples(order))


def _kuhn_tets(nx: int, ny: int, nz: int) -> np.ndarray:
    """Six-tetrahedra split of every cell of an (nx, ny, nz) vertex-indexed box grid."""
    vid = lambda i, j, k: (i * (ny + 1) + j) * (nz + 1) + k  # noqa: E731
    I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    tets = []
    for perm in permutations(range(3)):
        off = np.zeros(3, dtype=np.int64)
        path = [off.copy()]
        for ax in perm:
            off[ax] += 1
            path.append(off.copy())
        tets.append(np.stack([vid(I + o[0], J + o[1], K + o[2]) for o in path]))
    # interleave so the six tets of one cell are consecutive
    return np.stack(tets, axis=2).reshape(4, -1)


def slope_mesh_3d(nx: int, ny: int, nz: int, *, depth: float = 30.0, elem_type: str = "P2",
                  n_layers: int = 1) -> SlopeMesh:
    grid2 = _vertex_grid_2d(nx, ny)  # (2, nx+1, ny+1)
    nx = grid2.shape[1] - 1
    zs = np.linspace(0.0, depth, nz + 1)
    X = np.repeat(grid2[0][:, :, None], nz + 1, axis=2)
    Y = np.repeat(grid2[1][:, :, None], nz + 1, axis=2)
    Z = np.broadcast_to(zs[None, None, :], X.shape)
    vcoord = np.stack((X.ravel(), Y.ravel(), Z.ravel()))
    tet4 = _kuhn_tets(nx, ny, nz)
    order = {"P1": 1, "P2": 2, "P4": 4}[elem_type.upper()]
    coord, elem = elevate_tets(vcoord, tet4, order)
    q_mask = boundary_mask_3d(coord, depth)
    cy = vcoord[1, tet4].mean(axis=0)
    top = Y1 + Y2
    material_id = np.minimum((cy / top * n_layers).astype(np.int64), n_layers - 1)
    return SlopeMesh(3, elem_type.upper(), coord, elem, q_mask, material_id, {"depth": depth})


def boundary_mask_3d(coord: np.ndarray, depth: float) -> np.ndarray:
    """Bottom fixed, lateral faces fixed in their normal direction (3D analogue of
    ``src/slope_stability/mesh/slope_2d.py:22-27``)."""
    x, y, z = coord
    tol = 1.0e-9
    x_max = X1 + X2 + X3
    q = np.ones((3, coord.shape[1]), dtype=bool)
    bottom = y <= tol
    q[:, bottom] = False
    q[0, (x <= tol) | (x >= x_max - tol)] = False
    q[2, (z <= tol) | (z >= depth - tol)] = False
    return q


def slope_mesh_2d(nx: int, ny: int, *, elem_type: str = "P2", n_layers: int = 1) -> SlopeMesh:
    grid = _vertex_grid_2d(nx, ny)
    nx = grid.shape[1] - 1
    vcoord = grid.reshape(2, -1)
    vid = lambda i, j: i * (ny + 1) + j  # noqa: E731
    I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    I, J = I.ravel(), J.ravel()
    t1 = np.stack((vid(I, J), vid(I + 1, J), vid(I + 1, J + 1)))
    t2 = np.stack((vid(I, J), vid(I + 1, J + 1), vid(I, J + 1)))
    tri = np.stack((t1, t2), axis=2).reshape(3, -1)
    order = {"P1": 1, "P2": 2, "P4": 4}.get(elem_type.upper())
    if order is None:
        raise ValueError(f"unsupported 2D element type {elem_type!r}")
    coord, elem = elevate_triangles(vcoord, tri.astype(np.int64), order)
    x_max = float(np.max(coord[0])) - 1.0e-9
    q = np.zeros((2, coord.shape[1]), dtype=bool)
    q[0] = (coord[0] > 0.0) & (coord[1] > 0.0) & (coord[0] < x_max)
    q[1] = coord[1] > 0.0
    cy = vcoord[1, tri].mean(axis=0)
    material_id = np.minimum((cy / (Y1 + Y2) * n_layers).astype(np.int64), n_layers - 1)
    return SlopeMesh(2, elem_type.upper(), coord, elem, q, material_id, {})


def displacement_field(mesh: SlopeMesh, materials: MaterialSet, amplitude: float, *,
                       band_width: float = 0.5, angle_deg: float = 30.0, seed: int = 0,
                       noise: float = 1.0e-3) -> np.ndarray:
    """Gravity settlement plus a tanh shear band through the toe, shape (dim, n_nodes)."""
    rng = np.random.default_rng(seed)
    xy = mesh.coord[:2]
    top = surface_height(xy[0])
    lam = float(np.mean(materials.lame))
    mu = float(np.mean(materials.shear))
    gam = float(np.mean(materials.gamma))
    m_mod = lam + 2.0 * mu
    y = xy[1]
    u = np.zeros_like(mesh.coord)
    u[1] = -(gam / m_mod) * (top * y - 0.5 * y * y)
    ang = np.deg2rad(angle_deg)
    tang = np.array([np.cos(ang), np.sin(ang)])
    normal = np.array([-np.sin(ang), np.cos(ang)])
    d = (xy - TOE[:, None]).T @ normal
    slide = amplitude * 0.5 * (1.0 + np.tanh(d / band_width))
    taper = 1.0
    if mesh.dim == 3:
        depth = float(mesh.extra.get("depth", 30.0))
        taper = 0.5 + 0.5 * np.sin(np.pi * mesh.coord[2] / depth)
        u[2] = 0.05 * amplitude * np.tanh(d / band_width) * np.cos(np.pi * mesh.coord[2] / depth)
    u[0] -= slide * taper * tang[0]
    u[1] -= slide * taper * tang[1]
    u += noise * amplitude * rng.standard_normal(u.shape)
    u[~mesh.q_mask] = 0.0
    return u


def displacement_basis(mesh: SlopeMesh, materials: MaterialSet, *, seed: int = 0, **kw) -> tuple[np.ndarray, np.ndarray]:
    """(G, V) with displacement_field(mesh, materials, a, seed=seed) = G + a V: the field is affine in
    the shear-band amplitude (its noise is scaled by the amplitude too), so a continuation's states
    g G + a V (load factor g, band amplitude a) cost one axpy each."""
    G = displacement_field(mesh, materials, 0.0, seed=seed, **kw)
    V = displacement_field(mesh, materials, 1.0, seed=seed, **kw) - G
    return G, V


def point_materials(mesh: SlopeMesh, materials: MaterialSet, n_q: int) -> dict[str, np.ndarray]:
    """Per-integration-point material arrays (``src/slope_stability/mesh/materials.py:33-101``)."""
    mid = np.repeat(mesh.material_id, n_q)
    return {
        "c0": materials.c0[mid].astype(np.float64),
        "phi": np.deg2rad(materials.phi[mid]).astype(np.float64),
        "psi": np.deg2rad(materials.psi[mid]).astype(np.float64),
        "shear": materials.shear[mid].astype(np.float64),
        "bulk": materials.bulk[mid].astype(np.float64),
        "lame": materials.lame[mid].astype(np.float64),
        "gamma": materials.gamma[mid].astype(np.float64),
    }


# Sizes of the reference's benchmark configurations (elements are approximate).  ``amplitude``
# is the shear-band displacement (m) that makes about 10 % of the quadrature points yield at
# lambda = 1 (found once with the CPU restatement of the return mapping; the layered sets yield
# about 7.5 % under gravity alone).
CONFIGS = {
    "2d_p2_homo": dict(dim=2, elem_type="P2", nx=100, ny=100, n_layers=1, amplitude=0.0072),  # 20,000 triangles
    "2d_p4_homo": dict(dim=2, elem_type="P4", nx=80, ny=72, n_layers=1, amplitude=0.0072),  # 11,520 triangles
    "3d_p2_homo": dict(dim=3, elem_type="P2", nx=40, ny=14, nz=30, n_layers=1, amplitude=0.0157),  # 100,800 tets
    "3d_p2_hetero": dict(dim=3, elem_type="P2", nx=64, ny=26, nz=40, n_layers=4, amplitude=0.003),  # 399,360 tets
    "3d_p4_hetero": dict(dim=3, elem_type="P4", nx=30, ny=12, nz=23, n_layers=4, amplitude=0.003),  # 49,680 tets
    "3d_p2_large": dict(dim=3, elem_type="P2", nx=110, ny=44, nz=70, n_layers=4, amplitude=0.003),  # 2,032,800 tets
    # a smaller copy of 3d_p2_homo for detailed profiles (still larger than L2 per step)
    "3d_p2_profile": dict(dim=3, elem_type="P2", nx=20, ny=8, nz=20, n_layers=1, amplitude=0.0157),  # 19,200 tets
    # a smaller copy of 3d_p4_hetero for detailed profiles
    "3d_p4_profile": dict(dim=3, elem_type="P4", nx=14, ny=6, nz=10, n_layers=4, amplitude=0.003),  # 5,040 tets
}


def register_mesh_file(path, *, elem_type: str = "P2", amplitude: float = 0.003, name: str | None = None) -> str:
    """Make a gmsh tet4 file (e.g. one of the reference's slope meshes) a named workload: its
    tetrahedra elevated to ``elem_type``, its material ids as the layers of the seeded layered
    material set, and the same synthetic gravity + shear-band displacement as the other workloads."""
    from .mesh_io import load_mesh_file

    et = str(elem_type).upper()
    data = load_mesh_file(path, elem_type=et)
    key = name or f"file:{Path(path).stem}:{et.lower()}"
    n_mat = int(data.material.max()) + 1 if data.material.size else 1
    CONFIGS[key] = dict(dim=3, elem_type=et, amplitude=float(amplitude), n_layers=max(n_mat, 1), mesh=data)
    return key


def build_config_mesh(name: str) -> SlopeMesh:
    cfg = dict(CONFIGS[name])
    cfg.pop("amplitude", None)
    if "mesh" in cfg:
        d = cfg["mesh"]
        depth = float(d.coord[2].max() - d.coord[2].min()) if d.coord.size else 0.0
        return SlopeMesh(3, cfg["elem_type"], d.coord, d.elem, d.q_mask, np.asarray(d.material, dtype=np.int64),
                         {"depth": depth})
    if cfg.pop("dim") == 2:
        return slope_mesh_2d(cfg["nx"], cfg["ny"], elem_type=cfg["elem_type"], n_layers=cfg["n_layers"])
    return slope_mesh_3d(cfg["nx"], cfg["ny"], cfg["nz"], elem_type=cfg["elem_type"], n_layers=cfg["n_layers"])


def config_workload(name: str):
    """A named configuration as a workload: mesh, material set, the reference's material specs and
    the displacement basis (G, V) (displacement_basis, seed 3) with the configuration's shear-band
    amplitude, so its states are g G + a V."""
    from types import SimpleNamespace

    cfg = CONFIGS[name]
    mesh = build_config_mesh(name)
    mats = MaterialSet.layered(4, seed=0) if cfg["n_layers"] > 1 else MaterialSet.homogeneous()
    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=float(mats.psi[i]), young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=float(mats.gamma[i]), gamma_unsat=float(mats.gamma[i]))
             for i in range(mats.c0.size)]
    G, V = displacement_basis(mesh, mats, seed=3)
    return SimpleNamespace(name=name, mesh=mesh, mats=mats, specs=specs, G=G, V=V, amp=float(cfg["amplitude"]))


def element_sample(mesh: SlopeMesh, n_elem_goal: int, chunks: int = 16) -> tuple[SlopeMesh, np.ndarray]:
    """A bounded sample of a mesh as a mesh of its own: about n_elem_goal elements taken as `chunks`
    contiguous runs spread evenly over the element order (so the sample sees every part of the
    slope, plastic zone included), their nodes renumbered in their original order.  Returns the
    sample and the original ids of its nodes (to restrict a displacement: U[:, nodes])."""
    n_el = mesh.n_elem
    if n_elem_goal >= n_el:
        return mesh, np.arange(mesh.n_nodes)
    run = max(1, n_elem_goal // chunks)
    starts = (np.arange(chunks) * (n_el // chunks)).astype(np.int64)
    sel = np.unique(np.concatenate([np.arange(s0, min(s0 + run, n_el)) for s0 in starts]))
    elem = mesh.elem[:, sel]
    nodes = np.unique(elem)
    lid = np.full(mesh.n_nodes, -1, dtype=np.int64)
    lid[nodes] = np.arange(nodes.size)
    sub = SlopeMesh(mesh.dim, mesh.elem_type, np.ascontiguousarray(mesh.coord[:, nodes]), lid[elem],
                    np.ascontiguousarray(mesh.q_mask[:, nodes]), np.asarray(mesh.material_id)[sel], dict(mesh.extra))
    return sub, nodes
