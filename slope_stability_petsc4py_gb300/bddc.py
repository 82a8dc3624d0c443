"""Non-overlapping subdomain (BDDC / MATIS) tangent assembly, GPU-resident.

Drop-in counterpart of the subdomain half of ``src/slope_stability/fem/distributed_tangent.py``:

* ``BDDCSubdomainPattern`` keeps the reference's field names (``:78-110``);
* ``prepare_bddc_subdomain_pattern`` (``:1178-1387``): the subdomain is every element whose
  smallest node lies in the owned node range; its local square pattern (rows: every local dof,
  columns: the free local dofs; a constrained row holds its diagonal only) is exactly the owned-row
  pattern of the local mesh with every local node owned, so the same C++ builder makes it (and the
  element->CSR scatter map); geometry and elastic values run on the GPU;
* ``assemble_bddc_subdomain_tangent_values`` (``:1390-1434``): K_e = sum_q B^T (w DS) B over the
  subdomain's elements, scattered through the map by the element tangent kernel
  (``ssp_tangent_element``), constrained diagonals set to 1.

The reference hands the local CSR to PETSc (``local_csr_to_petsc_matis_matrix``); here the
operator returns a ``SubdomainCSRMatrix`` carrying the same local CSR, local-to-global map and
metadata for that call.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from time import perf_counter

import numpy as np
from scipy.sparse import csr_matrix

from . import _lib
from .distributed_tangent import _elastic_ds_device, _ensure_int32_capacity, _is_torch, _PatternBuild
from .fem import N_NODES, quadrature, reference_gradients
from .materials import heterogenous_materials

ADJACENCY_SOURCES = ("csr", "none", "topology")


@dataclass(frozen=True)
class BDDCSubdomainPattern:
    """Local square subdomain assembly metadata for PETSc MATIS/PCBDDC (reference field names)."""

    dim: int
    n_strain: int
    owned_node_range: tuple[int, int]
    owned_coord: np.ndarray
    local_nodes: np.ndarray
    local_elements: np.ndarray
    local_coord: np.ndarray
    local_q_mask: np.ndarray
    local_global_dofs: np.ndarray
    local_matrix_pattern: csr_matrix
    elastic_values: np.ndarray
    local_assembly_weight: np.ndarray
    dphi1: np.ndarray
    dphi2: np.ndarray
    dphi3: np.ndarray
    local_int_indices: np.ndarray
    overlap_local_positions: np.ndarray
    scatter_map: np.ndarray
    local_dirichlet_dofs: np.ndarray
    constrained_diag_positions: np.ndarray
    local_field_dofs: tuple
    local_adjacency_indptr: np.ndarray
    local_adjacency_indices: np.ndarray
    local_primal_vertices: np.ndarray
    adjacency_source: str
    n_p: int
    n_q: int
    stats: dict
    timings: dict
    device: dict = field(default_factory=dict, repr=False, compare=False)

    @property
    def nnz(self) -> int:
        return int(self.local_matrix_pattern.nnz)

    @property
    def n_local_int(self) -> int:
        return int(self.local_int_indices.size)


def _dofs_of_nodes(nodes: np.ndarray, dim: int) -> np.ndarray:
    nodes = np.asarray(nodes, dtype=np.int64).ravel()
    return (dim * np.repeat(nodes, dim) + np.tile(np.arange(dim, dtype=np.int64), nodes.size)).astype(np.int64)


def _topology_adjacency(elem_local: np.ndarray, n_local_nodes: int, dim: int) -> tuple[np.ndarray, np.ndarray]:
    """Dof adjacency from shared elements: row dim*a+c lists, sorted, every dof of every node that
    shares an element with node a (a included), as ``distributed_tangent.py:559-589`` builds it."""
    n_p, n_el = elem_local.shape
    if n_local_nodes == 0:
        return np.zeros(1, dtype=np.int32), np.empty(0, dtype=np.int32)
    a = np.repeat(elem_local, n_p, axis=0).ravel()  # node pairs (a, b) of every element
    b = np.tile(elem_local, (n_p, 1)).ravel()
    key = np.unique(np.concatenate((a * n_local_nodes + b, np.arange(n_local_nodes, dtype=np.int64) * (n_local_nodes + 1))))
    na, nb = key // n_local_nodes, key % n_local_nodes  # grouped by a, b ascending within a group
    per_node = np.bincount(na, minlength=n_local_nodes)
    node_ptr = np.concatenate(([0], np.cumsum(per_node)))
    # every row of node a: dim * (its neighbours), each neighbour expanded to its dim dofs
    row_len = np.repeat(dim * per_node, dim)
    indptr = np.concatenate(([0], np.cumsum(row_len))).astype(np.int64)
    _ensure_int32_capacity("adjacency nnz", int(indptr[-1]))
    neigh_dofs = (dim * nb[:, None] + np.arange(dim)[None, :]).ravel()  # per node: its neighbours' dofs, sorted
    row_start = np.repeat(dim * node_ptr[:-1], dim)  # where a row's columns start in neigh_dofs
    offs = np.arange(int(indptr[-1])) - np.repeat(indptr[:-1], row_len)
    indices = neigh_dofs[np.repeat(row_start, row_len) + offs]
    return indptr.astype(np.int32), indices.astype(np.int32)


def _corner_primal_vertices(coord_local, interface_nodes_local, local_dirichlet_dofs, dim) -> np.ndarray:
    """The interface nodes nearest the 2^dim corners of the interface's bounding box (the first one
    on ties, each once), as free dofs, sorted (``distributed_tangent.py:592-623``)."""
    nodes = np.asarray(interface_nodes_local, dtype=np.int64).ravel()
    if nodes.size == 0:
        return np.empty(0, dtype=np.int32)
    pts = np.asarray(coord_local, dtype=np.float64)[:, nodes]
    lo, hi = pts.min(axis=1), pts.max(axis=1)
    chosen: list[int] = []
    for corner in range(1 << dim):
        target = np.array([hi[ax] if (corner >> ax) & 1 else lo[ax] for ax in range(dim)])
        cand = int(nodes[int(np.argmin(np.linalg.norm(pts.T - target[None, :], axis=1)))])
        if cand not in chosen:
            chosen.append(cand)
    dofs = _dofs_of_nodes(np.asarray(chosen), dim)
    dofs = np.setdiff1d(dofs, np.asarray(local_dirichlet_dofs, dtype=np.int64))
    return dofs.astype(np.int32)


def bddc_local_structure(coord, elem, q_mask, owned_node_range, *, n_q: int, overlap_local_int_indices=None,
                         adjacency_source: str = "csr", corner_only_primals: bool = False) -> dict:
    """Host part of the subdomain pattern (no GPU): element and node selection, local square CSR
    pattern and scatter map (C++ builder), Dirichlet rows and their diagonal positions, dof
    adjacency, primal vertices and the overlap positions of the subdomain's points."""
    elem = np.asarray(elem, dtype=np.int64)
    q_mask = np.asarray(q_mask, dtype=bool)
    dim, n_nodes = q_mask.shape
    n_p, n_elem = elem.shape
    node0, node1 = (int(v) for v in owned_node_range)
    mode = str(adjacency_source).strip().lower()
    if mode not in ADJACENCY_SOURCES:
        raise ValueError(f"Unsupported BDDC adjacency_source {adjacency_source!r}; expected one of {list(ADJACENCY_SOURCES)}")
    owners = np.min(elem, axis=0) if n_elem else np.empty(0, dtype=np.int64)
    local_elements = np.flatnonzero((owners >= node0) & (owners < node1)).astype(np.int64)
    if local_elements.size:
        local_nodes = np.unique(elem[:, local_elements]).astype(np.int64)
        lid = np.full(n_nodes, -1, dtype=np.int64)
        lid[local_nodes] = np.arange(local_nodes.size)
        elem_local = lid[elem[:, local_elements]]
    else:
        local_nodes = np.empty(0, dtype=np.int64)
        elem_local = np.empty((n_p, 0), dtype=np.int64)
    n_loc = int(local_nodes.size)
    local_global_dofs = _dofs_of_nodes(local_nodes, dim)
    q_local = q_mask[:, local_nodes]
    free_local = q_local.reshape(-1, order="F")
    n_ld = dim * n_p
    if n_loc:
        pb = _PatternBuild(elem_local, q_local, (0, n_loc))
        g = {k: pb.get(k) for k in ("overlap_elements", "indptr", "indices", "scatter_map", "constrained_diag_positions")}
        pb.close()
        if not np.array_equal(g["overlap_elements"], np.arange(local_elements.size)):
            raise RuntimeError("local square pattern: every subdomain element must touch the subdomain's nodes")
    else:
        g = {"indptr": np.zeros(1, dtype=np.int32), "indices": np.empty(0, dtype=np.int32),
             "scatter_map": np.empty((0, n_ld * n_ld), dtype=np.int32),
             "constrained_diag_positions": np.empty(0, dtype=np.int32)}
    n_dofs = dim * n_loc
    pattern = csr_matrix((np.ones(g["indices"].size), g["indices"], g["indptr"]), shape=(n_dofs, n_dofs))
    dirichlet = np.flatnonzero(~free_local).astype(np.int32)
    if mode == "csr":
        adj_ptr, adj_idx = g["indptr"].astype(np.int32).copy(), g["indices"].astype(np.int32).copy()
    elif mode == "topology":
        adj_ptr, adj_idx = _topology_adjacency(elem_local, n_loc, dim)
    else:
        adj_ptr, adj_idx = np.empty(0, dtype=np.int32), np.empty(0, dtype=np.int32)
    interface = np.empty(0, dtype=np.int64)
    if local_elements.size and local_elements.size < n_elem:
        elsewhere = np.ones(n_elem, dtype=bool)
        elsewhere[local_elements] = False
        touched = np.zeros(n_nodes, dtype=bool)
        touched[elem[:, elsewhere].ravel()] = True
        interface = np.flatnonzero(touched[local_nodes]).astype(np.int64)  # local ids, ascending
    if corner_only_primals:
        primal = _corner_primal_vertices(np.asarray(coord, dtype=np.float64)[:, local_nodes], interface, dirichlet, dim)
    else:
        # PETSc derives the primal space itself unless corners are forced (distributed_tangent.py:1310-1313)
        primal = np.empty(0, dtype=np.int32)
    local_int_indices = (local_elements[:, None] * n_q + np.arange(n_q)[None, :]).reshape(-1)
    if overlap_local_int_indices is None or local_int_indices.size == 0:
        positions = np.empty(0, dtype=np.int32)
    else:
        # position of every subdomain point in the overlap ordering (the last one if repeated, as
        # the reference's dictionary lookup gives); a point the overlap lacks raises KeyError
        ov = np.asarray(overlap_local_int_indices, dtype=np.int64).ravel()
        if ov.size == 0:
            raise KeyError(int(local_int_indices[0]))
        order = np.argsort(ov, kind="stable")
        at = np.searchsorted(ov, local_int_indices, side="right", sorter=order) - 1
        hit = (at >= 0) & (ov[order[np.maximum(at, 0)]] == local_int_indices)
        if not hit.all():
            raise KeyError(int(local_int_indices[np.flatnonzero(~hit)[0]]))
        positions = order[at].astype(np.int32)
    return {
        "local_elements": local_elements, "local_nodes": local_nodes, "elem_local": elem_local,
        "local_global_dofs": local_global_dofs, "local_q_mask": q_local, "free_local": free_local,
        "local_matrix_pattern": pattern, "scatter_map": g["scatter_map"],
        "constrained_diag_positions": g["constrained_diag_positions"].astype(np.int32), "local_dirichlet_dofs": dirichlet,
        "local_adjacency_indptr": adj_ptr, "local_adjacency_indices": adj_idx, "interface_nodes_local": interface,
        "local_primal_vertices": primal,
        "local_int_indices": local_int_indices, "overlap_local_positions": positions,
        "local_field_dofs": tuple(np.arange(c, n_dofs, dim, dtype=np.int32) for c in range(dim)),
        "adjacency_source": mode,
    }


def prepare_bddc_subdomain_pattern(coord, elem, q_mask, material_identifier, materials, owned_node_range, *,
                                   elem_type: str = "P2", overlap_local_int_indices=None, adjacency_source: str = "csr",
                                   corner_only_primals: bool = False) -> BDDCSubdomainPattern:
    """Prepare a non-overlapping local subdomain pattern for MATIS/PCBDDC (on the current CUDA
    device); the arguments and fields are the reference's (``distributed_tangent.py:1178-1387``)."""
    t = _lib.require_cuda()
    coord = np.asarray(coord, dtype=np.float64)
    elem = np.asarray(elem, dtype=np.int64)
    q_mask = np.asarray(q_mask, dtype=bool)
    dim, n_nodes = coord.shape
    if q_mask.shape != (dim, n_nodes):
        raise ValueError("q_mask shape must match coord")
    et = str(elem_type).upper()
    n_p = int(elem.shape[0])
    if N_NODES.get((dim, et)) != n_p:
        raise ValueError(f"elem has {n_p} nodes per element, which is not {dim}D {et}")
    node0, node1 = (int(v) for v in owned_node_range)
    xi, wf = quadrature(dim, et)
    n_q = int(xi.shape[1])
    t0 = perf_counter()
    s = bddc_local_structure(coord, elem, q_mask, (node0, node1), n_q=n_q,
                             overlap_local_int_indices=overlap_local_int_indices, adjacency_source=adjacency_source,
                             corner_only_primals=corner_only_primals)
    pattern_time = perf_counter() - t0
    local_elements, local_nodes, elem_local = s["local_elements"], s["local_nodes"], s["elem_local"]
    n_el, n_int, nnz = int(local_elements.size), int(local_elements.size) * n_q, int(s["local_matrix_pattern"].nnz)
    _ensure_int32_capacity("n_int", n_int)
    f64 = t.float64
    dev = {}
    t1 = perf_counter()
    coord_local = np.ascontiguousarray(coord[:, local_nodes])
    dev["dphi1"] = t.empty((n_int, n_p), dtype=f64, device="cuda")
    dev["dphi2"] = t.empty((n_int, n_p), dtype=f64, device="cuda")
    dev["dphi3"] = t.empty((n_int, n_p) if dim == 3 else (1, 1), dtype=f64, device="cuda")
    dev["weight"] = t.empty(n_int, dtype=f64, device="cuda")
    if n_el:
        coord_d = _lib.to_device(coord_local, f64)
        elem_d = _lib.to_device(np.ascontiguousarray(elem_local), t.int64)
        dhat = _lib.to_device(np.ascontiguousarray(reference_gradients(dim, et)), f64)
        wf_d = _lib.to_device(np.asarray(wf, dtype=np.float64), f64)
        _lib.call("ssp_geometry", dim, _lib.ptr(coord_d), _lib.ptr(elem_d), _lib.ptr(dhat), _lib.ptr(wf_d),
                  int(local_nodes.size), n_el, n_p, n_q, _lib.ptr(dev["dphi1"]), _lib.ptr(dev["dphi2"]),
                  _lib.ptr(dev["dphi3"]) if dim == 3 else None, _lib.ptr(dev["weight"]), _lib.stream_handle())
    geometry_time = perf_counter() - t1
    t2 = perf_counter()
    dev["scatter_map"] = _lib.to_device(np.ascontiguousarray(s["scatter_map"]), t.int32)
    dev["cdiag"] = _lib.to_device(s["constrained_diag_positions"], t.int32)
    dev["elastic_values"] = t.zeros(max(nnz, 1), dtype=f64, device="cuda")[:nnz]
    if n_el:
        _c0, _phi, _psi, shear, bulk, lame, _gamma = heterogenous_materials(
            np.asarray(material_identifier, dtype=np.int64).ravel()[local_elements], np.ones(n_int, dtype=bool), n_q,
            materials)
        dev["shear"], dev["lame"] = _lib.to_device(shear, f64), _lib.to_device(lame, f64)
        ds_el = _elastic_ds_device(t, dim, dev["shear"], _lib.to_device(bulk, f64), dev["lame"])
        _lib.call("ssp_tangent_element", dim, 1, _lib.ptr(dev["dphi1"]), _lib.ptr(dev["dphi2"]),
                  _lib.ptr(dev["dphi3"]) if dim == 3 else None, _lib.ptr(ds_el), _lib.ptr(dev["weight"]),
                  _lib.ptr(dev["scatter_map"]), n_el, n_p, n_q, nnz, _lib.ptr(dev["elastic_values"]), 0,
                  _lib.stream_handle())
        _lib.call("ssp_finish_values", _lib.ptr(dev["elastic_values"]), nnz, _lib.ptr(dev["cdiag"]),
                  int(dev["cdiag"].numel()), None, 0.0, _lib.stream_handle())
    t.cuda.synchronize()
    _lib.raise_on_device_status()
    elastic_time = perf_counter() - t2
    host = {k: dev[k].cpu().numpy() for k in ("dphi1", "dphi2", "weight")}
    dphi3 = dev["dphi3"].cpu().numpy() if dim == 3 else np.empty((0, 0), dtype=np.float64)
    elastic_values = dev["elastic_values"].cpu().numpy()
    lp = s["local_matrix_pattern"]
    scatter_bytes = int(s["scatter_map"].nbytes)
    pattern_bytes = int(lp.indptr.nbytes + lp.indices.nbytes + 8 * nnz)
    dphi_bytes = int(host["dphi1"].nbytes + host["dphi2"].nbytes + dphi3.nbytes)
    return BDDCSubdomainPattern(
        dim=dim, n_strain=6 if dim == 3 else 3, owned_node_range=(node0, node1),
        owned_coord=np.ascontiguousarray(coord[:, node0:node1]), local_nodes=local_nodes,
        local_elements=local_elements, local_coord=coord_local, local_q_mask=np.ascontiguousarray(s["local_q_mask"]),
        local_global_dofs=s["local_global_dofs"], local_matrix_pattern=lp, elastic_values=elastic_values,
        local_assembly_weight=host["weight"], dphi1=host["dphi1"], dphi2=host["dphi2"], dphi3=dphi3,
        local_int_indices=s["local_int_indices"], overlap_local_positions=s["overlap_local_positions"],
        scatter_map=np.ascontiguousarray(s["scatter_map"]), local_dirichlet_dofs=s["local_dirichlet_dofs"],
        constrained_diag_positions=s["constrained_diag_positions"], local_field_dofs=s["local_field_dofs"],
        local_adjacency_indptr=s["local_adjacency_indptr"], local_adjacency_indices=s["local_adjacency_indices"],
        local_primal_vertices=s["local_primal_vertices"], adjacency_source=s["adjacency_source"], n_p=n_p, n_q=n_q,
        stats={
            "local_pattern_bytes": float(pattern_bytes), "local_scatter_bytes": float(scatter_bytes),
            "local_elastic_bytes": float(8 * nnz), "local_dphi_bytes": float(dphi_bytes),
            "local_total_bytes": float(pattern_bytes + scatter_bytes + 8 * nnz + dphi_bytes),
            "local_interface_nodes_count": float(s["interface_nodes_local"].size),
            "local_primal_vertices_count": float(s["local_primal_vertices"].size),
            "explicit_primal_vertices_used": float(bool(s["local_primal_vertices"].size)),
            "adjacency_source": float({"none": 0, "csr": 1, "topology": 2}[s["adjacency_source"]]),
        },
        timings={"local_partition_s": 0.0, "local_geometry_s": float(geometry_time),
                 "local_elastic_s": float(elastic_time), "local_pattern_s": float(pattern_time),
                 "local_scatter_missing": 0.0},
        device=dev,
    )


def bddc_tangent_values_device(pattern: BDDCSubdomainPattern, DS_aos, *, out=None):
    """Subdomain tangent values on the device from per-point DS rows (n_local_int, n_strain^2),
    CUDA tensor in and out; constrained diagonals set to 1."""
    t = _lib.require_cuda()
    d = pattern.device
    nnz, n_el = pattern.nnz, int(pattern.local_elements.size)
    vals = out if out is not None else t.empty(max(nnz, 1), dtype=t.float64, device="cuda")[:nnz]
    st = _lib.stream_handle()
    if n_el == 0:
        vals.zero_()
        return vals
    _lib.call("ssp_tangent_element", pattern.dim, 0, _lib.ptr(d["dphi1"]), _lib.ptr(d["dphi2"]),
              _lib.ptr(d["dphi3"]) if pattern.dim == 3 else None, _lib.ptr(DS_aos), _lib.ptr(d["weight"]),
              _lib.ptr(d["scatter_map"]), n_el, pattern.n_p, pattern.n_q, nnz, _lib.ptr(vals), 0, st)
    _lib.call("ssp_finish_values", _lib.ptr(vals), nnz, _lib.ptr(d["cdiag"]), int(d["cdiag"].numel()), None, 0.0, st)
    return vals


def assemble_bddc_subdomain_tangent_values(pattern: BDDCSubdomainPattern, DS, *, use_compiled: bool = True):
    """Local square tangent values of the subdomain (``distributed_tangent.py:1390-1434``).

    DS: (n_strain^2, n) with n the subdomain's point count or the global point count (then the
    subdomain's columns, ``local_int_indices``, are taken).  NumPy in -> NumPy out; a CUDA tensor
    in -> a CUDA tensor out.  ``use_compiled`` is accepted for signature compatibility."""
    t = _lib.require_cuda()
    rows = int(pattern.n_strain * pattern.n_strain)
    n_loc = int(pattern.local_int_indices.size)
    if _is_torch(DS):
        if DS.ndim != 2 or DS.shape[0] != rows:
            raise ValueError(f"DS must have shape ({rows}, n_int)")
        src = DS.to(device="cuda", dtype=t.float64)
        if src.shape[1] != n_loc:
            src = src[:, t.as_tensor(pattern.local_int_indices, device="cuda")]
        vals = bddc_tangent_values_device(pattern, src.T.contiguous())
        _lib.raise_on_device_status()
        return vals
    ds = np.asarray(DS, dtype=np.float64)
    if ds.ndim != 2 or ds.shape[0] != rows:
        raise ValueError(f"DS must have shape ({rows}, n_int)")
    local = ds.T if ds.shape[1] == n_loc else ds[:, pattern.local_int_indices].T
    vals = bddc_tangent_values_device(pattern, _lib.to_device(np.ascontiguousarray(local), t.float64))
    out = vals.cpu().numpy()
    _lib.raise_on_device_status()
    return out
