"""Fixed owned-row tangent pattern and the assembly functions, GPU-resident.

Drop-in counterpart of ``src/slope_stability/fem/distributed_tangent.py``:

* ``OwnedTangentPattern`` carries the reference's field names (``:29-77``); the arrays the hot
  path reads (dphi, weights, element->CSR map, dof lids, CSR pattern, elastic values) live in
  HBM under ``pattern.device``; host copies are made only when a caller reads a host field.
* ``prepare_owned_tangent_pattern`` (``:937-1175``) builds the CSR pattern and maps with the
  C++ builder (bit-identical to the reference's dictionary loops) and the geometry and elastic
  values with CUDA kernels.
* ``assemble_overlap_strain`` (``:886-907``), ``assemble_owned_force_from_local_stress``
  (``:910-934``), ``assemble_owned_tangent_values`` (``:1559-1612``),
  ``assemble_owned_tangent_matrix`` (``:1615-1628``) and ``assemble_owned_regularized_matrix``
  (``:1631-1647``) keep their signatures.  Inputs may be NumPy arrays (results come back as
  NumPy, as in the reference) or CUDA tensors (results stay on the device).

``use_compiled`` is accepted for signature compatibility; there is one implementation, the
CUDA one, and no CPU fallback.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from time import perf_counter

import numpy as np
from scipy.sparse import csr_matrix

from . import _lib
from .fem import N_NODES, quadrature, reference_gradients
from .materials import heterogenous_materials

INT32_MAX = int(np.iinfo(np.int32).max)
DEFAULT_TANGENT_KERNEL = "rows"
SUPPORTED_TANGENT_KERNELS = frozenset({"legacy", "rows", "rows_gather"})


def _ensure_int32_capacity(name: str, value: int) -> None:
    if int(value) > INT32_MAX:
        raise OverflowError(f"{name}={int(value)} exceeds int32 capacity")


def _normalize_tangent_kernel(kernel) -> str:
    k = DEFAULT_TANGENT_KERNEL if kernel is None else str(kernel).strip().lower()
    if k not in SUPPORTED_TANGENT_KERNELS:
        raise ValueError(f"Unsupported tangent kernel {kernel!r}; expected one of {sorted(SUPPORTED_TANGENT_KERNELS)}")
    return k


def _elem_type_from_np(dim: int, n_p: int) -> str:
    for (d, et), n in N_NODES.items():
        if d == dim and n == n_p:
            return et
    raise ValueError(f"no {dim}D element with {n_p} nodes")


class _PatternBuild:
    """RAII wrapper around the C++ pattern builder handle."""

    NAMES = {
        "overlap_elements": np.int64, "overlap_nodes": np.int64, "overlap_element_dof_lids": np.int32,
        "owned_local_overlap_dofs": np.int64, "indptr": np.int32, "indices": np.int32,
        "constrained_diag_positions": np.int32, "scatter_map": np.int32, "row_slot_ptr": np.int32,
        "slot_elem": np.int32, "slot_lrow": np.uint8, "slot_pos": np.int32, "elem_row": np.int32,
        "owned_free_mask": np.uint8,
    }

    def __init__(self, elem, q_mask, owned_node_range):
        lib = _lib.load()
        elem = np.ascontiguousarray(elem, dtype=np.int64)
        q_mask = np.asarray(q_mask, dtype=bool)
        self.dim, n_nodes = q_mask.shape
        self.n_p, self.n_elem = elem.shape
        free = np.ascontiguousarray(q_mask.reshape(-1, order="F").astype(np.uint8))
        n0, n1 = (int(v) for v in owned_node_range)
        handle = ctypes.c_void_p()
        _lib.check(lib.ssp_pattern_build(self.dim, n_nodes, self.n_p, self.n_elem, elem.ctypes.data, free.ctypes.data, n0,
                                         n1, ctypes.byref(handle)), "ssp_pattern_build")
        self.handle = handle
        sizes = np.zeros(7, dtype=np.int64)
        _lib.check(lib.ssp_pattern_sizes(handle, sizes.ctypes.data), "ssp_pattern_sizes")
        n_ov, n_ovn, n_rows, nnz, n_slots, n_cd, n_ld = (int(v) for v in sizes)
        self.sizes = dict(n_ov=n_ov, n_ovn=n_ovn, n_rows=n_rows, nnz=nnz, n_slots=n_slots, n_cd=n_cd, n_ld=n_ld)
        self.shapes = {
            "overlap_elements": (n_ov,), "overlap_nodes": (n_ovn,), "overlap_element_dof_lids": (n_ov, n_ld),
            "owned_local_overlap_dofs": (n_rows,), "indptr": (n_rows + 1,), "indices": (nnz,),
            "constrained_diag_positions": (n_cd,), "scatter_map": (n_ov, n_ld * n_ld), "row_slot_ptr": (n_rows + 1,),
            "slot_elem": (n_slots,), "slot_lrow": (n_slots,), "slot_pos": (n_slots, n_ld), "elem_row": (n_ov, n_ld),
            "owned_free_mask": (n_rows,),
        }

    def get(self, name):
        out = np.empty(self.shapes[name], dtype=self.NAMES[name])
        if out.size:
            _lib.check(_lib.load().ssp_pattern_copy(self.handle, name.encode(), out.ctypes.data), "ssp_pattern_copy")
        return out

    def close(self):
        if self.handle:
            _lib.load().ssp_pattern_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class OwnedTangentPattern:
    """Fixed owned-row tangent sparsity and local assembly metadata (reference field names)."""

    dim: int
    n_strain: int
    owned_node_range: tuple[int, int]
    owned_row_range: tuple[int, int]
    overlap_nodes: np.ndarray
    overlap_elements: np.ndarray
    overlap_global_dofs: np.ndarray
    overlap_B: object
    overlap_element_dof_lids: np.ndarray
    owned_local_overlap_dofs: np.ndarray
    owned_free_mask: np.ndarray
    owned_free_local_rows: np.ndarray
    global_free_size: int
    local_matrix_pattern: csr_matrix
    local_int_indices: np.ndarray
    unique_nodes: np.ndarray
    unique_elements: np.ndarray
    unique_local_int_indices: np.ndarray
    scatter_map: np.ndarray
    row_slot_ptr: np.ndarray
    slot_elem: np.ndarray
    slot_lrow: np.ndarray
    slot_pos: np.ndarray
    constrained_diag_positions: np.ndarray
    n_p: int
    n_q: int
    elem_type: str
    device: dict = field(repr=False)
    stats: dict = field(default_factory=dict)
    timings: dict = field(default_factory=dict)
    # whether every overlap element is affine (the mixed form's J^{-1} strain and force); None: not checked
    affine: bool | None = field(default=None, repr=False)
    # whether the plain form's regrouped P2 strain and force apply (3D P2, every element affine to
    # rounding); None: not checked
    affine_p2: bool | None = field(default=None, repr=False)
    # whether the plain form's J^{-1} strain and force apply (3D P1 / P4, every element affine to
    # rounding); None: not checked
    affine_fp64: bool | None = field(default=None, repr=False)

    # host views of device-resident per-point data (copied on first access)
    def _host(self, key):
        cache = self.__dict__.setdefault("_host_cache", {})
        if key not in cache:
            cache[key] = self.device[key].cpu().numpy()
        return cache[key]

    @property
    def dphi1(self):
        return self._host("dphi1")

    @property
    def dphi2(self):
        return self._host("dphi2")

    @property
    def dphi3(self):
        return self._host("dphi3") if self.dim == 3 else np.empty((0, 0))

    @property
    def overlap_assembly_weight(self):
        return self._host("weight")

    @property
    def elastic_values(self):
        return self._host("elastic_values")

    @property
    def unique_global_dofs(self):
        return (self.dim * np.repeat(self.unique_nodes, self.dim) + np.tile(np.arange(self.dim), self.unique_nodes.size))

    @property
    def nnz(self) -> int:
        return int(self.local_matrix_pattern.nnz)

    @property
    def n_local_int(self) -> int:
        return int(self.local_int_indices.size)


def _elastic_ds_device(t, dim, shear, bulk, lame):
    """Per-point elastic D (AoS, column-major blocks) of build_elastic_stiffness_matrix
    (src/slope_stability/fem/assembly.py:248-307)."""
    n = shear.numel()
    if dim == 3:
        iota = t.tensor([1.0, 1.0, 1.0, 0.0, 0.0, 0.0], dtype=t.float64, device=shear.device)
        vol = t.outer(iota, iota)
        ident = t.diag(t.tensor([1.0, 1.0, 1.0, 0.5, 0.5, 0.5], dtype=t.float64, device=shear.device)) - vol / 3.0
        vol_f, id_f = vol.T.reshape(-1), ident.T.reshape(-1)
        return (vol_f[None, :] * bulk[:, None] + 2.0 * id_f[None, :] * shear[:, None]).contiguous()
    iota = t.tensor([1.0, 1.0, 0.0], dtype=t.float64, device=shear.device)
    vol = t.outer(iota, iota)
    ident = t.diag(t.tensor([1.0, 1.0, 0.5], dtype=t.float64, device=shear.device))
    vol_f, id_f = vol.T.reshape(-1), ident.T.reshape(-1)
    return (vol_f[None, :] * lame[:, None] + 2.0 * id_f[None, :] * shear[:, None]).contiguous().reshape(n, 9)


def _project_values_onto_pattern(source, indptr, indices, n_cols: int) -> np.ndarray:
    """Values of a CSR matrix ``source`` (rows = the pattern's rows) at the pattern's positions;
    entries outside the pattern are dropped, positions without an entry are 0, and of repeated
    entries the last one counts -- what the reference's per-row dictionary lookup gives
    (distributed_tangent.py:628-640)."""
    src = source.tocsr() if hasattr(source, "tocsr") else source
    indptr = np.asarray(indptr, dtype=np.int64)
    n_rows = indptr.size - 1
    if src.shape[0] != n_rows:
        raise ValueError(f"elastic rows have {src.shape[0]} rows, the pattern {n_rows}")
    keys = np.repeat(np.arange(n_rows, dtype=np.int64), np.diff(indptr)) * n_cols + np.asarray(indices, np.int64)
    s_ptr = np.asarray(src.indptr, dtype=np.int64)
    s_keys = np.repeat(np.arange(n_rows, dtype=np.int64), np.diff(s_ptr)) * n_cols + np.asarray(src.indices, np.int64)
    out = np.zeros(keys.size, dtype=np.float64)
    if keys.size == 0 or s_keys.size == 0:
        return out
    pos = np.minimum(np.searchsorted(keys, s_keys), keys.size - 1)
    hit = keys[pos] == s_keys
    out[pos[hit]] = np.asarray(src.data, dtype=np.float64)[hit]  # repeated positions: the last entry is kept
    return out


def _strain_operator(dim: int, dphi, elem_ov, n_q: int, n_nodes: int) -> csr_matrix:
    """Sparse strain operator of a (sub)mesh from its per-point gradients dphi[k] (n_int, n_p):
    E[s + n_strain * p] = sum_j B[s + n_strain * p, j] u[j], engineering shears, the reference's
    row/column layout and canonical CSR form (fem/assembly.py:205-230 for 3D, :96-122 for 2D)."""
    from scipy.sparse import coo_matrix

    elem_ov = np.asarray(elem_ov, dtype=np.int64)
    n_p, n_el = elem_ov.shape
    n_int = n_el * n_q
    pts = np.arange(n_int, dtype=np.int64)
    node = np.repeat(elem_ov.T, n_q, axis=0)  # (n_int, n_p): node of local node a at point p
    if dim == 3:
        # (strain row, component, gradient) of the nine nonzeros of a node's 6x3 block
        terms = ((0, 0, 0), (3, 0, 1), (5, 0, 2), (1, 1, 1), (3, 1, 0), (4, 1, 2), (2, 2, 2), (4, 2, 1), (5, 2, 0))
    else:
        terms = ((0, 0, 0), (2, 0, 1), (1, 1, 1), (2, 1, 0))
    ns = 6 if dim == 3 else 3
    rows = [np.broadcast_to((ns * pts + s)[:, None], (n_int, n_p)) for s, _c, _k in terms]
    cols = [dim * node + c for _s, c, _k in terms]
    vals = [np.asarray(dphi[k], dtype=np.float64) for _s, _c, k in terms]
    B = coo_matrix((np.concatenate([v.ravel() for v in vals]),
                    (np.concatenate([r.ravel() for r in rows]), np.concatenate([c.ravel() for c in cols]))),
                   shape=(ns * n_int, dim * n_nodes)).tocsr()
    B.eliminate_zeros()
    return B


def prepare_owned_tangent_pattern(coord, elem, q_mask, material_identifier, materials, owned_node_range, *,
                                  elem_type: str = "P2", include_unique: bool = True,
                                  include_legacy_scatter: bool = True, include_overlap_B: bool = True,
                                  elastic_rows=None, keep_slot_metadata: bool = True) -> OwnedTangentPattern:
    """Prepare the fixed owned-row pattern for repeated tangent assembly (on the current CUDA device).

    ``include_overlap_B``: build the overlap submesh's sparse strain operator ``overlap_B``
    (scipy CSR, rows ``s + n_strain * point``, columns the overlap dofs), as the reference does
    (fem/assembly.py:205-230, 2D :96-122).  The CUDA kernels never read it; it costs host memory
    and a device -> host copy of the gradients, so ``ConstitutiveOperator.from_mesh`` passes False.
    ``elastic_rows``: the reference's ``OwnedElasticRows`` for the same owned range (its
    ``local_matrix`` values are projected onto the pattern, as distributed_tangent.py:1040 does),
    or a previously prepared pattern of this package for the same mesh and range (its device
    elastic values are reused).  ``keep_slot_metadata=False`` skips the host copies of the
    row-slot arrays (the device path does not read them).
    """
    t = _lib.require_cuda()
    timings = {}
    t0 = perf_counter()
    coord = np.asarray(coord, dtype=np.float64)
    elem = np.asarray(elem, dtype=np.int64)
    q_mask = np.asarray(q_mask, dtype=bool)
    dim, n_nodes = q_mask.shape
    if coord.shape != (dim, n_nodes):
        raise ValueError("q_mask shape must match coord")
    n_p, n_elem = elem.shape
    et = str(elem_type).upper()
    if N_NODES.get((dim, et)) != n_p:
        raise ValueError(f"elem has {n_p} nodes per element, which is not {dim}D {et}")
    n0, n1 = (int(v) for v in owned_node_range)
    if n0 < 0 or n1 > n_nodes or n1 < n0:
        raise ValueError("owned_node_range is outside the mesh")
    pb = _PatternBuild(elem, q_mask, (n0, n1))
    timings["structural_pattern_s"] = perf_counter() - t0
    g = {k: pb.get(k) for k in ("overlap_elements", "overlap_nodes", "overlap_element_dof_lids",
                                "owned_local_overlap_dofs", "indptr", "indices", "constrained_diag_positions",
                                "scatter_map", "elem_row", "owned_free_mask")}
    if keep_slot_metadata:
        for k in ("row_slot_ptr", "slot_elem", "slot_lrow", "slot_pos"):
            g[k] = pb.get(k)
    sizes = pb.sizes
    pb.close()
    ov_el, ov_nodes = g["overlap_elements"], g["overlap_nodes"]
    n_rows, nnz = sizes["n_rows"], sizes["nnz"]
    owned_free = g["owned_free_mask"].astype(bool)

    # geometry of the overlap submesh on the device
    t1 = perf_counter()
    xi, wf = quadrature(dim, et)
    n_q = xi.shape[1]
    lid = np.full(n_nodes, -1, dtype=np.int64)
    lid[ov_nodes] = np.arange(ov_nodes.size)
    elem_ov = np.ascontiguousarray(lid[elem[:, ov_el]])
    n_ov = int(ov_el.size)
    n_int = n_ov * n_q
    _ensure_int32_capacity("n_int", n_int)
    dev = {}
    f64 = t.float64
    coord_ov = _lib.to_device(np.ascontiguousarray(coord[:, ov_nodes]), f64)
    elem_d = _lib.to_device(elem_ov, t.int64)
    dhat = _lib.to_device(np.ascontiguousarray(reference_gradients(dim, et)), f64)
    wf_d = _lib.to_device(np.asarray(wf, dtype=np.float64), f64)
    dev["dphi1"] = t.empty((n_int, n_p), dtype=f64, device="cuda")
    dev["dphi2"] = t.empty((n_int, n_p), dtype=f64, device="cuda")
    dev["dphi3"] = t.empty((n_int, n_p) if dim == 3 else (1, 1), dtype=f64, device="cuda")
    dev["weight"] = t.empty(n_int, dtype=f64, device="cuda")
    _lib.call("ssp_geometry", dim, _lib.ptr(coord_ov), _lib.ptr(elem_d), _lib.ptr(dhat), _lib.ptr(wf_d),
              int(ov_nodes.size), n_ov, n_p, n_q, _lib.ptr(dev["dphi1"]), _lib.ptr(dev["dphi2"]),
              _lib.ptr(dev["dphi3"]) if dim == 3 else None, _lib.ptr(dev["weight"]), _lib.stream_handle())
    del coord_ov, elem_d
    owned_el = owned_element_mask(elem, ov_el, (n0, n1))
    if not owned_el.all():
        # the overlap elements whose smallest node the range owns: over the ranks they partition
        # the mesh, so the ranks' integrated potential energies add up to the whole mesh's
        dev["energy_weight"] = dev["weight"] * _lib.to_device(np.repeat(owned_el.astype(np.float64), n_q), f64)
    if dim == 3 and n_ov:
        # J^{-1} of every overlap element from its vertices, J = [x1 - x0, x2 - x0, x3 - x0] (the
        # mixed form's affine strain and force use it where the elements are straight-sided)
        xv = coord[:, elem[:4, ov_el]]  # (3, 4, n_ov)
        J = np.transpose(xv[:, 1:4, :] - xv[:, :1, :], (2, 0, 1))  # (n_ov, 3, 3): J[e, i, j] = x_{j+1,i} - x_{0,i}
        dev["jinv"] = _lib.to_device(np.ascontiguousarray(np.linalg.inv(J).reshape(n_ov, 9)), f64)
    timings["overlap_geometry_s"] = perf_counter() - t1

    t2 = perf_counter()
    dev["dof_lids"] = _lib.to_device(g["overlap_element_dof_lids"], t.int32)
    dev["scatter_map"] = _lib.to_device(g["scatter_map"], t.int32)
    dev["elem_row"] = _lib.to_device(g["elem_row"], t.int32)
    dev["cdiag"] = _lib.to_device(g["constrained_diag_positions"], t.int32)
    owned_free_rows = np.flatnonzero(owned_free).astype(np.int64)
    dev["owned_free_rows"] = _lib.to_device(owned_free_rows.astype(np.int32), t.int32)
    overlap_global_dofs = (dim * np.repeat(ov_nodes, dim) + np.tile(np.arange(dim), ov_nodes.size)).astype(np.int64)
    _ensure_int32_capacity("global dofs", dim * n_nodes)
    dev["overlap_global_dofs32"] = _lib.to_device(overlap_global_dofs.astype(np.int32), t.int32)
    # the same dofs as indices into U stored (dim, n_nodes) row-major: comp * n_nodes + node
    dev["overlap_dofs_rowmajor32"] = _lib.to_device(
        ((overlap_global_dofs % dim) * n_nodes + overlap_global_dofs // dim).astype(np.int32), t.int32)
    if keep_slot_metadata and dim == 3:
        dev["row_slot_ptr"] = _lib.to_device(g["row_slot_ptr"], t.int32)
        dev["slot_elem"] = _lib.to_device(g["slot_elem"], t.int32)
        dev["slot_lrow"] = _lib.to_device(g["slot_lrow"], t.uint8)
        dev["slot_pos"] = _lib.to_device(g["slot_pos"], t.int32)

    # elastic values: owned rows of K_elast on the pattern, constrained diagonals = 1
    if elastic_rows is not None and tuple(int(v) for v in elastic_rows.owned_node_range) != (n0, n1):
        raise ValueError("Prebuilt elastic_rows owned_node_range does not match prepare_owned_tangent_pattern request")
    if elastic_rows is not None and isinstance(elastic_rows, OwnedTangentPattern):
        dev["elastic_values"] = elastic_rows.device["elastic_values"]
        reused = True
    elif elastic_rows is not None:  # the reference's OwnedElasticRows: its assembled rows, projected
        vals = _project_values_onto_pattern(elastic_rows.local_matrix, g["indptr"], g["indices"], dim * n_nodes)
        dev["elastic_values"] = _lib.to_device(vals, f64)
        reused = True
    else:
        _c0, _phi, _psi, shear, bulk, lame, _gamma = heterogenous_materials(
            np.asarray(material_identifier, dtype=np.int64).ravel()[ov_el], np.ones(n_int, dtype=bool), n_q, materials)
        ds_el = _elastic_ds_device(t, dim, _lib.to_device(shear, f64), _lib.to_device(bulk, f64), _lib.to_device(lame, f64))
        vals = t.empty(nnz, dtype=f64, device="cuda")
        _lib.call("ssp_tangent_element", dim, 1, _lib.ptr(dev["dphi1"]), _lib.ptr(dev["dphi2"]),
                  _lib.ptr(dev["dphi3"]) if dim == 3 else None, _lib.ptr(ds_el), _lib.ptr(dev["weight"]),
                  _lib.ptr(dev["scatter_map"]), n_ov, n_p, n_q, nnz, _lib.ptr(vals), 0, _lib.stream_handle())
        _lib.call("ssp_finish_values", _lib.ptr(vals), nnz, _lib.ptr(dev["cdiag"]), int(dev["cdiag"].numel()), None, 0.0,
                  _lib.stream_handle())
        dev["elastic_values"] = vals
        reused = False
    t.cuda.synchronize()
    _lib.raise_on_device_status()
    timings["scatter_map_s"] = perf_counter() - t2

    local_int_indices = (ov_el[:, None] * n_q + np.arange(n_q)[None, :]).reshape(-1)
    if include_unique:
        owners = np.min(elem, axis=0)
        unique_elements = np.flatnonzero((owners >= n0) & (owners < n1)).astype(np.int64)
        unique_nodes = (np.unique(elem[:, unique_elements]) if unique_elements.size else np.empty(0, np.int64)).astype(np.int64)
        unique_local_int_indices = (unique_elements[:, None] * n_q + np.arange(n_q)[None, :]).reshape(-1)
    else:
        unique_elements = unique_nodes = unique_local_int_indices = np.empty(0, dtype=np.int64)

    pattern_matrix = csr_matrix((np.ones(nnz), g["indices"], g["indptr"]), shape=(n_rows, dim * n_nodes))
    overlap_B = None
    if include_overlap_B:
        overlap_B = _strain_operator(dim, [dev[k].cpu().numpy() for k in ("dphi1", "dphi2", "dphi3")[:dim]], elem_ov,
                                     n_q, int(ov_nodes.size))
    n_ld = dim * n_p
    scatter_host = g["scatter_map"] if include_legacy_scatter else np.empty((n_ov, 0), dtype=np.int32)
    empty_i32 = np.empty(0, dtype=np.int32)
    pat = OwnedTangentPattern(
        dim=dim, n_strain=6 if dim == 3 else 3, owned_node_range=(n0, n1), owned_row_range=(dim * n0, dim * n1),
        overlap_nodes=ov_nodes, overlap_elements=ov_el, overlap_global_dofs=overlap_global_dofs, overlap_B=overlap_B,
        overlap_element_dof_lids=g["overlap_element_dof_lids"], owned_local_overlap_dofs=g["owned_local_overlap_dofs"],
        owned_free_mask=owned_free, owned_free_local_rows=owned_free_rows,
        global_free_size=int(np.count_nonzero(q_mask)), local_matrix_pattern=pattern_matrix,
        local_int_indices=local_int_indices, unique_nodes=unique_nodes, unique_elements=unique_elements,
        unique_local_int_indices=unique_local_int_indices, scatter_map=scatter_host,
        row_slot_ptr=g.get("row_slot_ptr", empty_i32), slot_elem=g.get("slot_elem", empty_i32),
        slot_lrow=g.get("slot_lrow", np.empty(0, np.uint8)), slot_pos=g.get("slot_pos", np.empty((0, n_ld), np.int32)),
        constrained_diag_positions=g["constrained_diag_positions"], n_p=n_p, n_q=n_q, elem_type=et, device=dev,
    )
    pat.stats.update({
        "scatter_bytes": float(scatter_host.nbytes),
        "row_slot_bytes": float(sum(np.asarray(g[k]).nbytes for k in ("row_slot_ptr", "slot_elem", "slot_lrow", "slot_pos")
                                    if k in g)),
        "overlap_B_bytes": float(0 if overlap_B is None else
                                 overlap_B.data.nbytes + overlap_B.indices.nbytes + overlap_B.indptr.nbytes),
        "unique_B_bytes": 0.0,
        "dphi_bytes": float(sum(dev[k].numel() * 8 for k in ("dphi1", "dphi2", "dphi3"))),
        "device_bytes": float(sum(v.numel() * v.element_size() for v in dev.values())),
        "avg_active_rows_per_overlap_element": float((g["elem_row"] >= 0).sum(axis=1).mean()) if n_ov else 0.0,
        "max_active_rows_per_overlap_element": float((g["elem_row"] >= 0).sum(axis=1).max()) if n_ov else 0.0,
        "legacy_scatter_enabled": float(bool(include_legacy_scatter)),
    })
    timings["elastic_pattern_reused"] = float(reused)
    timings["scatter_missing_entries"] = 0.0
    pat.timings.update(timings)
    pat.__dict__["_include_legacy_scatter"] = bool(include_legacy_scatter)
    return pat


# ----------------------------------------------------------------------------- assembly


def _is_torch(a) -> bool:
    t = _lib.torch()
    return isinstance(a, t.Tensor)


def _u_overlap_device(pattern, U):
    """U as (dim, n_nodes) array / tensor (or flat Fortran vector) -> overlap dof values on device."""
    t = _lib.require_cuda()
    # a (dim, n_nodes) field is uploaded as stored (row-major, asynchronously when it is pinned)
    # and gathered by row-major indices on the device; a flat vector is in dof order
    if _is_torch(U):
        u = U if U.dtype == t.float64 else U.to(t.float64)
        rowmajor = u.dim() == 2
        u = u.contiguous()
        u_flat = u.to("cuda", non_blocking=True).reshape(-1)
    else:
        a = np.asarray(U, dtype=np.float64)
        rowmajor = a.ndim == 2
        u_flat = _lib.to_device(a if rowmajor else a.reshape(-1), t.float64).reshape(-1)
    idx = pattern.device["overlap_dofs_rowmajor32" if rowmajor else "overlap_global_dofs32"]
    u_ov = t.empty(idx.numel(), dtype=t.float64, device="cuda")
    _lib.call("ssp_gather", _lib.ptr(u_flat.contiguous()), _lib.ptr(idx), int(idx.numel()), _lib.ptr(u_ov),
              _lib.stream_handle())
    return u_ov


def _split_pairs(x, scale=None, group: int = 1):
    """hi + lo float pairs of an FP64 CUDA tensor (ssp_split_f64), flat float32 (2 per value)."""
    t = _lib.require_cuda()
    out = t.empty(2 * x.numel(), dtype=t.float32, device="cuda")
    _lib.call("ssp_split_f64", _lib.ptr(x), _lib.ptr(scale) if scale is not None else None, int(x.numel()), int(group),
              _lib.ptr(out), _lib.stream_handle())
    return out


def _affine_elements(pattern, rtol: float = 1e-10, chunk: int = 1 << 16) -> bool:
    """Whether every overlap element's gradients are J^{-T} ghat(q) (straight-sided tetrahedra):
    the stored dphi against the reconstruction from J^{-1} and the reference table, per element,
    relative to the element's largest gradient."""
    t = _lib.torch()
    d = pattern.device
    if pattern.dim != 3 or "jinv" not in d:
        return False
    n_el, n_q, n_p = int(pattern.overlap_elements.size), pattern.n_q, pattern.n_p
    ghat = t.as_tensor(np.ascontiguousarray(np.transpose(reference_gradients(3, pattern.elem_type), (2, 1, 0))),
                       device="cuda")  # (n_q, n_p, 3): [q][a][k]
    for e0 in range(0, n_el, chunk):
        e1 = min(n_el, e0 + chunk)
        jinv = d["jinv"][e0:e1].reshape(-1, 3, 3)  # [e][k][j]
        rec = t.einsum("ekj,qak->eqaj", jinv, ghat)  # dphi_j of node a at point q
        stored = t.stack([d[k][e0 * n_q:e1 * n_q].reshape(e1 - e0, n_q, n_p) for k in ("dphi1", "dphi2", "dphi3")], -1)
        scale = stored.abs().amax(dim=(1, 2, 3))
        if bool(((rec - stored).abs().amax(dim=(1, 2, 3)) > rtol * scale).any()):
            return False
    return True


def owned_element_mask(elem, overlap_elements, owned_node_range) -> np.ndarray:
    """Which overlap elements the owned node range owns: those whose smallest node lies in it
    (the BDDC subdomains' rule, distributed_tangent.py:481-623).  Over ranks whose node ranges
    partition the nodes, the owned elements partition the mesh; the potential energy sums over
    them."""
    n0, n1 = (int(v) for v in owned_node_range)
    ov = np.asarray(overlap_elements, dtype=np.int64)
    if ov.size == 0:
        return np.zeros(0, dtype=bool)
    owner = np.asarray(elem)[:, ov].min(axis=0)
    return (owner >= n0) & (owner < n1)


def _p2_affine_inputs(pattern):
    """The device arrays with J^{-1} per element and the quadrature points' barycentric
    coordinates when the pattern is 3D P2 and every element is affine to rounding, else None.
    Affine to rounding: the stored (isoparametric) gradients and J^{-T} ghat agree within 1e-12 of
    the element's largest gradient -- the rounding of the isoparametric gradients of straight-sided
    elements reaches 5e-14 on the 100k-element slope mesh and 1.4e-13 on the 2M-element one, while a
    mid-edge node moved off its edge by d shows as ~d/h.  Checked once per pattern."""
    d = pattern.device
    if pattern.affine_p2 is None:
        ok = pattern.dim == 3 and pattern.n_p == 10 and "jinv" in d and _affine_elements(pattern, rtol=1e-12)
        if ok:
            xi, _ = quadrature(3, pattern.elem_type)
            bary = np.ascontiguousarray(np.vstack([1.0 - xi[0] - xi[1] - xi[2], xi]).T)  # (n_q, 4)
            d["bary"] = _lib.to_device(bary, _lib.torch().float64)
        pattern.affine_p2 = bool(ok)
    return d if pattern.affine_p2 else None


def _affine_fp64_inputs(pattern):
    """The device arrays with J^{-1} per element and the reference gradient table (FP64) when the
    pattern is 3D P1 or P4 and every element is affine to rounding (the criterion of
    _p2_affine_inputs), else None.  Checked once per pattern."""
    d = pattern.device
    if pattern.affine_fp64 is None:
        ok = pattern.dim == 3 and pattern.n_p != 10 and "jinv" in d and _affine_elements(pattern, rtol=1e-12)
        if ok:
            table = np.ascontiguousarray(np.transpose(reference_gradients(3, pattern.elem_type), (2, 1, 0)))
            d["ghat"] = _lib.to_device(table, _lib.torch().float64)  # [n_q][n_p][3]
        pattern.affine_fp64 = bool(ok)
    return d if pattern.affine_fp64 else None


def _mixed_inputs(pattern):
    """Per-pattern hi + lo pairs of the mixed form's constant inputs, split once and kept with the
    pattern's device arrays: of the gradients and w * gradient, or, when every element is affine,
    of J^{-1} per element, the reference gradient table and the weights."""
    d = pattern.device
    if pattern.affine is None:
        pattern.affine = _affine_elements(pattern)
        if pattern.affine:
            t = _lib.torch()
            table = np.ascontiguousarray(np.transpose(reference_gradients(3, pattern.elem_type), (2, 1, 0)))
            d["ghat_hl"] = _split_pairs(t.as_tensor(table, device="cuda"))
            d["jinv_hl"] = _split_pairs(d["jinv"])
            d["w_hl"] = _split_pairs(d["weight"])
            if pattern.n_p == 10:  # P2: the barycentric form reads the points' barycentric coordinates
                xi, _ = quadrature(3, pattern.elem_type)
                bary = np.ascontiguousarray(np.vstack([1.0 - xi[0] - xi[1] - xi[2], xi]).T)
                d["bary_hl"] = _split_pairs(t.as_tensor(bary, device="cuda"))
        else:
            for k in ("dphi1", "dphi2", "dphi3"):
                d[k + "_hl"] = _split_pairs(d[k])
                d["w" + k + "_hl"] = _split_pairs(d[k], d["weight"], pattern.n_p)
    return d


def overlap_strain_device(pattern, U, *, mixed: bool = False):
    """E of every overlap point as an AoS (n_int, n_strain) CUDA tensor; mixed (3D): the
    compensated FP32 kernel of the mixed-precision form."""
    t = _lib.require_cuda()
    u_ov = _u_overlap_device(pattern, U)
    n_int = pattern.n_local_int
    n_el = int(pattern.overlap_elements.size)
    d = pattern.device
    E = t.empty((n_int, pattern.n_strain), dtype=t.float64, device="cuda")
    st = _lib.stream_handle()
    if pattern.dim == 3 and mixed:
        d = _mixed_inputs(pattern)
        u_hl = _split_pairs(u_ov)
        if pattern.affine and pattern.n_p == 10:
            _lib.call("ssp_assemble_overlap_strain_3d_p2_affine_mixed", _lib.ptr(d["jinv_hl"]), _lib.ptr(d["bary_hl"]),
                      _lib.ptr(u_hl), int(u_ov.numel()), _lib.ptr(d["dof_lids"]), n_int, n_el, pattern.n_q,
                      _lib.ptr(E), st)
        elif pattern.affine:
            _lib.call("ssp_assemble_overlap_strain_3d_affine_mixed", _lib.ptr(d["jinv_hl"]), _lib.ptr(d["ghat_hl"]),
                      _lib.ptr(u_hl), int(u_ov.numel()), _lib.ptr(d["dof_lids"]), n_int, n_el, pattern.n_p,
                      pattern.n_q, _lib.ptr(E), st)
        else:
            _lib.call("ssp_assemble_overlap_strain_3d_mixed", _lib.ptr(d["dphi1_hl"]), _lib.ptr(d["dphi2_hl"]),
                      _lib.ptr(d["dphi3_hl"]), _lib.ptr(u_hl), int(u_ov.numel()), _lib.ptr(d["dof_lids"]), n_int, n_el,
                      pattern.n_p, pattern.n_q, _lib.ptr(E), st)
    elif pattern.dim == 3 and _p2_affine_inputs(pattern) is not None:
        _lib.call("ssp_assemble_overlap_strain_3d_p2_affine", _lib.ptr(d["jinv"]), _lib.ptr(d["bary"]), _lib.ptr(u_ov),
                  int(u_ov.numel()), _lib.ptr(d["dof_lids"]), n_int, n_el, pattern.n_q, _lib.ptr(E), st)
    elif pattern.dim == 3 and _affine_fp64_inputs(pattern) is not None:
        _lib.call("ssp_assemble_overlap_strain_3d_affine", _lib.ptr(d["jinv"]), _lib.ptr(d["ghat"]), _lib.ptr(u_ov),
                  int(u_ov.numel()), _lib.ptr(d["dof_lids"]), n_int, n_el, pattern.n_p, pattern.n_q, _lib.ptr(E), st)
    elif pattern.dim == 3:
        _lib.call("ssp_assemble_overlap_strain_3d", _lib.ptr(d["dphi1"]), _lib.ptr(d["dphi2"]), _lib.ptr(d["dphi3"]),
                  _lib.ptr(u_ov), int(u_ov.numel()), _lib.ptr(d["dof_lids"]), n_int, n_el, pattern.n_p, pattern.n_q,
                  _lib.ptr(E), st)
    else:
        _lib.call("ssp_assemble_overlap_strain_2d", _lib.ptr(d["dphi1"]), _lib.ptr(d["dphi2"]), _lib.ptr(u_ov),
                  int(u_ov.numel()), _lib.ptr(d["dof_lids"]), n_int, n_el, pattern.n_p, pattern.n_q, _lib.ptr(E), st)
    return E


def assemble_overlap_strain(pattern: OwnedTangentPattern, U, *, use_compiled: bool = True):
    """Strain of every overlap integration point, shape (n_strain, n_int_local)."""
    E = overlap_strain_device(pattern, U)
    if _is_torch(U):
        return E.T
    out = E.cpu().numpy().T
    _lib.raise_on_device_status()
    return out


def _local_field_aos(pattern, field, rows: int):
    """(rows, n_int) host array / tensor, or (rows, n_int_global) with local_int_indices -> AoS CUDA tensor."""
    t = _lib.require_cuda()
    n_loc = pattern.n_local_int
    if _is_torch(field):
        f = field.to(t.float64).cuda()
    else:
        f = np.asarray(field, dtype=np.float64)
    if f.ndim != 2 or f.shape[0] != rows:
        raise ValueError(f"expected shape ({rows}, n_int)")
    if f.shape[1] != n_loc:
        idx = pattern.local_int_indices
        f = f[:, t.as_tensor(idx, device=f.device) if _is_torch(f) else idx]
    if _is_torch(f):
        return f.T.contiguous()
    return _lib.to_device(np.ascontiguousarray(f.T), t.float64)


def owned_force_device(pattern, S_aos, *, mixed: bool = False):
    """Owned internal force B^T (w S) on owned rows (constrained rows = 0), CUDA tensor (n_rows,);
    mixed (3D): the compensated FP32 kernel of the mixed-precision form."""
    t = _lib.require_cuda()
    d = pattern.device
    n_rows = int(pattern.local_matrix_pattern.shape[0])
    F = t.empty(n_rows, dtype=t.float64, device="cuda")
    if mixed and pattern.dim == 3:
        d = _mixed_inputs(pattern)
        if pattern.affine and pattern.n_p == 10:
            _lib.call("ssp_assemble_force_element_p2_affine_mixed", _lib.ptr(d["jinv_hl"]), _lib.ptr(d["bary_hl"]),
                      _lib.ptr(d["w_hl"]), _lib.ptr(S_aos), _lib.ptr(d["elem_row"]), int(pattern.overlap_elements.size),
                      pattern.n_q, n_rows, _lib.ptr(F), _lib.stream_handle())
        elif pattern.affine:
            _lib.call("ssp_assemble_force_element_affine_mixed", _lib.ptr(d["jinv_hl"]), _lib.ptr(d["ghat_hl"]),
                      _lib.ptr(d["w_hl"]), _lib.ptr(S_aos), _lib.ptr(d["elem_row"]), int(pattern.overlap_elements.size),
                      pattern.n_p, pattern.n_q, n_rows, _lib.ptr(F), _lib.stream_handle())
        else:
            _lib.call("ssp_assemble_force_element_mixed", _lib.ptr(d["wdphi1_hl"]), _lib.ptr(d["wdphi2_hl"]),
                      _lib.ptr(d["wdphi3_hl"]), _lib.ptr(S_aos), _lib.ptr(d["elem_row"]),
                      int(pattern.overlap_elements.size), pattern.n_p, pattern.n_q, n_rows, _lib.ptr(F),
                      _lib.stream_handle())
        return F
    if pattern.dim == 3 and _p2_affine_inputs(pattern) is not None:
        _lib.call("ssp_assemble_force_element_p2_affine", _lib.ptr(d["jinv"]), _lib.ptr(d["bary"]), _lib.ptr(S_aos),
                  _lib.ptr(d["weight"]), _lib.ptr(d["elem_row"]), int(pattern.overlap_elements.size), pattern.n_q,
                  n_rows, _lib.ptr(F), _lib.stream_handle())
        return F
    if pattern.dim == 3 and _affine_fp64_inputs(pattern) is not None:
        _lib.call("ssp_assemble_force_element_affine", _lib.ptr(d["jinv"]), _lib.ptr(d["ghat"]), _lib.ptr(S_aos),
                  _lib.ptr(d["weight"]), _lib.ptr(d["elem_row"]), int(pattern.overlap_elements.size), pattern.n_p,
                  pattern.n_q, n_rows, _lib.ptr(F), _lib.stream_handle())
        return F
    _lib.call("ssp_assemble_force_element", pattern.dim, _lib.ptr(d["dphi1"]), _lib.ptr(d["dphi2"]),
              _lib.ptr(d["dphi3"]) if pattern.dim == 3 else None, _lib.ptr(S_aos), _lib.ptr(d["weight"]),
              _lib.ptr(d["elem_row"]), int(pattern.overlap_elements.size), pattern.n_p, pattern.n_q, n_rows,
              _lib.ptr(F), _lib.stream_handle())
    return F


def owned_force_rows_device(pattern, S_aos):
    """Same as owned_force_device through the reference's row-slot gather (3D only)."""
    t = _lib.require_cuda()
    d = pattern.device
    if pattern.dim != 3 or "row_slot_ptr" not in d:
        raise ValueError("row-slot force needs a 3D pattern prepared with keep_slot_metadata=True")
    n_rows = int(pattern.local_matrix_pattern.shape[0])
    F = t.empty(n_rows, dtype=t.float64, device="cuda")
    _lib.call("ssp_assemble_force_3d_rows", _lib.ptr(d["dphi1"]), _lib.ptr(d["dphi2"]), _lib.ptr(d["dphi3"]),
              _lib.ptr(S_aos), _lib.ptr(d["weight"]), _lib.ptr(d["row_slot_ptr"]), _lib.ptr(d["slot_elem"]),
              _lib.ptr(d["slot_lrow"]), pattern.n_local_int, n_rows, int(d["slot_elem"].numel()), pattern.n_p,
              pattern.n_q, _lib.ptr(F), _lib.stream_handle())
    F[~t.as_tensor(pattern.owned_free_mask, device="cuda")] = 0.0
    return F


def assemble_owned_force_from_local_stress(pattern: OwnedTangentPattern, stress_local, *, use_compiled: bool = True):
    if np.shape(stress_local)[0] != int(pattern.n_strain):
        raise ValueError(f"stress_local must have shape ({int(pattern.n_strain)}, n_int_local)")
    S = _local_field_aos(pattern, stress_local, pattern.n_strain)
    F = owned_force_device(pattern, S)
    if _is_torch(stress_local):
        return F
    out = F.cpu().numpy()
    _lib.raise_on_device_status()
    return out


def tangent_values_device(pattern, DS_aos, *, kernel: str = DEFAULT_TANGENT_KERNEL, symmetric: bool = False,
                          out=None, finish: bool = True):
    """CSR values of the owned tangent rows (constrained diagonals = 1 when finish) as a CUDA tensor."""
    t = _lib.require_cuda()
    k = _normalize_tangent_kernel(kernel)
    d = pattern.device
    nnz = pattern.nnz
    if k == "legacy" and not pattern.__dict__.get("_include_legacy_scatter", True) and pattern.overlap_elements.size:
        raise ValueError("Legacy tangent kernel requires scatter_map; prepare the pattern with include_legacy_scatter=True")
    vals = out if out is not None else t.empty(nnz, dtype=t.float64, device="cuda")
    st = _lib.stream_handle()
    n_el = int(pattern.overlap_elements.size)
    if k == "rows_gather":
        if pattern.dim != 3 or "row_slot_ptr" not in d:
            raise ValueError("rows_gather needs a 3D pattern prepared with keep_slot_metadata=True")
        _lib.call("ssp_assemble_tangent_values_3d_rows", _lib.ptr(d["dphi1"]), _lib.ptr(d["dphi2"]), _lib.ptr(d["dphi3"]),
                  _lib.ptr(DS_aos), _lib.ptr(d["weight"]), _lib.ptr(d["row_slot_ptr"]), _lib.ptr(d["slot_elem"]),
                  _lib.ptr(d["slot_lrow"]), _lib.ptr(d["slot_pos"]), pattern.n_local_int,
                  int(pattern.local_matrix_pattern.shape[0]), int(d["slot_elem"].numel()), pattern.n_p, pattern.n_q, nnz,
                  _lib.ptr(vals), st)
    else:
        _lib.call("ssp_tangent_element", pattern.dim, 1 if symmetric else 0, _lib.ptr(d["dphi1"]), _lib.ptr(d["dphi2"]),
                  _lib.ptr(d["dphi3"]) if pattern.dim == 3 else None, _lib.ptr(DS_aos), _lib.ptr(d["weight"]),
                  _lib.ptr(d["scatter_map"]), n_el, pattern.n_p, pattern.n_q, nnz, _lib.ptr(vals), 0, st)
    if finish:
        _lib.call("ssp_finish_values", _lib.ptr(vals), nnz, _lib.ptr(d["cdiag"]), int(d["cdiag"].numel()), None, 0.0, st)
    return vals


def assemble_owned_tangent_values(pattern: OwnedTangentPattern, DS, *, use_compiled: bool = True,
                                  kernel: str = DEFAULT_TANGENT_KERNEL):
    """Assemble tangent values on the fixed owned-row CSR pattern."""
    _normalize_tangent_kernel(kernel)
    ns2 = int(pattern.n_strain * pattern.n_strain)
    shp = tuple(DS.shape) if hasattr(DS, "shape") else np.shape(DS)
    if len(shp) != 2 or shp[0] != ns2:
        raise ValueError(f"DS must have shape ({ns2}, n_int) for owned tangent assembly")
    from .arrays import DeviceArray

    if isinstance(DS, DeviceArray):
        ds_aos, as_torch = DS.aos, False
    else:
        ds_aos, as_torch = _local_field_aos(pattern, DS, ns2), _is_torch(DS)
    vals = tangent_values_device(pattern, ds_aos, kernel=kernel, symmetric=False)
    if as_torch:
        return vals
    out = vals.cpu().numpy()
    _lib.raise_on_device_status()
    return out


def assemble_owned_tangent_matrix(pattern: OwnedTangentPattern, DS, *, use_compiled: bool = True,
                                  kernel: str = DEFAULT_TANGENT_KERNEL) -> csr_matrix:
    values = np.asarray(assemble_owned_tangent_values(pattern, DS, kernel=kernel), dtype=np.float64)
    lp = pattern.local_matrix_pattern
    return csr_matrix((values.copy(), lp.indices.copy(), lp.indptr.copy()), shape=lp.shape)


def assemble_owned_regularized_matrix(pattern: OwnedTangentPattern, DS, r: float, *, use_compiled: bool = True,
                                      kernel: str = DEFAULT_TANGENT_KERNEL) -> csr_matrix:
    """Owned rows of K_r = r*K_elast + (1-r)*K_tangent on the fixed pattern."""
    t = _lib.require_cuda()
    ns2 = int(pattern.n_strain * pattern.n_strain)
    vals = tangent_values_device(pattern, _local_field_aos(pattern, DS, ns2), kernel=kernel)
    _lib.call("ssp_finish_values", _lib.ptr(vals), pattern.nnz, None, 0, _lib.ptr(pattern.device["elastic_values"]),
              float(r), _lib.stream_handle())
    values = vals.cpu().numpy()
    _lib.raise_on_device_status()
    lp = pattern.local_matrix_pattern
    return csr_matrix((values, lp.indices.copy(), lp.indptr.copy()), shape=lp.shape)


_BDDC_NAMES = ("BDDCSubdomainPattern", "prepare_bddc_subdomain_pattern", "assemble_bddc_subdomain_tangent_values")


def __getattr__(name):
    # the subdomain (BDDC) half of the reference module lives in .bddc, which imports this module
    if name in _BDDC_NAMES:
        from . import bddc

        return getattr(bddc, name)
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")
