"""``ConstitutiveOperator``: the reference's constitutive builder, with the hot path on the GPU.

Drop-in for ``src/slope_stability/constitutive/problem.py:1192-2210``.  Newton, damping and the
continuation drivers talk to the builder only through the method names below (they probe them
with ``getattr`` and ``owned_tangent_pattern is not None``, nonlinear/newton.py:290-336); every
one of them is provided with the reference's semantics:

* ``reduction(lam)`` -> Davis-reduced ``c_bar``/``sin_phi`` per local point (CUDA kernel);
* ``constitutive_problem_stress(U)`` / ``constitutive_problem_stress_tangent(U)`` -> strain
  kernel + return-mapping kernel; S and DS stay in HBM (``_owned_local_S``/``_owned_local_DS``
  are ``DeviceArray`` views that convert to NumPy on demand);
* ``build_F*`` -> owned internal force (element kernel), returned as NumPy like the reference;
* ``build_K_regularized(r)`` / ``build_F_K_*`` -> tangent CSR values on the fixed pattern,
  constrained diagonals, the regularised blend, and an in-place update of one stable matrix
  object (a PETSc AIJ matrix when petsc4py is importable, otherwise ``OwnedCSRMatrix``);
* ``get_total_time()`` with the reference's keys, ``release_petsc_caches()``,
  ``set_owned_tangent_pattern(...)``.

Only the owned-pattern path exists (it is the reference's production path).  An operator without
a pattern raises on the first hot-path call; ``ConstitutiveOperator.from_mesh`` builds one with
the whole mesh owned.  Constitutive modes ``overlap``, ``unique_gather`` and ``unique_exchange``
coincide on one device (they differ only in MPI traffic) and all run the overlap kernels.
"""

from __future__ import annotations

from dataclasses import dataclass
from time import perf_counter
from typing import Any

import numpy as np
from scipy.sparse import csr_matrix

from . import _lib
from .arrays import DeviceArray
from .distributed_tangent import (
    DEFAULT_TANGENT_KERNEL,
    OwnedTangentPattern,
    _normalize_tangent_kernel,
    _p2_affine_inputs,
    overlap_strain_device,
    owned_force_device,
    prepare_owned_tangent_pattern,
    tangent_values_device,
)

try:  # pragma: no cover - PETSc is absent in most environments of this package
    from petsc4py import PETSc
except Exception:  # pragma: no cover
    PETSc = None

_OWNED_MODES = {"overlap", "unique_exchange", "unique", "unique_gather", "no_overlap", "partitioned"}
# (dim, nodes per element) with a mixed-precision plastic-correction kernel (CUDA-core warp kernel
# for the triangles and P1/P2 tets, tcgen05 tensor-core kernel for P4 tets)
MIXED_TANGENT_ELEMENTS = {(2, 3), (2, 6), (2, 15), (3, 4), (3, 10), (3, 35)}


class OwnedCSRMatrix:
    """Owned-row CSR matrix on the fixed pattern, updated in place (stable ``handle``).

    ``values`` is the CUDA tensor the kernels write; ``data`` is a pinned host mirror refreshed by
    ``sync_host()`` (what a PETSc ``setValuesCSR`` would read, utils.py:288-306).  The device ->
    host copy runs on a side stream, so the caller's stream can go on (the operator computes the
    internal force meanwhile); ``getValuesCSR`` / ``to_scipy`` wait for it, and ``fence()`` makes
    the current stream wait for it before the values are overwritten."""

    _next_handle = 1

    def __init__(self, pattern: OwnedTangentPattern, values):
        self.indptr = np.asarray(pattern.local_matrix_pattern.indptr, dtype=np.int32)
        self.indices = np.asarray(pattern.local_matrix_pattern.indices, dtype=np.int32)
        self.shape = pattern.local_matrix_pattern.shape
        self.values = values
        t = _lib.torch()
        self._host = t.empty(values.numel(), dtype=t.float64, pin_memory=True)
        self.data = self._host.numpy()
        self._copy_stream = t.cuda.Stream()
        self._copied = None  # event recorded after the last host copy
        self._indptr_dev = t.as_tensor(self.indptr, device=values.device)  # for the row-wise refresh
        # which build the host mirror holds: (start key, build number) or None (unknown)
        self.mirror = None
        # blocks per SM of the row-wise host refresh (1..8): a part of each SM runs it beside the
        # internal force of the same iteration instead of ahead of it
        self.copy_share = 4
        self.handle = OwnedCSRMatrix._next_handle
        OwnedCSRMatrix._next_handle += 1

    def sync_host(self, stream=None, *, rows=None, mirror=None):
        """Refresh the pinned host mirror from the device values on a side stream.  rows: a device
        uint8 mark per CSR row; only the marked rows are stored (ssp_copy_rows_out), the caller
        having established that the other rows equal the mirror already.  mirror: the state the
        mirror holds afterwards."""
        t = _lib.torch()
        cur = t.cuda.current_stream()
        self._copy_stream.wait_stream(cur)
        with t.cuda.stream(self._copy_stream):
            if rows is not None:
                _lib.call("ssp_copy_rows_out_share", _lib.ptr(self.values), _lib.ptr(self._indptr_dev),
                          _lib.ptr(rows), int(self.shape[0]), int(self.values.numel()), self._host.data_ptr(),
                          int(self.copy_share), self._copy_stream.cuda_stream)
            else:
                self._host.copy_(self.values, non_blocking=True)
            self._copied = t.cuda.Event()
            self._copied.record(self._copy_stream)
        self.values.record_stream(self._copy_stream)
        self.mirror = mirror
        self._last_rows = rows
        return self

    def host_copy_bytes(self) -> int:
        """Bytes of CSR values the last sync_host moved to the host (synchronises)."""
        rows = getattr(self, "_last_rows", None)
        if rows is None:
            return 8 * int(self.values.numel())
        lengths = self._indptr_dev[1:] - self._indptr_dev[:-1]
        return 8 * int((lengths * rows[: lengths.numel()].to(lengths.dtype)).sum().item())

    def fence(self):
        """Make the current stream wait until the last host copy has read the values."""
        if self._copied is not None:
            _lib.torch().cuda.current_stream().wait_event(self._copied)

    def _wait(self):
        t = _lib.torch()
        t.cuda.current_stream().synchronize()
        if self._copied is not None:
            self._copied.synchronize()

    def getValuesCSR(self):
        self._wait()
        return self.indptr, self.indices, self.data

    def to_scipy(self) -> csr_matrix:
        self._wait()
        return csr_matrix((self.data.copy(), self.indices.copy(), self.indptr.copy()), shape=self.shape)

    def destroy(self):
        self.values = None


class SubdomainCSRMatrix(OwnedCSRMatrix):
    """Local square CSR of a BDDC subdomain, updated in place (stable ``handle``): what the
    reference passes to ``local_csr_to_petsc_matis_matrix`` (problem.py:1738-1749) -- the local
    values and pattern, the local-to-global dof map, the global size, block size, local vector size
    and the BDDC metadata (problem.py:1658-1708, without the PETSc objects)."""

    def __init__(self, pattern, values, *, global_size: int, block_size: int, metadata: dict):
        super().__init__(pattern, values)
        self.local_to_global = np.asarray(pattern.local_global_dofs, dtype=np.int64)
        self.global_size = int(global_size)
        self.block_size = int(block_size)
        self.local_vector_size = int(block_size * (pattern.owned_node_range[1] - pattern.owned_node_range[0]))
        self.metadata = metadata


class CapturedBuild:
    """A composite Newton build recorded as a CUDA graph (ConstitutiveOperator.capture_regularized_build)."""

    def __init__(self, graph, F, K, op):
        self.graph, self.F, self.K, self._op = graph, F, K, op
        # the graph addresses the operator's device buffers as they were at capture: hold them, so
        # a later change of the operator's configuration cannot free memory the graph still writes
        # (such a change needs a new capture to take effect)
        t = _lib.torch()
        keep, todo = [], [op.__dict__, getattr(op.owned_tangent_pattern, "device", {})]
        while todo:
            x = todo.pop()
            if isinstance(x, t.Tensor):
                keep.append(x)
            elif isinstance(x, dict):
                todo.extend(x.values())
            elif isinstance(x, (list, tuple)):
                todo.extend(x)
            elif isinstance(x, OwnedCSRMatrix):
                keep.append(x.values)
        self._buffers = keep

    def replay(self):
        """Re-run the recorded kernels on the current contents of U; returns (F, K)."""
        self.graph.replay()
        return self.F, self.K


@dataclass
class ConstitutiveOperator:
    B: Any
    c0: np.ndarray
    phi: np.ndarray
    psi: np.ndarray
    Davis_type: str
    shear: np.ndarray
    bulk: np.ndarray
    lame: np.ndarray
    WEIGHT: np.ndarray
    n_strain: int
    n_int: int
    dim: int
    q_mask: np.ndarray | None = None

    def __post_init__(self):
        for name in ("c0", "phi", "psi", "shear", "bulk", "lame", "WEIGHT"):
            setattr(self, name, np.asarray(getattr(self, name), dtype=np.float64))
        self.q_mask = None if self.q_mask is None else np.asarray(self.q_mask, dtype=bool)
        self.S = None
        self.DS = None
        self.c_bar = None
        self.sin_phi = None
        self.time_reduction = []
        self.time_stress = []
        self.time_stress_tangent = []
        self.time_build_F = []
        self.time_build_F_K_tangent = []
        self.time_potential = []
        self.time_build_tangent_local = []
        self.time_local_strain = []
        self.time_local_constitutive = []
        self.time_local_constitutive_comm = []
        self.time_local_force_assembly = []
        self.time_local_force_gather = []
        self.owned_tangent_pattern: OwnedTangentPattern | None = None
        self.bddc_subdomain_pattern = None
        self._bddc = {}  # BDDC subdomain matrices and value buffers, per kind
        self.use_compiled_owned_tangent = True
        self.owned_tangent_kernel = DEFAULT_TANGENT_KERNEL
        self.use_compiled_owned_constitutive = True
        self.owned_constitutive_mode = "global"
        # host (True) or device-resident (False) hand-off of F and K values
        self.host_outputs = True
        # list to collect (start, end) CUDA events around each tangent-kernel launch, or None
        self.tangent_events = None
        self._S_aos = None
        self._DS_aos = None
        self._ds_symmetric = False
        self._branch = None  # per-point return branch of the last tangent evaluation (int8, device)
        self._prev_branch = None  # branch codes of the last evaluation that produced them ("previous")
        # The screened 3D return mappings leave the DS rows of the points that return elastic
        # unwritten (they equal the elastic matrix, which the tangent's plastic corrections never
        # read); _owned_local_DS and every path that reads all rows fill them first (_complete_ds).
        self.lazy_elastic_ds = True
        self._ds_elastic_pending = False
        self._K_el = None  # elastic tangent CSR values (device), built on first use
        self._blend_base = None  # (r, (1-r) K_el,t + r K_el) for the last regularisation factor
        self._dev = None
        # composite regularised builds copy the tangent's starting values on a second stream while
        # the strain and return mapping run (_stage_values); (key, values, event) of that copy
        self.stage_values = True
        self._staged_values = None
        # how the tangent's starting values are copied: "kernel" (the library's SM copy; measured as
        # fast as a stream memcpy in direct calls and, unlike a memcpy node, no slower in a
        # captured graph) or "memcpy"
        self.values_copy = "kernel"
        # restore only the rows the previous build's plastic elements changed (same start values)
        self.incremental_values = True
        # host outputs: the pinned mirror of the values is refreshed row by row where the values
        # can have changed since the previous build (_changed_rows), else copied in full
        self.incremental_host_copy = True
        self._last_build = {}
        self._build_no = 0
        # How 3D tangents are evaluated (all give the same results): "binned" -- two passes with
        # exact branch binning; "unsorted" -- one pass in point order; "learned" -- points binned
        # by the branch_model's proposal, then the exact return mapping bin by bin; "previous" --
        # points binned by the previous evaluation's branch codes (the trivial predictor; the first
        # evaluation of a pattern runs "binned").
        self.return_mapping = "binned"
        self.branch_model = None
        self._scratch = None
        self._energy_scratch = None  # block partials + total of potential_energy
        # plain form on straight-sided P2 tetrahedra: elements with at least this many plastic points
        # get their correction in moment form (ssp_tangent_plastic_correction_p2_moments, fewer FP64
        # operations from five points up), the others point by point; 0 disables it.  The mixed form's
        # moment kernel (FP32 after the FP64 DS - D_el) costs less than its point-by-point kernel from
        # one plastic point up: every plastic element by default.
        self.moment_min_points = 5
        self.moment_min_points_mixed = 1
        # "plain": FP64 throughout (the drop-in, parity 1e-12 with the reference);
        # "mixed": the plastic-point tangent products in FP32 (CUDA cores for P1/P2, tensor cores
        # for P4) with H = w D B formed in compensated double-float arithmetic, and the 3D strain and
        # force in compensated double-float arithmetic (~1e-13); the return mapping and every CSR /
        # force accumulation stay FP64 (about 1e-7 relative tangent error)
        self.tangent_form = "plain"
        # composite builds with device outputs: True runs the force on the second stream at the same
        # time as the tangent; measured 2-5 % slower than one stream on the GB300 (the two compete
        # for the SMs), so off by default
        self.concurrent_force = False
        # blocks per SM of the staged row restore (1..8); None: chosen from the points per CSR entry
        self.restore_share = None
        self._force_stream = None
        self._owned_overlap_c_bar = None
        self._owned_overlap_sin_phi = None
        self._red_key = None
        self._owned_unique_c_bar = None
        self._owned_unique_sin_phi = None
        self._dev_mat = None
        self._owned_tangent_mat = None
        self._owned_regularized_mat = None
        self._tangent_values = None
        self._regularized_values = None
        self._force = None

    # -------------------------------------------------------------------- construction

    @classmethod
    def from_mesh(cls, coord, elem, q_mask, material_identifier, materials, *, elem_type="P2", Davis_type="B",
                  tangent_kernel=DEFAULT_TANGENT_KERNEL):
        """Operator plus an owned pattern covering the whole mesh (one device owns every row)."""
        from .materials import heterogenous_materials

        coord = np.asarray(coord, dtype=np.float64)
        elem = np.asarray(elem, dtype=np.int64)
        pat = prepare_owned_tangent_pattern(coord, elem, q_mask, material_identifier, materials, (0, coord.shape[1]),
                                            elem_type=elem_type, include_legacy_scatter=False, include_overlap_B=False,
                                            keep_slot_metadata=False)
        n_int = elem.shape[1] * pat.n_q
        c0, phi, psi, shear, bulk, lame, _g = heterogenous_materials(material_identifier, np.ones(n_int, bool), pat.n_q,
                                                                     materials)
        op = cls(B=None, c0=c0, phi=phi, psi=psi, Davis_type=Davis_type, shear=shear, bulk=bulk, lame=lame,
                 WEIGHT=np.zeros(0), n_strain=pat.n_strain, n_int=n_int, dim=pat.dim, q_mask=q_mask)
        op.set_owned_tangent_pattern(pat, tangent_kernel=tangent_kernel, constitutive_mode="overlap")
        return op

    def set_owned_tangent_pattern(self, pattern, *, use_compiled=True, tangent_kernel=DEFAULT_TANGENT_KERNEL,
                                  constitutive_mode="global", use_compiled_constitutive=True) -> None:
        self.owned_tangent_pattern = pattern
        self.use_compiled_owned_tangent = bool(use_compiled)
        self.owned_tangent_kernel = _normalize_tangent_kernel(tangent_kernel)
        self.use_compiled_owned_constitutive = bool(use_compiled_constitutive)
        self.owned_constitutive_mode = str(constitutive_mode).lower()
        self.release_petsc_caches()
        self._dev = None
        self._K_el = None
        self._blend_base = None
        self._staged_values = None
        self._last_build = {}
        self._red_key = None
        self._clear_owned_local_cache()
        self._prev_branch = None
        if pattern is not None:
            t = _lib.require_cuda()
            idx = np.asarray(pattern.local_int_indices, dtype=np.int64)
            pick = lambda a: _lib.to_device(np.ascontiguousarray(np.asarray(a, dtype=np.float64)[idx]), t.float64)  # noqa
            self._dev = {k: pick(getattr(self, k)) for k in ("c0", "phi", "psi", "shear", "bulk", "lame")}
            # The reduction of a point depends only on its (c0, phi, psi).  Soils come in a few
            # materials, so the distinct triples are reduced once and expanded to the points.
            trip = np.stack([np.asarray(getattr(self, k), dtype=np.float64)[idx] for k in ("c0", "phi", "psi")], axis=1)
            uniq, inv = np.unique(trip, axis=0, return_inverse=True)
            if uniq.shape[0] <= 4096:
                self._dev["red_unique"] = [_lib.to_device(np.ascontiguousarray(uniq[:, k]), t.float64) for k in range(3)]
                self._dev["red_index"] = _lib.to_device(inv.reshape(-1).astype(np.int32), t.int32)

    def set_bddc_subdomain_pattern(self, pattern) -> None:
        """Attach a BDDCSubdomainPattern (problem.py:1297-1298); its matrices are rebuilt on demand."""
        self.bddc_subdomain_pattern = pattern
        self._bddc = {}

    # -------------------------------------------------------------------- state views

    def _require_pattern(self) -> OwnedTangentPattern:
        if self.owned_tangent_pattern is None:
            raise RuntimeError("The GPU constitutive operator runs on an owned tangent pattern; call "
                               "set_owned_tangent_pattern() or build it with ConstitutiveOperator.from_mesh()")
        return self.owned_tangent_pattern

    def _use_owned_constitutive(self) -> bool:
        return self.owned_tangent_pattern is not None and str(self.owned_constitutive_mode).lower() != "global"

    @property
    def _owned_local_S(self):
        return None if self._S_aos is None else DeviceArray(self._S_aos)

    @_owned_local_S.setter
    def _owned_local_S(self, value):
        self._S_aos = self._ingest_field(value, self.n_strain)

    @property
    def _owned_local_DS(self):
        if self._DS_aos is None:
            return None
        self._complete_ds()
        return DeviceArray(self._DS_aos)

    @_owned_local_DS.setter
    def _owned_local_DS(self, value):
        self._DS_aos = self._ingest_field(value, self.n_strain * self.n_strain)
        self._ds_symmetric = False  # a caller-provided tangent is not known to be symmetric
        self._branch = None
        self._ds_elastic_pending = False

    def _complete_ds(self):
        """Write the DS rows the return mapping left out (lazy_elastic_ds): the rows of the points
        that returned elastic get the elastic matrix, bit for bit what the return mapping emits."""
        if not self._ds_elastic_pending or self._DS_aos is None:
            return
        pat = self._require_pattern()
        d = self._dev
        _lib.call("ssp_fill_elastic_ds", pat.dim, _lib.ptr(self._branch), _lib.ptr(d["shear"]), _lib.ptr(d["lame"]),
                  int(pat.n_local_int), _lib.ptr(self._DS_aos), _lib.stream_handle())
        self._ds_elastic_pending = False

    def _ingest_field(self, value, rows):
        if value is None:
            return None
        if isinstance(value, DeviceArray):
            return value.aos
        t = _lib.require_cuda()
        if isinstance(value, t.Tensor):
            return value.to(t.float64).cuda().T.contiguous()
        arr = np.asarray(value, dtype=np.float64)
        if arr.ndim != 2 or arr.shape[0] != rows:
            raise ValueError(f"expected a ({rows}, n_int) field")
        return _lib.to_device(np.ascontiguousarray(arr.T), t.float64)

    def _clear_owned_local_cache(self):
        self._S_aos = None
        self._DS_aos = None
        self._ds_symmetric = False
        self._branch = None
        self._ds_elastic_pending = False

    # -------------------------------------------------------------------- hot path

    def reduction(self, lam: float):
        t0 = perf_counter()
        pat = self._require_pattern()
        t = _lib.require_cuda()
        if not (float(lam) > 0.0):
            raise ValueError("Reduction parameter lambda must be positive")
        davis = str(self.Davis_type).upper()
        if davis not in ("A", "B", "C"):
            raise ValueError("Incorrect choice of the Davis approach")
        key = (float(lam), davis)
        if self._red_key == key and self._owned_overlap_c_bar is not None:
            # c_bar and sin_phi depend on (lambda, Davis type) and the materials only: Newton
            # iterations at one lambda reuse the arrays of the first
            self.time_reduction.append(perf_counter() - t0)
            return
        n = pat.n_local_int
        cb = t.empty(n, dtype=t.float64, device="cuda")
        sp = t.empty(n, dtype=t.float64, device="cuda")
        d = self._dev
        st = _lib.stream_handle()
        if "red_unique" in d:
            c0u, phu, psu = d["red_unique"]
            m = int(c0u.numel())
            cbu = t.empty(m, dtype=t.float64, device="cuda")
            spu = t.empty(m, dtype=t.float64, device="cuda")
            _lib.call("ssp_reduction", _lib.ptr(c0u), _lib.ptr(phu), _lib.ptr(psu), m, float(lam), davis.encode(),
                      _lib.ptr(cbu), _lib.ptr(spu), st)
            _lib.call("ssp_gather", _lib.ptr(cbu), _lib.ptr(d["red_index"]), n, _lib.ptr(cb), st)
            _lib.call("ssp_gather", _lib.ptr(spu), _lib.ptr(d["red_index"]), n, _lib.ptr(sp), st)
        else:
            _lib.call("ssp_reduction", _lib.ptr(d["c0"]), _lib.ptr(d["phi"]), _lib.ptr(d["psi"]), n, float(lam),
                      davis.encode(), _lib.ptr(cb), _lib.ptr(sp), st)
        self._owned_overlap_c_bar, self._owned_overlap_sin_phi = cb, sp
        self._owned_unique_c_bar, self._owned_unique_sin_phi = cb, sp
        self._red_key = key
        self.c_bar = None
        self.sin_phi = None
        self.time_reduction.append(perf_counter() - t0)

    def _evaluate(self, U, *, tangent: bool):
        pat = self._require_pattern()
        if self._owned_overlap_c_bar is None:
            raise ValueError("Material reduction not set. Call reduction(lambda) first.")
        mode = str(self.owned_constitutive_mode).lower()
        if mode != "global" and mode not in _OWNED_MODES:
            raise ValueError(f"Unsupported owned constitutive mode {self.owned_constitutive_mode!r}")
        t = _lib.require_cuda()
        t0 = perf_counter()
        E = overlap_strain_device(pat, U, mixed=self.tangent_form == "mixed")
        self.time_local_strain.append(perf_counter() - t0)
        t1 = perf_counter()
        n = pat.n_local_int
        d = self._dev
        S = t.empty((n, 6 if pat.dim == 3 else 4), dtype=t.float64, device="cuda")
        DS = t.empty((n, self.n_strain * self.n_strain), dtype=t.float64, device="cuda") if tangent else None
        st = _lib.stream_handle()
        args = (_lib.ptr(E), _lib.ptr(self._owned_overlap_c_bar), _lib.ptr(self._owned_overlap_sin_phi),
                _lib.ptr(d["shear"]), _lib.ptr(d["bulk"]), _lib.ptr(d["lame"]), n)
        branch = None
        pending = False
        mode = self.return_mapping if pat.dim == 3 else ("unsorted" if self.return_mapping == "unsorted" else "binned2d")
        if tangent and mode == "binned2d":  # elastic points finished first, the return mapping on the rest
            branch = t.empty(n, dtype=t.int8, device="cuda")
            if self._scratch is None or self._scratch.numel() < n + 1:
                self._scratch = t.empty(3 * n + 12, dtype=t.int32, device="cuda")
            _lib.call("ssp_constitutive_2d_sds_binned", _lib.ptr(E), _lib.ptr(self._owned_overlap_c_bar),
                      _lib.ptr(self._owned_overlap_sin_phi), _lib.ptr(d["shear"]), _lib.ptr(d["lame"]), n, _lib.ptr(S),
                      _lib.ptr(DS), _lib.ptr(branch), _lib.ptr(self._scratch), st)
        elif tangent and mode in ("binned", "learned", "previous"):
            prev = self._prev_branch if mode == "previous" else None
            if mode == "previous" and (prev is None or prev.numel() != n):
                mode = "binned"
            branch = t.empty(n, dtype=t.int8, device="cuda")
            need = (3 if mode == "binned" else 8) * n + 12
            if self._scratch is None or self._scratch.numel() < need:
                self._scratch = t.empty(need, dtype=t.int32, device="cuda")
            # the mixed form: the plastic points' DS in double-float arithmetic (S, branches FP64)
            options = (_lib.RM_COMPENSATED_DS if self.tangent_form == "mixed" else 0) | \
                (_lib.RM_PLASTIC_DS_ONLY if self.lazy_elastic_ds else 0)
            if mode == "learned":
                if self.branch_model is None:
                    raise ValueError("return_mapping='learned' needs a trained branch_model")
                bins, source = _lib.BINS_LEARNED, _lib.ptr(self.branch_model.params)
            elif mode == "previous":
                bins, source = _lib.BINS_GIVEN, _lib.ptr(prev)
            else:
                bins, source = _lib.BINS_EXACT, None
            _lib.call("ssp_constitutive_3d_sds_screened", _lib.ptr(E), _lib.ptr(self._owned_overlap_c_bar),
                      _lib.ptr(self._owned_overlap_sin_phi), _lib.ptr(d["shear"]), _lib.ptr(d["lame"]), n, _lib.ptr(S),
                      _lib.ptr(DS), _lib.ptr(branch), _lib.ptr(self._scratch), bins, source, options, st)
            pending = self.lazy_elastic_ds
        elif tangent:
            branch = t.empty(n, dtype=t.int8, device="cuda")
            _lib.call("ssp_constitutive_sds_branch", pat.dim, _lib.ptr(E), _lib.ptr(self._owned_overlap_c_bar),
                      _lib.ptr(self._owned_overlap_sin_phi), _lib.ptr(d["shear"]), _lib.ptr(d["lame"]), n, _lib.ptr(S),
                      _lib.ptr(DS), _lib.ptr(branch), st)
        elif pat.dim == 3:
            _lib.call("ssp_constitutive_3d_s", *args, _lib.ptr(S), st)
        else:
            _lib.call("ssp_constitutive_2d", *args, _lib.ptr(S), None, st)
        self.time_local_constitutive.append(perf_counter() - t1)
        self._S_aos = S
        self._DS_aos = DS
        self._branch = branch
        self._ds_elastic_pending = pending
        if branch is not None:
            self._prev_branch = branch
        self._ds_symmetric = bool(tangent)
        self.S = None
        self.DS = None

    def constitutive_problem_stress(self, U):
        t0 = perf_counter()
        self._evaluate(U, tangent=False)
        self.time_stress.append(perf_counter() - t0)
        return self._owned_local_S

    def constitutive_problem_stress_tangent(self, U):
        t0 = perf_counter()
        self._evaluate(U, tangent=True)
        self.time_stress_tangent.append(perf_counter() - t0)
        return self._owned_local_S

    def _force_device(self):
        pat = self._require_pattern()
        if self._S_aos is None:
            raise ValueError("Stress tensor not computed")
        t0 = perf_counter()
        S = self._S_aos[:, : self.n_strain].contiguous() if self._S_aos.shape[1] != self.n_strain else self._S_aos
        F = owned_force_device(pat, S, mixed=self.tangent_form == "mixed")
        self.time_local_force_assembly.append(perf_counter() - t0)
        return F

    def _to_host(self, x):
        return x.cpu().numpy() if self.host_outputs else x

    def build_F_local(self):
        t0 = perf_counter()
        out = self._to_host(self._force_device())
        self.time_build_F.append(perf_counter() - t0)
        return out

    def build_F_free_local(self):
        t0 = perf_counter()
        F = self._force_device()
        t = _lib.torch()
        idx = self.owned_tangent_pattern.device["owned_free_rows"]
        free = t.empty(idx.numel(), dtype=t.float64, device="cuda")
        _lib.call("ssp_gather", _lib.ptr(F), _lib.ptr(idx), int(idx.numel()), _lib.ptr(free), _lib.stream_handle())
        out = self._to_host(free)
        self.time_build_F.append(perf_counter() - t0)
        return out

    def _single_rank_check(self):
        pat = self._require_pattern()
        if pat.owned_row_range != (0, int(pat.local_matrix_pattern.shape[1])):
            raise RuntimeError("Global force gathering needs every row owned by this device (one-GPU operator)")
        return pat

    def build_F(self):
        pat = self._single_rank_check()
        t0 = perf_counter()
        F = self._force_device()
        self.time_local_force_gather.append(0.0)
        out = F.cpu().numpy().reshape(self.dim, -1, order="F") if self.host_outputs else F.reshape(-1, self.dim).T
        self.time_build_F.append(perf_counter() - t0)
        return out

    def build_F_free(self):
        self._single_rank_check()
        return self.build_F_free_local()

    def _elastic_tangent_values(self):
        """CSR values of the tangent with every point elastic (constrained diagonals = 1), assembled
        once per pattern; the base of the elastic-predictor / plastic-correction assembly."""
        if self._K_el is None:
            t = _lib.require_cuda()
            pat = self._require_pattern()
            n = pat.n_local_int
            d = self._dev
            blocks = t.empty((n, self.n_strain * self.n_strain), dtype=t.float64, device="cuda")
            _lib.call("ssp_elastic_tangent_blocks", pat.dim, _lib.ptr(d["shear"]), _lib.ptr(d["lame"]), n,
                      _lib.ptr(blocks), _lib.stream_handle())
            self._K_el = tangent_values_device(pat, blocks, symmetric=True)
            del blocks
        return self._K_el

    def _regularized_start(self, r):
        """(1-r) K_el,t + r K_el: it depends on r and the pattern only, so it is blended once per r
        and each regularised build starts from a copy of it."""
        pat = self._require_pattern()
        base = self._elastic_tangent_values()
        rr = float(r)
        if self._blend_base is None or self._blend_base[0] != rr:
            self._drain_staged()  # a staged copy may still read the old blend
            buf = self._blend_base[1] if self._blend_base is not None else _lib.torch().empty_like(base)
            _lib.call("ssp_blend_values", _lib.ptr(buf), _lib.ptr(base), _lib.ptr(pat.device["elastic_values"]), rr,
                      pat.nnz, _lib.stream_handle())
            self._blend_base = (rr, buf)
        return self._blend_base[1]

    def _drain_staged(self):
        """Order the current stream after a staged copy that no build has waited for yet."""
        staged, self._staged_values = self._staged_values, None
        if staged is not None:
            _lib.torch().cuda.current_stream().wait_event(staged[2])
        return staged

    def _copy_values(self, dst, src):
        """dst := src (CSR values, device): a stream memcpy, or with values_copy = "kernel" the
        library's SM copy kernel (a kernel node when the build is captured in a CUDA graph)."""
        if self.values_copy == "kernel":
            _lib.call("ssp_copy_device", _lib.ptr(src), int(src.numel()), _lib.ptr(dst), _lib.stream_handle())
        else:
            dst.copy_(src)

    def _restore_start(self, values, start, kind, key, staged=False):
        """values := start.  When values holds start plus the corrections of the last build of this
        kind with the same start (key), only the rows of that build's plastic elements differ from
        start, and only those rows are copied (row marks through the element -> row map, then a row
        copy); otherwise every value is copied.  In a captured CUDA graph the build reads and rewrites
        the same plastic-element list (_tangent_into), so every replay restores the rows of the
        previous replay's list."""
        t = _lib.torch()
        last = self._last_build.get(kind)
        if not (self.incremental_values and last is not None and last["key"] == key and last["values"] is values):
            self._copy_values(values, start)
            return
        pat = self._require_pattern()
        dv, d = self._dev, pat.device
        n_rows, n_el = int(pat.local_matrix_pattern.shape[0]), int(pat.overlap_elements.size)
        mark, st = dv["restore_mark"], _lib.stream_handle()  # allocated with the plastic lists
        mark.zero_()
        elist, ecount = dv["plastic_lists"][kind][last["list"]]
        _lib.call("ssp_mark_element_rows", _lib.ptr(d["elem_row"]), n_el, pat.dim * pat.n_p, _lib.ptr(elist),
                  _lib.ptr(ecount), n_rows, _lib.ptr(mark), st)
        # staged beside the strain and return mapping: with many points per CSR entry (P2) those run
        # long enough to hide a slower copy on a small share of the SMs (two blocks per SM); with few
        # (P4) they are short, and shares of 4 to 8 blocks per SM measured the same, so the copy
        # keeps the whole device.  The single-pass (unsorted) and learned return mappings run kernels
        # that need a whole SM (their registers, or the network's tensor memory) and would wait for
        # the copy instead: there too it takes the whole device
        share = 8
        if staged and self.return_mapping in ("binned", "previous"):
            share = self.restore_share or (2 if pat.n_local_int >= 0.01 * pat.nnz else 8)
        _lib.call("ssp_copy_rows_device_share", _lib.ptr(start), _lib.ptr(d["indptr"]), _lib.ptr(mark), n_rows,
                  int(values.numel()), _lib.ptr(values), int(share), st)

    def _stage_values(self, r):
        """Issue the copy of the regularised tangent's starting values into its values array on the
        second stream, ahead of the strain and return-mapping kernels that the build runs first:
        the copy (nnz doubles read and written, HBM-bound) overlaps those FP64-bound kernels, and
        the tangent assembly waits for it instead of copying."""
        self._drain_staged()
        if not self.stage_values or self.owned_tangent_pattern is None or \
                self.owned_tangent_kernel not in ("rows", "legacy"):
            return
        t = _lib.require_cuda()
        pat = self.owned_tangent_pattern
        start = self._regularized_start(r)
        if self._regularized_values is None:
            self._regularized_values = t.empty(pat.nnz, dtype=t.float64, device="cuda")
        values = self._regularized_values
        if self._owned_regularized_mat is not None and hasattr(self._owned_regularized_mat, "fence"):
            self._owned_regularized_mat.fence()  # the last host copy of these values has read them
        main, side = t.cuda.current_stream(), self._aux_stream()
        side.wait_stream(main)
        with t.cuda.stream(side):
            self._restore_start(values, start, "regularized", ("regularized", float(r)), staged=True)
        values.record_stream(side)
        start.record_stream(side)
        done = t.cuda.Event()
        done.record(side)
        self._staged_values = (("regularized", float(r)), values, done)

    def _tangent_into(self, values, r=None):
        pat = self._require_pattern()
        if self._DS_aos is None:
            raise ValueError("Tangent DS not computed")
        t0 = perf_counter()
        ev = self.tangent_events
        if ev is not None:  # optional CUDA-event bracket of the tangent kernel (measurement)
            t = _lib.torch()
            e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
        st = _lib.stream_handle()
        d = pat.device
        if self._ds_symmetric and self._branch is not None and self.owned_tangent_kernel in ("rows", "legacy"):
            # tangent = elastic tangent + plastic-point corrections (FP64 work on plastic points only)
            base = self._elastic_tangent_values()
            if r is None:
                start, key, scale = base, ("tangent",), 1.0
            else:
                start, key, scale = self._regularized_start(r), ("regularized", float(r)), 1.0 - float(r)
            staged = self._drain_staged()
            if staged is None or staged[0] != key or staged[1] is not values:
                self._restore_start(values, start, key[0], key)
            # else the copy of start, issued on the second stream ahead of the strain and return
            # mapping (_stage_values), has overlapped them
            if ev is not None:
                e0.record()
            entry = "ssp_tangent_plastic_correction"
            if self.tangent_form == "mixed" and (pat.dim, pat.n_p) in MIXED_TANGENT_ELEMENTS:
                entry = "ssp_tangent_plastic_correction_mixed"
            n_el = int(pat.overlap_elements.size)
            dv = self._dev
            kind = key[0]
            lists = dv.setdefault("plastic_lists", {})
            if kind not in lists:
                t = _lib.torch()
                lists[kind] = [(t.empty(max(n_el, 1), dtype=t.int32, device="cuda"),
                                t.empty(1, dtype=t.int32, device="cuda")) for _ in range(2)]
                # buffers of the incremental restore (_restore_start), allocated before any capture
                n_rows = int(pat.local_matrix_pattern.shape[0])
                if "restore_mark" not in dv:
                    dv["restore_mark"] = t.empty(max(n_rows, 1), dtype=t.uint8, device="cuda")
                if "indptr" not in d:
                    d["indptr"] = t.as_tensor(np.asarray(pat.local_matrix_pattern.indptr, dtype=np.int32),
                                              device="cuda")
            # two plastic-element lists per kind, alternating: the previous build's list stays
            # valid for the incremental host refresh (_changed_rows)
            last = self._last_build.get(kind)
            same = last is not None and last["key"] == key and last["values"] is values
            cur = 1 - last["list"] if last is not None else 0
            if same and _lib.torch().cuda.is_current_stream_capturing():
                # a graph's replays do not alternate: the build restores (_restore_start) and then
                # rewrites the one list, so each replay restores the previous replay's rows
                cur = last["list"]
            elist, ecount = lists[kind][cur]
            # the correction visits the plastic elements only (an even share per warp)
            _lib.call("ssp_plastic_elements", _lib.ptr(self._branch), n_el, pat.n_q, _lib.ptr(elist), _lib.ptr(ecount),
                      st)
            mixed_entry = entry == "ssp_tangent_plastic_correction_mixed"
            split = int(self.moment_min_points_mixed if mixed_entry else self.moment_min_points)
            moments = split > 0 and pat.dim == 3 and pat.n_p == 10 and _p2_affine_inputs(pat) is not None
            clist, ccount = elist, ecount
            if moments and split <= 1:  # every plastic element in moment form
                many, n_many, clist = elist, ecount, None
            elif moments:  # elements with many plastic points in moment form, the others point by point
                if "split_lists" not in dv:
                    t = _lib.torch()
                    dv["split_lists"] = tuple(t.empty(max(n, 1), dtype=t.int32, device="cuda")
                                              for n in (n_el, 1, n_el, 1))
                few, n_few, many, n_many = dv["split_lists"]
                _lib.call("ssp_plastic_elements_split", _lib.ptr(self._branch), n_el, pat.n_q, split, _lib.ptr(few),
                          _lib.ptr(n_few), _lib.ptr(many), _lib.ptr(n_many), st)
                clist, ccount = few, n_few
            if clist is not None:
                _lib.call(entry, pat.dim, _lib.ptr(d["dphi1"]), _lib.ptr(d["dphi2"]),
                          _lib.ptr(d["dphi3"]) if pat.dim == 3 else None, _lib.ptr(self._DS_aos),
                          _lib.ptr(d["weight"]), _lib.ptr(self._branch), _lib.ptr(dv["shear"]), _lib.ptr(dv["lame"]),
                          _lib.ptr(d["scatter_map"]), n_el, pat.n_p, pat.n_q, pat.nnz, scale, _lib.ptr(values),
                          _lib.ptr(clist), _lib.ptr(ccount), st)
            if moments:
                _lib.call("ssp_tangent_plastic_correction_p2_moments" + ("_mixed" if mixed_entry else ""),
                          _lib.ptr(d["jinv"]), _lib.ptr(d["bary"]), _lib.ptr(self._DS_aos), _lib.ptr(d["weight"]),
                          _lib.ptr(self._branch), _lib.ptr(dv["shear"]), _lib.ptr(dv["lame"]),
                          _lib.ptr(d["scatter_map"]), n_el, pat.n_q, pat.nnz, scale, _lib.ptr(values), _lib.ptr(many),
                          _lib.ptr(n_many), st)
            self._build_no += 1
            self._last_build[kind] = {"kind": kind, "key": key, "values": values, "list": cur,
                                      "prev": last["list"] if same else None, "no": self._build_no,
                                      "prev_no": last["no"] if same else None}
            if ev is not None:
                e1.record()
                ev.append((e0, e1))
        else:
            self._complete_ds()
            if ev is not None:
                e0.record()
            self._last_build.clear()
            tangent_values_device(pat, self._DS_aos, kernel=self.owned_tangent_kernel, symmetric=self._ds_symmetric,
                                  out=values)
            if ev is not None:
                e1.record()
                ev.append((e0, e1))
            if r is not None:
                _lib.call("ssp_finish_values", _lib.ptr(values), pat.nnz, None, 0, _lib.ptr(d["elastic_values"]),
                          float(r), st)
        self.time_build_tangent_local.append(perf_counter() - t0)

    def _matrix(self, which: str, values):
        pat = self._require_pattern()
        attr = "_owned_tangent_mat" if which == "tangent" else "_owned_regularized_mat"
        mat = getattr(self, attr)
        if PETSc is not None and self.host_outputs:  # pragma: no cover - needs petsc4py
            vals = values.cpu().numpy()
            lp = pat.local_matrix_pattern
            if mat is None:
                n_glob = int(lp.shape[1])
                mat = PETSc.Mat().createAIJ(size=((lp.shape[0], n_glob), (lp.shape[0], n_glob)),
                                            csr=(lp.indptr.astype(PETSc.IntType), lp.indices.astype(PETSc.IntType), vals))
                mat.setBlockSize(self.dim)
                mat.assemble()
            else:
                mat.setValuesCSR(lp.indptr.astype(PETSc.IntType), lp.indices.astype(PETSc.IntType), vals)
                mat.assemble()
        else:
            if mat is None:
                mat = OwnedCSRMatrix(pat, values)
            if self.host_outputs:
                kind = "tangent" if which == "tangent" else "regularized"
                info = self._last_build.get(kind)
                rows = self._changed_rows(info, mat) if info is not None else None
                mat.sync_host(rows=rows, mirror=(info["key"], info["no"]) if info is not None else None)
        setattr(self, attr, mat)
        return mat

    def _changed_rows(self, info, mat):
        """Row marks of the CSR rows that can differ between the host mirror and the device values:
        when the mirror holds the previous build of the same kind and start (the same r), only the
        rows of that build's and the current build's plastic elements (every other entry equals the start
        values in both).  None: refresh everything."""
        if not self.incremental_host_copy or info["prev"] is None or mat.mirror != (info["key"], info["prev_no"]):
            return None
        if not _lib.host_writable(mat._host.data_ptr()):
            return None
        t = _lib.torch()
        pat = self._require_pattern()
        n_rows, n_el = int(pat.local_matrix_pattern.shape[0]), int(pat.overlap_elements.size)
        dv = self._dev
        if "row_mark" not in dv:
            dv["row_mark"] = t.empty(max(n_rows, 1), dtype=t.uint8, device="cuda")
        mark = dv["row_mark"]
        mark.zero_()
        lists = dv["plastic_lists"][info["kind"]]
        for idx in (info["prev"], info["list"]):
            elist, ecount = lists[idx]
            _lib.call("ssp_mark_element_rows", _lib.ptr(pat.device["elem_row"]), n_el, pat.dim * pat.n_p, _lib.ptr(elist),
                      _lib.ptr(ecount), n_rows, _lib.ptr(mark), _lib.stream_handle())
        return mark

    def _build_owned_tangent_matrix(self):
        t = _lib.require_cuda()
        pat = self._require_pattern()
        if self._tangent_values is None:
            self._tangent_values = t.empty(pat.nnz, dtype=t.float64, device="cuda")
        if self._owned_tangent_mat is not None and hasattr(self._owned_tangent_mat, "fence"):
            self._owned_tangent_mat.fence()
        self._tangent_into(self._tangent_values)
        return self._matrix("tangent", self._tangent_values)

    def _build_owned_regularized_matrix(self, r: float):
        t = _lib.require_cuda()
        pat = self._require_pattern()
        if self._regularized_values is None:
            self._regularized_values = t.empty(pat.nnz, dtype=t.float64, device="cuda")
        if self._owned_regularized_mat is not None and hasattr(self._owned_regularized_mat, "fence"):
            self._owned_regularized_mat.fence()
        self._tangent_into(self._regularized_values, r=r)
        return self._matrix("regularized", self._regularized_values)

    # -------------------------------------------------------------------- BDDC subdomain matrices

    def _bddc_pattern(self):
        pattern = self.bddc_subdomain_pattern
        if pattern is None:
            raise ValueError("BDDC subdomain pattern not configured")
        return pattern

    def _bddc_local_DS(self, complete: bool = True):
        """DS rows of the subdomain's points as an AoS CUDA tensor (n_local, n_strain^2): gathered
        from the owned (overlap) evaluation, else taken from a global ``DS`` (problem.py:1646-1656).
        complete=False: the elastic points' rows may be left as the return mapping left them (the
        plastic corrections read only the plastic points' rows)."""
        t = _lib.require_cuda()
        pattern = self._bddc_pattern()
        if self._DS_aos is not None:
            if complete:
                self._complete_ds()
            if int(pattern.overlap_local_positions.size) != int(pattern.local_int_indices.size):
                raise RuntimeError("BDDC overlap-local integration-point map is incomplete")
            pos = pattern.device.get("overlap_positions")
            if pos is None:
                pos = pattern.device["overlap_positions"] = t.as_tensor(
                    pattern.overlap_local_positions.astype(np.int64), device="cuda")
            return self._DS_aos.index_select(0, pos)
        if self.DS is None:
            raise ValueError("Tangent DS not computed")
        ds = np.asarray(self.DS, dtype=np.float64)[:, pattern.local_int_indices]
        return _lib.to_device(np.ascontiguousarray(ds.T), t.float64)

    def _bddc_matrix_metadata(self, pattern) -> dict:
        """The BDDC set-up data handed over with the subdomain matrix (problem.py:1658-1708):
        Dirichlet rows, coordinates, block size, dof ordering, adjacency, per-component fields and
        primal vertices, as integer arrays where the reference builds PETSc index sets.  The
        near-nullspace bases the reference adds there come from its linear-solver utilities and stay
        with the solver."""
        owned_coord = np.asarray(pattern.owned_coord, dtype=np.float64)
        dim = int(self.dim)
        nodes = np.asarray(pattern.local_nodes, dtype=np.int64)
        vertex_major = dim * np.repeat(nodes, dim) + np.tile(np.arange(dim, dtype=np.int64), nodes.size)
        meta = {
            "bddc_dirichlet_local": np.asarray(pattern.local_dirichlet_dofs, dtype=np.int32),
            "bddc_local_coordinates": np.asarray(owned_coord.T, dtype=np.float64),
            "bddc_local_block_size": dim,
            "bddc_adjacency_source": str(pattern.adjacency_source),
            "bddc_local_vertex_major_ordering": bool(np.array_equal(pattern.local_global_dofs, vertex_major)),
        }
        if pattern.local_field_dofs:
            meta["bddc_field_is_local"] = tuple(np.asarray(v, dtype=np.int32) for v in pattern.local_field_dofs)
        if int(pattern.local_adjacency_indptr.size) and int(pattern.local_adjacency_indices.size):
            meta["bddc_local_adjacency"] = (np.asarray(pattern.local_adjacency_indptr, dtype=np.int32),
                                            np.asarray(pattern.local_adjacency_indices, dtype=np.int32))
        if int(pattern.local_primal_vertices.size):
            meta["bddc_primal_vertices_local"] = np.asarray(pattern.local_primal_vertices, dtype=np.int32)
        return meta

    def _bddc_matrix(self, kind: str, values):
        pattern = self._bddc_pattern()
        mat = self._bddc.get(kind + "_mat")
        if mat is None:
            global_size = int(self.q_mask.size) if self.q_mask is not None else 0
            mat = SubdomainCSRMatrix(pattern, values, global_size=global_size, block_size=self.dim,
                                     metadata=self._bddc_matrix_metadata(pattern))
            self._bddc[kind + "_mat"] = mat
        if self.host_outputs:
            mat.sync_host()
        return mat

    def _bddc_values(self, kind: str):
        t = _lib.torch()
        buf = self._bddc.get(kind)
        if buf is None:
            mat = self._bddc.get(kind + "_mat")
            if mat is not None:
                mat.fence()
            nnz = self._bddc_pattern().nnz
            buf = self._bddc[kind] = t.empty(max(nnz, 1), dtype=t.float64, device="cuda")[:nnz]
        elif self._bddc.get(kind + "_mat") is not None:
            self._bddc[kind + "_mat"].fence()
        return buf

    def _bddc_predictor_ok(self, pattern) -> bool:
        """Whether the subdomain tangent may start from the pattern's elastic values: the subdomain's
        DS rows come from this operator's own evaluation (symmetric, branch codes known) and the
        pattern's elastic moduli are the operator's at the same points (checked once per pattern)."""
        if self._branch is None or not self._ds_symmetric or self._DS_aos is None:
            return False
        if "predictor_ok" not in self._bddc:
            t = _lib.torch()
            d, pos = pattern.device, pattern.device.get("overlap_positions")
            ok = pos is not None and "shear" in d and "lame" in d
            if ok:
                ok = bool(t.equal(self._dev["shear"].index_select(0, pos), d["shear"])) and bool(
                    t.equal(self._dev["lame"].index_select(0, pos), d["lame"]))
            self._bddc["predictor_ok"] = ok
        return self._bddc["predictor_ok"]

    def _bddc_tangent_into(self, values, r=None):
        """Subdomain tangent values into ``values``; with r, the regularised (1-r) K + r K_el.

        When the elastic predictor applies (_bddc_predictor_ok), the elastic subdomain values plus
        the plastic elements' corrections B^T w (DS - D_el) B scaled by (1-r) -- the owned path's
        assembly, FP64 or mixed-precision by ``tangent_form``; otherwise the full element contraction
        of every subdomain point (problem.py:1710-1857)."""
        from .bddc import bddc_tangent_values_device

        pattern = self._bddc_pattern()
        d, st = pattern.device, _lib.stream_handle()
        n_el = int(pattern.local_elements.size)
        predictor = bool(n_el) and self._bddc_predictor_ok(pattern)
        ds = self._bddc_local_DS(complete=not predictor)
        if predictor:
            t = _lib.torch()
            branch = self._branch.index_select(0, d["overlap_positions"])
            if "plastic_list" not in self._bddc:
                self._bddc["plastic_list"] = (t.empty(n_el, dtype=t.int32, device="cuda"),
                                              t.empty(1, dtype=t.int32, device="cuda"))
            elist, ecount = self._bddc["plastic_list"]
            values.copy_(d["elastic_values"])
            _lib.call("ssp_plastic_elements", _lib.ptr(branch), n_el, pattern.n_q, _lib.ptr(elist), _lib.ptr(ecount), st)
            mixed = self.tangent_form == "mixed" and (pattern.dim, pattern.n_p) in MIXED_TANGENT_ELEMENTS
            entry = "ssp_tangent_plastic_correction_mixed" if mixed else "ssp_tangent_plastic_correction"
            _lib.call(entry, pattern.dim, _lib.ptr(d["dphi1"]), _lib.ptr(d["dphi2"]),
                      _lib.ptr(d["dphi3"]) if pattern.dim == 3 else None, _lib.ptr(ds), _lib.ptr(d["weight"]),
                      _lib.ptr(branch), _lib.ptr(d["shear"]), _lib.ptr(d["lame"]), _lib.ptr(d["scatter_map"]), n_el,
                      pattern.n_p, pattern.n_q, pattern.nnz, 1.0 if r is None else 1.0 - float(r), _lib.ptr(values),
                      _lib.ptr(elist), _lib.ptr(ecount), st)
            return values
        bddc_tangent_values_device(pattern, ds, out=values)
        if r is not None and pattern.nnz:
            _lib.call("ssp_finish_values", _lib.ptr(values), pattern.nnz, None, 0, _lib.ptr(d["elastic_values"]),
                      float(r), st)
        return values

    def _build_bddc_tangent_matrix(self, *, local_mat_type: str = "aij"):
        """Subdomain tangent (problem.py:1710-1767); ``local_mat_type`` is accepted for compatibility."""
        t0 = perf_counter()
        vals = self._bddc_tangent_into(self._bddc_values("tangent"))
        self.time_build_tangent_local.append(perf_counter() - t0)
        return self._bddc_matrix("tangent", vals)

    def _build_bddc_elastic_matrix(self, *, local_mat_type: str = "aij"):
        """Subdomain elastic matrix (problem.py:1769-1801)."""
        pattern = self._bddc_pattern()
        vals = self._bddc_values("elastic")
        vals.copy_(pattern.device["elastic_values"])
        return self._bddc_matrix("elastic", vals)

    def _build_bddc_regularized_matrix(self, r: float, *, local_mat_type: str = "aij"):
        """(1-r) K_tangent + r K_elastic on the subdomain pattern (problem.py:1803-1857)."""
        t0 = perf_counter()
        vals = self._bddc_tangent_into(self._bddc_values("regularized"), r=r)
        self.time_build_tangent_local.append(perf_counter() - t0)
        return self._bddc_matrix("regularized", vals)

    # public BDDC builders (problem.py:2099-2112): the reference's Newton loop finds them with
    # getattr (nonlinear/newton.py:188-206) and asks for the subdomain matrix it preconditions with
    def build_bddc_tangent_matrix(self, *, local_mat_type: str = "aij"):
        if self.bddc_subdomain_pattern is None:
            raise RuntimeError("BDDC subdomain pattern not configured")
        return self._build_bddc_tangent_matrix(local_mat_type=local_mat_type)

    def build_bddc_regularized_matrix(self, r: float, *, local_mat_type: str = "aij"):
        if self.bddc_subdomain_pattern is None:
            raise RuntimeError("BDDC subdomain pattern not configured")
        return self._build_bddc_regularized_matrix(r, local_mat_type=local_mat_type)

    def build_bddc_elastic_matrix(self, *, local_mat_type: str = "aij"):
        if self.bddc_subdomain_pattern is None:
            raise RuntimeError("BDDC subdomain pattern not configured")
        return self._build_bddc_elastic_matrix(local_mat_type=local_mat_type)

    def build_K_regularized(self, r: float):
        if self.owned_tangent_pattern is None:
            raise RuntimeError("Regularized in-place matrix path requires owned_tangent_pattern")
        return self._build_owned_regularized_matrix(r)

    def build_F_K_tangent(self):
        if self._DS_aos is None:
            raise ValueError("Tangent DS not computed")
        t0 = perf_counter()
        F = self.build_F()
        K = self._build_owned_tangent_matrix()
        self.time_build_F_K_tangent.append(perf_counter() - t0)
        return F, K

    # composite entry points (problem.py:2030-2146)
    def build_F_all(self, lam, U):
        self.reduction(lam)
        self.constitutive_problem_stress(U)
        return self.build_F()

    def build_F_all_local(self, lam, U):
        self.reduction(lam)
        self.constitutive_problem_stress(U)
        return self.build_F_local()

    def build_F_all_free(self, lam, U):
        self.reduction(lam)
        self.constitutive_problem_stress(U)
        return self.build_F_free()

    def build_F_all_free_local(self, lam, U):
        self.reduction(lam)
        self.constitutive_problem_stress(U)
        return self.build_F_free_local()

    def build_F_K_tangent_all(self, lam, U):
        self.reduction(lam)
        self.constitutive_problem_stress_tangent(U)
        return self.build_F_K_tangent()

    def build_F_K_tangent_all_free(self, lam, U):
        self.reduction(lam)
        self.constitutive_problem_stress_tangent(U)
        return self.build_F_free(), self._build_owned_tangent_matrix()

    def build_F_reduced(self, U):
        self.constitutive_problem_stress(U)
        return self.build_F()

    def build_F_reduced_local(self, U):
        self.constitutive_problem_stress(U)
        return self.build_F_local()

    def build_F_reduced_free(self, U):
        self.constitutive_problem_stress(U)
        return self.build_F_free()

    def build_F_reduced_free_local(self, U):
        self.constitutive_problem_stress(U)
        return self.build_F_free_local()

    def build_F_K_tangent_reduced(self, U):
        self.constitutive_problem_stress_tangent(U)
        return self.build_F_K_tangent()

    def build_F_K_tangent_reduced_free(self, U):
        self.constitutive_problem_stress_tangent(U)
        return self.build_F_free(), self._build_owned_tangent_matrix()

    def _aux_stream(self):
        if self._force_stream is None:
            self._force_stream = _lib.torch().cuda.Stream()
        return self._force_stream

    def _regularized_pair(self, F_fn, r):
        """(F, K_r) of one Newton iteration, the tangent first.  Device outputs: the internal force
        runs on a second stream at the same time as the tangent and the caller's stream waits for
        both.  Host outputs: both on the caller's stream, so the force runs while the tangent's
        values are copied to the host (the copy, not the kernels, bounds that path)."""
        t0 = perf_counter()
        t = _lib.torch()
        if self.host_outputs or not self.concurrent_force:
            K = self.build_K_regularized(r)
            F = F_fn()
        else:
            main = t.cuda.current_stream()
            stress_ready = t.cuda.Event()
            stress_ready.record(main)
            K = self.build_K_regularized(r)
            side = self._aux_stream()
            side.wait_event(stress_ready)
            with t.cuda.stream(side):
                F = F_fn()
            main.wait_stream(side)
            if isinstance(F, t.Tensor):
                F.record_stream(main)
        self.time_build_F_K_tangent.append(perf_counter() - t0)
        return F, K

    def build_F_K_regularized_all(self, lam, U, r):
        self._stage_values(r)
        self.reduction(lam)
        self.constitutive_problem_stress_tangent(U)
        return self._regularized_pair(self.build_F, r)

    def build_F_K_regularized_all_free(self, lam, U, r):
        self._stage_values(r)
        self.reduction(lam)
        self.constitutive_problem_stress_tangent(U)
        return self._regularized_pair(self.build_F_free, r)

    def capture_regularized_build(self, lam, U, r, *, free: bool = True):
        """One Newton iteration's composite build as a CUDA graph, for a fixed strength-reduction
        factor lam and regularisation r (both fixed while Newton iterates on one continuation step).

        U must be a CUDA float64 array [dim, n_nodes] (or its flat form) that the caller updates in
        place between replays.  Returns a CapturedBuild whose replay() re-runs, on the current
        stream, every kernel build_F_K_regularized_all[_free](lam, U, r) launches (the staged
        values copy, strain, return mapping, tangent corrections and internal force) and whose F and
        K are the device outputs that each replay overwrites.  Replays skip the host work of the
        Python entry point (argument checks, ctypes calls, allocations): the launches are recorded
        once.  Requires device outputs (host_outputs = False).  The graph keeps the configuration
        it was captured with (tangent_form, return_mapping, branch model): capture again after
        changing one."""
        t = _lib.require_cuda()
        if self.host_outputs:
            raise ValueError("capture_regularized_build needs host_outputs = False (device outputs)")
        if not (isinstance(U, t.Tensor) and U.is_cuda and U.dtype == t.float64):
            raise ValueError("U must be a CUDA float64 tensor updated in place between replays")
        build = self.build_F_K_regularized_all_free if free else self.build_F_K_regularized_all
        # first use: buffers, caches, the reduction for lam and the blend for r, outside the graph
        side = t.cuda.Stream()
        side.wait_stream(t.cuda.current_stream())
        with t.cuda.stream(side):
            build(lam, U, r)
        t.cuda.current_stream().wait_stream(side)
        t.cuda.synchronize()
        graph = t.cuda.CUDAGraph()
        with t.cuda.graph(graph):
            F, K = build(lam, U, r)
        return CapturedBuild(graph, F, K, self)

    def build_F_K_regularized_reduced(self, U, r):
        self._stage_values(r)
        self.constitutive_problem_stress_tangent(U)
        return self._regularized_pair(self.build_F, r)

    def build_F_K_regularized_reduced_free(self, U, r):
        self._stage_values(r)
        self.constitutive_problem_stress_tangent(U)
        return self._regularized_pair(self.build_F_free, r)

    def potential_energy(self, U):
        """Integrated Mohr-Coulomb potential energy sum_p w_p Psi(E_p(U)) at the current reduction,
        a float (the reference's ConstitutiveOperator.potential_energy, problem.py:2148-2157,
        which the direct SSR continuation calls twice per step, continuation/omega.py:61,83).

        FP64 strain and energy at every overlap point in one kernel with a deterministic block
        sum.  With an owned node range that is part of the mesh, each rank sums the elements whose
        smallest node it owns, and the ranks' sums are all-reduced when a process group is up, so
        every rank returns the whole mesh's energy as the reference's global evaluation does."""
        t0 = perf_counter()
        pat = self._require_pattern()
        if self._owned_overlap_c_bar is None:
            raise ValueError("Material reduction not set. Call reduction(lambda) first.")
        t = _lib.require_cuda()
        E = overlap_strain_device(pat, U)
        d = self._dev
        w = pat.device.get("energy_weight", pat.device["weight"])
        if self._energy_scratch is None:
            self._energy_scratch = t.empty(_lib.POTENTIAL_PARTIALS + 1, dtype=t.float64, device="cuda")
        part, total = self._energy_scratch[:-1], self._energy_scratch[-1:]
        _lib.call("ssp_potential_energy", pat.dim, _lib.ptr(E), _lib.ptr(self._owned_overlap_c_bar),
                  _lib.ptr(self._owned_overlap_sin_phi), _lib.ptr(d["shear"]), _lib.ptr(d["bulk"]), _lib.ptr(d["lame"]),
                  _lib.ptr(w), int(pat.n_local_int), None, None, _lib.ptr(part), _lib.ptr(total),
                  _lib.stream_handle())
        value = float(total.item())
        _lib.raise_on_device_status()
        if "energy_weight" in pat.device:
            import torch.distributed as dist

            if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
                on_gpu = dist.get_backend() == "nccl"
                buf = t.tensor([value], dtype=t.float64, device="cuda" if on_gpu else "cpu")
                dist.all_reduce(buf)
                value = float(buf.item())
        self.time_potential.append(perf_counter() - t0)
        return value

    def get_total_time(self):
        return {
            "reduction": sum(self.time_reduction),
            "stress": sum(self.time_stress),
            "stress_tangent": sum(self.time_stress_tangent),
            "build_F": sum(self.time_build_F),
            "build_F_K_tangent": sum(self.time_build_F_K_tangent),
            "build_tangent_local": sum(self.time_build_tangent_local),
            "local_strain": sum(self.time_local_strain),
            "local_constitutive": sum(self.time_local_constitutive),
            "local_constitutive_comm": sum(self.time_local_constitutive_comm),
            "local_force_assembly": sum(self.time_local_force_assembly),
            "local_force_gather": sum(self.time_local_force_gather),
            "potential": sum(self.time_potential),
        }

    def release_petsc_caches(self) -> None:
        self._drain_staged()
        for attr in ("_owned_tangent_mat", "_owned_regularized_mat"):
            mat = getattr(self, attr, None)
            if mat is not None and hasattr(mat, "destroy"):
                mat.destroy()
            setattr(self, attr, None)
        self._tangent_values = None
        self._regularized_values = None
        self._staged_values = None
        self._last_build = {}
        for key, mat in list(self._bddc.items()):
            if key.endswith("_mat"):
                mat.destroy()
        self._bddc = {}
