"""CPU-side checks of the C-ABI library: it loads, exports every declared entry point, and its
host pattern builder reproduces the reference's CSR pattern and maps bit for bit.  No CUDA
kernel is launched here."""

from __future__ import annotations

import ctypes
import re

import numpy as np
import pytest

from conftest import REPO, golden, golden_files

from slope_stability_petsc4py_gb300 import _lib, synthetic
from slope_stability_petsc4py_gb300.distributed_tangent import _ensure_int32_capacity, _PatternBuild

PATTERN_KEYS = ("overlap_elements", "overlap_nodes", "overlap_element_dof_lids", "owned_local_overlap_dofs", "indptr",
                "indices", "constrained_diag_positions", "scatter_map", "row_slot_ptr", "slot_elem", "slot_lrow",
                "slot_pos")


def declared_symbols():
    text = (REPO / "include" / "ssp_gb300.h").read_text()
    return sorted(set(re.findall(r"\b(?:int|void)\s+(ssp_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_symbols()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(_lib.exported_symbols())


def test_invalid_arguments_are_rejected_before_launch():
    lib = _lib.load()
    # negative sizes and null outputs return SSP_ERR_INVALID without touching the GPU
    assert lib.ssp_constitutive_3d_sds(None, None, None, None, None, None, -1, None, None, None) == 1
    assert lib.ssp_constitutive_3d_sds(None, None, None, None, None, None, 0, None, None, None) == 0
    assert lib.ssp_reduction(None, None, None, 4, 0.0, b"A", None, None, None) == 1
    assert lib.ssp_reduction(None, None, None, 4, 1.0, b"Z", None, None, None) == 1
    assert lib.ssp_tangent_element(4, 0, *[None] * 6, 1, 10, 11, 10, None, 0, None) == 1
    assert lib.ssp_assemble_overlap_strain_3d(None, None, None, None, 0, None, 12, 2, 10, 5, None, None) == 1
    v = ctypes.c_int(0)
    assert lib.ssp_device_status(None, 0) == 1


@pytest.mark.parametrize("name", golden_files("pattern_") + golden_files("pattern2d_"))
def test_host_pattern_builder_bit_exact_with_reference(name):
    g = golden(name)
    pb = _PatternBuild(g["elem"], g["q_mask"], tuple(g["owned_node_range"]))
    keys = PATTERN_KEYS if not name.startswith("pattern2d") else PATTERN_KEYS[:8]
    for key in keys:
        got = pb.get(key)
        assert got.dtype == g[key].dtype, (key, got.dtype, g[key].dtype)
        assert np.array_equal(got, g[key]), key
    assert np.array_equal(pb.get("owned_free_mask").astype(bool), g["owned_free_mask"])
    pb.close()


@pytest.mark.parametrize("et,owned", [("P2", "full"), ("P2", "middle"), ("P4", "head"), ("P1", "tail")])
def test_host_pattern_builder_matches_oracle_on_slope_meshes(oracle, et, owned):
    m = synthetic.slope_mesh_3d(4, 2, 2, depth=6.0, elem_type=et)
    n = m.n_nodes
    rng = {"full": (0, n), "middle": (n // 3, 2 * n // 3), "head": (0, n // 5), "tail": (n - n // 4, n)}[owned]
    ref = oracle.owned_pattern(m.elem, m.q_mask, rng)
    pb = _PatternBuild(m.elem, m.q_mask, rng)
    for key in PATTERN_KEYS:
        assert np.array_equal(pb.get(key), ref[key]), key
    elem_row = pb.get("elem_row")
    # elem_row marks exactly the (element, local dof) pairs that own a row slot
    assert int((elem_row >= 0).sum()) == pb.sizes["n_slots"]
    pb.close()


def test_host_pattern_builder_2d_matches_oracle(oracle):
    m = synthetic.slope_mesh_2d(6, 4, elem_type="P2")
    rng = (5, m.n_nodes - 7)
    ref = oracle.owned_pattern(m.elem, m.q_mask, rng)
    pb = _PatternBuild(m.elem, m.q_mask, rng)
    for key in PATTERN_KEYS:
        assert np.array_equal(pb.get(key), ref[key]), key


def test_pattern_builder_rejects_bad_input():
    m = synthetic.slope_mesh_3d(3, 1, 1, depth=3.0, elem_type="P2")
    bad = m.elem.copy()
    bad[0, 0] = m.n_nodes + 5
    with pytest.raises(_lib.SSPError):
        _PatternBuild(bad, m.q_mask, (0, m.n_nodes))
    with pytest.raises(_lib.SSPError):
        _PatternBuild(m.elem, m.q_mask, (0, m.n_nodes + 1))


def test_int32_capacity_guard_raises():
    with pytest.raises(OverflowError):
        _ensure_int32_capacity("test", np.iinfo(np.int32).max + 1)


def test_quadrature_and_basis_match_reference_dphi(oracle):
    """fem tables reproduce the reference's dphi (checked through the oracle geometry)."""
    from slope_stability_petsc4py_gb300 import fem

    for name in golden_files("pattern2d_"):
        g = golden(name)
        et = str(g["elem_type"])
        xi, wf = fem.quadrature(2, et)
        (d1, d2), w = oracle.geometry(g["coord"], g["elem"][:, g["overlap_elements"]], 2, fem.reference_gradients(2, et), wf)
        assert np.max(np.abs(d2 - g["dphi2"])) <= 1e-12 * np.max(np.abs(g["dphi2"]))
        assert np.max(np.abs(d1 - g["dphi1"])) <= 1e-12 * np.max(np.abs(g["dphi1"]))
        assert np.max(np.abs(w - g["weight"])) <= 1e-12 * np.max(np.abs(g["weight"]))


def test_operator_api_surface_without_a_gpu():
    """The drop-in operator keeps the reference's constructor fields and entry points (checked on
    the class: constructing one needs a GPU)."""
    import dataclasses
    import inspect

    from slope_stability_petsc4py_gb300 import CapturedBuild, ConstitutiveOperator

    assert dataclasses.is_dataclass(ConstitutiveOperator) and not dataclasses.is_dataclass(CapturedBuild)
    fields = {f.name for f in dataclasses.fields(ConstitutiveOperator)}
    assert {"B", "c0", "phi", "psi", "Davis_type", "shear", "bulk", "lame", "WEIGHT", "n_strain", "n_int", "dim",
            "q_mask"} <= fields
    for name in ("reduction", "constitutive_problem_stress", "constitutive_problem_stress_tangent", "build_F",
                 "build_F_free", "build_K_regularized", "build_F_K_tangent", "build_F_K_regularized_all",
                 "build_F_K_regularized_all_free", "build_F_K_regularized_reduced",
                 "build_F_K_regularized_reduced_free", "set_owned_tangent_pattern", "capture_regularized_build"):
        assert callable(getattr(ConstitutiveOperator, name)), name
    assert list(inspect.signature(ConstitutiveOperator.build_F_K_regularized_all_free).parameters) == \
        ["self", "lam", "U", "r"]


@pytest.mark.parametrize("name", [n for n in golden_files("pattern2d_") if "P4" in n])
def test_triangle_p4_node_order_matches_reference_generator(name):
    """The reference's P4 triangle mesh places local node k at the barycentric point
    tri_node_tuples(4)[k] / 4 of its vertices, as the synthetic generator here does."""
    from slope_stability_petsc4py_gb300 import synthetic

    tup = np.asarray(synthetic.tri_node_tuples(4), dtype=np.float64) / 4.0
    for coord, elem in ((golden(name)["coord"], golden(name)["elem"]),
                        (lambda m: (m.coord, m.elem))(synthetic.slope_mesh_2d(4, 3, elem_type="P4"))):
        X = coord[:, elem]
        assert np.max(np.abs(np.einsum("dve,kv->dke", X[:, :3], tup) - X)) <= 1e-12 * np.max(np.abs(coord))


@pytest.mark.parametrize("name", golden_files("overlap_operator_"))
def test_overlap_strain_operator_equals_reference(name):
    """overlap_B (include_overlap_B=True) from the pattern's gradients: the reference's sparse strain
    operator, same rows, columns and canonical CSR structure, values to rounding of the gradients."""
    from scipy.sparse import csr_matrix

    from slope_stability_petsc4py_gb300.distributed_tangent import _strain_operator

    g = golden(name)
    dim = g["q_mask"].shape[0]
    nodes = g["overlap_nodes"]
    lid = np.full(g["coord"].shape[1], -1, dtype=np.int64)
    lid[nodes] = np.arange(nodes.size)
    elem_ov = lid[g["elem"][:, g["overlap_elements"]]]
    dphi = [g["dphi1"], g["dphi2"]] + ([g["dphi3"]] if dim == 3 else [])
    B = _strain_operator(dim, dphi, elem_ov, int(g["n_q"]), nodes.size)
    ref = csr_matrix((g["B_data"], g["B_indices"], g["B_indptr"]), shape=tuple(g["B_shape"]))
    assert B.shape == ref.shape
    assert np.array_equal(B.indptr, ref.indptr) and np.array_equal(B.indices, ref.indices)
    assert np.max(np.abs(B.data - ref.data)) <= 1e-12 * np.max(np.abs(ref.data))


@pytest.mark.parametrize("name", golden_files("overlap_operator_"))
def test_reference_elastic_rows_project_onto_the_pattern(name):
    """A reference OwnedElasticRows passed as elastic_rows: its assembled rows projected onto the
    owned pattern give the reference's elastic_values bit for bit (entries outside the pattern,
    such as constrained columns, are dropped)."""
    from scipy.sparse import csr_matrix

    from slope_stability_petsc4py_gb300.distributed_tangent import _project_values_onto_pattern

    g = golden(name)
    L = csr_matrix((g["L_data"], g["L_indices"], g["L_indptr"]), shape=tuple(g["L_shape"]))
    vals = _project_values_onto_pattern(L, g["indptr"], g["indices"], int(g["L_shape"][1]))
    assert np.array_equal(vals, g["elastic_values"])
    with pytest.raises(ValueError):
        _project_values_onto_pattern(L[:-1], g["indptr"], g["indices"], int(g["L_shape"][1]))
