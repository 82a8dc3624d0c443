"""Pin the oracle (the CPU restatement the CUDA kernels are compared with) against the reference's outputs.

The fixtures were produced by ``tests/golden/make_golden.py`` from the reference itself: its
compiled C kernels and its NumPy/Python paths.  These tests run on the CPU.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import PLAIN_RTOL, golden, golden_files, rel_err


def test_constitutive_3d_matches_reference_c_kernel(oracle):
    g = golden("constitutive_3d.npz")
    E = g["E"]
    for tag in ("bench_l1.0", "bench_l1.3", "test_l1.0", "test_l1.3"):
        args = [g[f"{tag}_{k}"] for k in ("c_bar", "sin_phi", "shear", "bulk", "lame")]
        S, DS = oracle.constitutive_3d(E, *args)
        assert rel_err(S, g[f"{tag}_S_c"]) <= PLAIN_RTOL
        assert rel_err(DS, g[f"{tag}_DS_c"]) <= PLAIN_RTOL
        S_only = oracle.constitutive_3d(E, *args, tangent=False)
        assert np.array_equal(S_only, S)
        # the reference's NumPy twin agrees with its C kernel at the same level
        assert rel_err(g[f"{tag}_S_np"], g[f"{tag}_S_c"]) <= PLAIN_RTOL
        assert rel_err(g[f"{tag}_DS_np"], g[f"{tag}_DS_c"]) <= 1.0e-11


def test_constitutive_3d_covers_every_branch(oracle):
    g = golden("constitutive_3d.npz")
    branches = set()
    for tag in ("bench_l1.0", "test_l1.3"):
        args = [g[f"{tag}_{k}"] for k in ("c_bar", "sin_phi", "shear", "bulk", "lame")]
        S, DS = oracle.constitutive_3d(g["E"], *args)
        lame = args[4]
        for p in range(S.shape[0]):
            D = DS[p].reshape(6, 6, order="F")
            if not np.any(D):
                branches.add("apex")
            elif np.allclose(D[0, 1], lame[p]) and np.allclose(D[3, 3], args[2][p]) and np.count_nonzero(D) == 12:
                branches.add("elastic")
            else:
                branches.add("plastic")
    assert branches == {"apex", "elastic", "plastic"}


def test_constitutive_2d_matches_reference_numpy(oracle):
    g = golden("constitutive_2d.npz")
    for tag in ("l1.0", "l1.2"):
        args = [g[f"{tag}_{k}"] for k in ("c_bar", "sin_phi", "shear", "bulk", "lame")]
        S, DS = oracle.constitutive_2d(g["E"], *args)
        assert rel_err(S, g[f"{tag}_S"]) <= PLAIN_RTOL
        assert rel_err(DS, g[f"{tag}_DS"]) <= PLAIN_RTOL


def test_reduction_matches_reference(oracle):
    g = golden("reduction.npz")
    for dav in ("A", "B", "C"):
        for lam in (0.8, 1.0, 1.35):
            cb, sp = oracle.reduction(g["c0"], g["phi"], g["psi"], lam, dav)
            assert rel_err(cb, g[f"{dav}_{lam}_c_bar"]) <= 1e-15
            assert rel_err(sp, g[f"{dav}_{lam}_sin_phi"]) <= 1e-15
    with pytest.raises(ValueError):
        oracle.reduction(g["c0"], g["phi"], g["psi"], 0.0, "A")


@pytest.mark.parametrize("name", golden_files("pattern_"))
def test_pattern_restatement_bit_exact(oracle, name):
    g = golden(name)
    p = oracle.owned_pattern(g["elem"], g["q_mask"], tuple(g["owned_node_range"]))
    for key in ("indptr", "indices", "scatter_map", "row_slot_ptr", "slot_elem", "slot_lrow", "slot_pos",
                "constrained_diag_positions", "overlap_elements", "overlap_nodes", "overlap_global_dofs",
                "overlap_element_dof_lids", "owned_local_overlap_dofs", "owned_free_mask"):
        assert np.array_equal(p[key], g[key]), key
        assert p[key].dtype == g[key].dtype or key in ("owned_free_mask",), (key, p[key].dtype, g[key].dtype)


@pytest.mark.parametrize("name", golden_files("pattern_") + golden_files("pattern2d_") + golden_files("overlap_operator_"))
def test_pattern_c_restatement_bit_exact(oracle, name):
    """The C restatement of the pattern builder (the one large meshes use) against the reference."""
    g = golden(name)
    p = oracle.owned_pattern_c(g["elem"], g["q_mask"], tuple(g["owned_node_range"]))
    for key in ("indptr", "indices", "row_slot_ptr", "slot_elem", "slot_lrow", "slot_pos", "constrained_diag_positions",
                "overlap_elements", "overlap_nodes", "overlap_global_dofs", "overlap_element_dof_lids",
                "owned_local_overlap_dofs", "owned_free_mask"):
        assert np.array_equal(p[key], g[key]), key
        assert p[key].dtype == g[key].dtype or key in ("owned_free_mask",), (key, p[key].dtype, g[key].dtype)


def test_pattern_c_restatement_equals_python_restatement_on_a_slope(oracle):
    """C and Python restatements on a larger partially owned P2 slope with a Dirichlet base."""
    from slope_stability_petsc4py_gb300 import synthetic

    m = synthetic.slope_mesh_3d(5, 3, 3, elem_type="P2")
    rng = (m.n_nodes // 5, 3 * m.n_nodes // 5)
    a = oracle.owned_pattern(m.elem, m.q_mask, rng)
    b = oracle.owned_pattern_c(m.elem, m.q_mask, rng)
    for key, val in b.items():
        assert np.array_equal(a[key], val), key


@pytest.mark.parametrize("name", golden_files("pattern_"))
def test_assembly_restatement_matches_reference(oracle, name):
    g = golden(name)
    n_q = int(g["n_q"])
    nnz = g["indices"].size
    d1, d2, d3, w = g["dphi1"], g["dphi2"], g["dphi3"], g["weight"]
    ds_aos = np.ascontiguousarray(g["ds"].T)
    rows = oracle.tangent_rows_3d(d1, d2, d3, ds_aos, w, g["row_slot_ptr"], g["slot_elem"], g["slot_lrow"],
                                  g["slot_pos"], n_q, nnz)
    rows[g["constrained_diag_positions"]] = 1.0
    legacy = oracle.tangent_scatter(3, d1, d2, d3, ds_aos, w, g["scatter_map"], n_q, nnz)
    legacy[g["constrained_diag_positions"]] = 1.0
    assert rel_err(rows, g["rows_c"]) <= PLAIN_RTOL
    assert rel_err(legacy, g["legacy_c"]) <= PLAIN_RTOL
    assert rel_err(g["rows_py"], g["rows_c"]) <= PLAIN_RTOL
    # strain B u and force B^T (w S)
    u_ov = g["U"].reshape(-1, order="F")[g["overlap_global_dofs"]]
    E = oracle.strain_3d(d1, d2, d3, u_ov, g["overlap_element_dof_lids"], n_q)
    assert rel_err(E.T, g["strain_c"]) <= PLAIN_RTOL
    F = oracle.force_rows_3d(d1, d2, d3, np.ascontiguousarray(g["stress"].T), w, g["row_slot_ptr"], g["slot_elem"],
                             g["slot_lrow"], n_q)
    F[~g["owned_free_mask"]] = 0.0
    assert rel_err(F, g["force_c"]) <= PLAIN_RTOL
    assert rel_err(F, g["force_py"]) <= PLAIN_RTOL


@pytest.mark.parametrize("name", golden_files("pattern2d_"))
def test_assembly_restatement_2d_matches_reference(oracle, name):
    g = golden(name)
    n_q = int(g["n_q"])
    nnz = g["indices"].size
    p = oracle.owned_pattern(g["elem"], g["q_mask"], tuple(g["owned_node_range"]))
    for key in ("indptr", "indices", "scatter_map", "constrained_diag_positions", "overlap_element_dof_lids"):
        assert np.array_equal(p[key], g[key]), key
    d1, d2, w = g["dphi1"], g["dphi2"], g["weight"]
    K = oracle.tangent_scatter(2, d1, d2, None, np.ascontiguousarray(g["ds"].T), w, g["scatter_map"], n_q, nnz)
    K[g["constrained_diag_positions"]] = 1.0
    assert rel_err(K, g["legacy_py"]) <= PLAIN_RTOL
    u_ov = g["U"].reshape(-1, order="F")[g["overlap_global_dofs"]]
    E = oracle.strain_2d(d1, d2, u_ov, g["overlap_element_dof_lids"], n_q)
    assert rel_err(E.T, g["strain_py"]) <= PLAIN_RTOL
    f_ov = oracle.overlap_force_2d(d1, d2, np.ascontiguousarray(g["stress"].T), w, g["overlap_element_dof_lids"], n_q,
                                   g["overlap_global_dofs"].size)
    F = f_ov[g["owned_local_overlap_dofs"]]
    F[~g["owned_free_mask"]] = 0.0
    assert rel_err(F, g["force_py"]) <= PLAIN_RTOL


@pytest.mark.parametrize("name", golden_files("pattern_"))
def test_geometry_restatement_matches_reference(oracle, name):
    from slope_stability_petsc4py_gb300 import fem

    g = golden(name)
    et = str(g["elem_type"])
    xi, wf = fem.quadrature(3, et)
    dhat = fem.reference_gradients(3, et)
    elem_ov = g["elem"][:, g["overlap_elements"]]
    (d1, d2, d3), w = oracle.geometry(g["coord"], elem_ov, 3, dhat, wf)
    assert rel_err(d1, g["dphi1"]) <= PLAIN_RTOL
    assert rel_err(d2, g["dphi2"]) <= PLAIN_RTOL
    assert rel_err(d3, g["dphi3"]) <= PLAIN_RTOL
    assert rel_err(w, g["weight"]) <= PLAIN_RTOL


@pytest.mark.parametrize("name", golden_files("pattern_"))
def test_geometry_c_restatement_matches_reference(oracle, name):
    from slope_stability_petsc4py_gb300 import fem

    g = golden(name)
    et = str(g["elem_type"])
    _xi, wf = fem.quadrature(3, et)
    (d1, d2, d3), w = oracle.geometry_3d_c(g["coord"], g["elem"][:, g["overlap_elements"]],
                                           fem.reference_gradients(3, et), wf)
    assert rel_err(d1, g["dphi1"]) <= PLAIN_RTOL
    assert rel_err(d2, g["dphi2"]) <= PLAIN_RTOL
    assert rel_err(d3, g["dphi3"]) <= PLAIN_RTOL
    assert rel_err(w, g["weight"]) <= PLAIN_RTOL


@pytest.mark.parametrize("name", golden_files("pattern_"))
def test_constitutive_operator_outputs_consistent(oracle, name):
    """The reference operator's S/DS/F/K (production settings) agree with the oracle chain."""
    g = golden(name)
    n_q = int(g["n_q"])
    idx = g["local_int_indices"]
    cb, sp = oracle.reduction(g["mat_c0"][idx], g["mat_phi"][idx], g["mat_psi"][idx], float(g["op_lambda"]), "B")
    u_ov = g["op_U"].reshape(-1, order="F")[g["overlap_global_dofs"]]
    E = oracle.strain_3d(g["dphi1"], g["dphi2"], g["dphi3"], u_ov, g["overlap_element_dof_lids"], n_q)
    S, DS = oracle.constitutive_3d(E, cb, sp, g["mat_shear"][idx], g["mat_bulk"][idx], g["mat_lame"][idx])
    assert rel_err(S.T, g["op_S"]) <= PLAIN_RTOL
    assert rel_err(DS.T, g["op_DS"]) <= PLAIN_RTOL
    F = oracle.force_rows_3d(g["dphi1"], g["dphi2"], g["dphi3"], S, g["weight"], g["row_slot_ptr"], g["slot_elem"],
                             g["slot_lrow"], n_q)
    F[~g["owned_free_mask"]] = 0.0
    assert rel_err(F, g["op_F"]) <= PLAIN_RTOL
    assert rel_err(F[g["owned_free_mask"]], g["op_F_free"]) <= PLAIN_RTOL


@pytest.mark.parametrize("dim", [3, 2])
def test_potential_restatement_matches_reference(oracle, dim):
    """The oracle's potential energy densities equal the reference's potential_3D / potential_2D
    (src/slope_stability/constitutive/problem.py:1029-1190) bit for bit, including what the
    reference computes for compressive plane-strain states and unhalved 3D shears."""
    g = golden("potential.npz")
    E = g["E3"] if dim == 3 else g["E2"]
    fn = oracle.potential_3d if dim == 3 else oracle.potential_2d
    for key in ("bench", "test"):
        tag = f"{key}_{dim}d"
        psi, br = fn(E, *(g[f"{tag}_{k}"] for k in ("c_bar", "sin_phi", "shear", "bulk", "lame")), with_branch=True)
        assert np.array_equal(psi, g[f"{tag}_psi"])
        assert np.bincount(br, minlength=5).min() > 0 or dim == 2  # every 3D branch is exercised
