"""BDDC subdomain tangent on the GPU against the reference (golden fixtures ``bddc_*.npz`` made by
the reference's ``prepare_bddc_subdomain_pattern`` / ``assemble_bddc_subdomain_tangent_values``) and,
through the operator, against the oracle.  Plain-path tolerance 1e-12 (max-norm relative); maps and
index arrays bit for bit."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import PLAIN_RTOL, golden, golden_files, rel_err

pytestmark = pytest.mark.gpu

MATERIAL = {"c0": 15.0, "phi": 30.0, "psi": 0.0, "young": 10000.0, "poisson": 0.33, "gamma_sat": 19.0,
            "gamma_unsat": 19.0}
MATERIALS = [MATERIAL, dict(MATERIAL, young=2.0 * MATERIAL["young"], poisson=0.3)]


@pytest.fixture(autouse=True)
def _clean_status(cuda_device):
    from slope_stability_petsc4py_gb300 import _lib

    _lib.device_status(clear=True)
    yield
    assert _lib.device_status(clear=True) == 0


def _prepare(g):
    from slope_stability_petsc4py_gb300 import prepare_bddc_subdomain_pattern

    return prepare_bddc_subdomain_pattern(
        g["coord"], g["elem"], g["q_mask"], g["material_identifier"], MATERIALS, tuple(g["owned_node_range"]),
        elem_type=str(g["elem_type"]), overlap_local_int_indices=g["overlap_local_int_indices"],
        adjacency_source=str(g["adjacency_source"]), corner_only_primals=bool(g["corner_only_primals"]))


@pytest.mark.parametrize("name", golden_files("bddc_"))
def test_bddc_pattern_and_values_match_reference(name):
    from slope_stability_petsc4py_gb300 import assemble_bddc_subdomain_tangent_values

    g = golden(name)
    pat = _prepare(g)
    for key in ("local_elements", "local_nodes", "scatter_map", "constrained_diag_positions", "local_dirichlet_dofs",
                "local_int_indices", "overlap_local_positions", "local_primal_vertices"):
        want, got = np.asarray(g[key]), np.asarray(getattr(pat, key))
        assert (want.size == 0 and got.size == 0) or np.array_equal(want, got), key
    assert np.array_equal(pat.local_matrix_pattern.indptr, g["indptr"])
    assert np.array_equal(pat.local_matrix_pattern.indices, g["indices"])
    if pat.local_elements.size == 0:
        assert pat.nnz == 0 and assemble_bddc_subdomain_tangent_values(pat, g["ds"]).size == 0
        return
    for key in ("dphi1", "dphi2", "local_assembly_weight", "elastic_values", "local_coord", "owned_coord"):
        assert rel_err(getattr(pat, key), g[key]) <= PLAIN_RTOL, key
    if pat.dim == 3:
        assert rel_err(pat.dphi3, g["dphi3"]) <= PLAIN_RTOL
    vals = assemble_bddc_subdomain_tangent_values(pat, g["ds"])
    assert rel_err(vals, g["values_py"]) <= PLAIN_RTOL
    if "values_c" in g:
        assert rel_err(vals, g["values_c"]) <= PLAIN_RTOL
    assert np.all(vals[pat.constrained_diag_positions] == 1.0)
    # a global DS (every point of the mesh): the subdomain's columns are taken
    n_glob = g["elem"].shape[1] * pat.n_q
    ds_glob = np.full((g["ds"].shape[0], n_glob), np.nan)
    ds_glob[:, pat.local_int_indices] = g["ds"]
    assert rel_err(assemble_bddc_subdomain_tangent_values(pat, ds_glob), g["values_py"]) <= PLAIN_RTOL
    with pytest.raises(ValueError):
        assemble_bddc_subdomain_tangent_values(pat, g["ds"][1:])


@pytest.mark.parametrize("dim,et", [(3, "P2"), (2, "P4")])
def test_operator_bddc_matrices_against_oracle(oracle, dim, et):
    """Operator flow: owned evaluation of S/DS, then the subdomain tangent, elastic and regularised
    matrices from the subdomain's DS rows, against the oracle's element scatter."""
    from slope_stability_petsc4py_gb300 import ConstitutiveOperator, prepare_bddc_subdomain_pattern, synthetic

    mats = synthetic.MaterialSet.layered(4, seed=5)
    mesh = (synthetic.slope_mesh_3d(6, 3, 3, elem_type=et, n_layers=4) if dim == 3
            else synthetic.slope_mesh_2d(8, 5, elem_type=et, n_layers=4))
    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=float(mats.psi[i]), young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=20.0, gamma_unsat=20.0) for i in range(mats.c0.size)]
    op = ConstitutiveOperator.from_mesh(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs, elem_type=et)
    owners = np.sort(mesh.elem.min(axis=0))
    owned = (int(owners[owners.size // 4]), int(owners[3 * owners.size // 4]))
    pat = prepare_bddc_subdomain_pattern(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs, owned,
                                         elem_type=et,
                                         overlap_local_int_indices=op.owned_tangent_pattern.local_int_indices,
                                         adjacency_source="topology", corner_only_primals=True)
    assert pat.local_elements.size > 0
    op.set_bddc_subdomain_pattern(pat)
    U = synthetic.displacement_field(mesh, mats, amplitude=0.05, seed=7)
    op.reduction(1.2)
    op.constitutive_problem_stress_tangent(U)
    DS = np.asarray(op._owned_local_DS)[:, pat.overlap_local_positions]
    K_o = oracle.tangent_scatter(dim, pat.dphi1, pat.dphi2, pat.dphi3 if dim == 3 else None, np.ascontiguousarray(DS.T),
                                 pat.local_assembly_weight, pat.scatter_map, pat.n_q, pat.nnz)
    K_o[pat.constrained_diag_positions] = 1.0
    # through the public names, found by getattr as the reference's Newton loop finds them
    # (nonlinear/newton.py:188-206)
    mat = getattr(op, "build_bddc_tangent_matrix")()
    rows, cols, vals = mat.getValuesCSR()
    assert np.array_equal(rows, pat.local_matrix_pattern.indptr) and np.array_equal(cols, pat.local_matrix_pattern.indices)
    assert rel_err(vals, K_o) <= PLAIN_RTOL
    assert np.array_equal(mat.local_to_global, pat.local_global_dofs) and mat.block_size == dim
    assert mat.global_size == mesh.q_mask.size and mat.metadata["bddc_local_vertex_major_ordering"]
    assert pat.local_primal_vertices.size > 0
    assert np.array_equal(mat.metadata.get("bddc_primal_vertices_local"), pat.local_primal_vertices)
    r = 0.3
    _, _, kr = getattr(op, "build_bddc_regularized_matrix")(r).getValuesCSR()
    assert rel_err(kr, (1.0 - r) * K_o + r * pat.elastic_values) <= PLAIN_RTOL
    _, _, ke = getattr(op, "build_bddc_elastic_matrix")().getValuesCSR()
    assert np.array_equal(ke, pat.elastic_values)
    handle = mat.handle
    op.reduction(1.0)
    op.constitutive_problem_stress_tangent(U)
    assert op.build_bddc_tangent_matrix().handle == handle  # updated in place
    # the mixed form (plastic corrections in compensated FP32) against the FP64 tangent
    op.reduction(1.2)
    op.tangent_form = "mixed"
    op.constitutive_problem_stress_tangent(U)
    _, _, km = op._build_bddc_regularized_matrix(r).getValuesCSR()
    err = rel_err(km, (1.0 - r) * K_o + r * pat.elastic_values)
    print(f"BDDC {dim}D {et}: mixed regularised subdomain tangent error {err:.2e}")
    assert err <= 1.0e-6
    op.release_petsc_caches()


def test_bddc_predictor_needs_matching_moduli(oracle):
    """A subdomain pattern prepared with other elastic moduli than the operator's: the subdomain
    tangent falls back to the full contraction of the operator's DS (still the reference's result)."""
    from slope_stability_petsc4py_gb300 import ConstitutiveOperator, prepare_bddc_subdomain_pattern, synthetic

    mats = synthetic.MaterialSet.layered(4, seed=5)
    mesh = synthetic.slope_mesh_3d(6, 3, 3, elem_type="P2", n_layers=4)
    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=float(mats.psi[i]), young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=20.0, gamma_unsat=20.0) for i in range(mats.c0.size)]
    op = ConstitutiveOperator.from_mesh(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs, elem_type="P2")
    other = [dict(sp, young=1.5 * sp["young"]) for sp in specs]
    pat = prepare_bddc_subdomain_pattern(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, other,
                                         (0, mesh.n_nodes), elem_type="P2",
                                         overlap_local_int_indices=op.owned_tangent_pattern.local_int_indices)
    op.set_bddc_subdomain_pattern(pat)
    op.reduction(1.2)
    op.constitutive_problem_stress_tangent(synthetic.displacement_field(mesh, mats, amplitude=0.05, seed=7))
    DS = np.asarray(op._owned_local_DS)[:, pat.overlap_local_positions]
    K_o = oracle.tangent_scatter(3, pat.dphi1, pat.dphi2, pat.dphi3, np.ascontiguousarray(DS.T),
                                 pat.local_assembly_weight, pat.scatter_map, pat.n_q, pat.nnz)
    K_o[pat.constrained_diag_positions] = 1.0
    _, _, vals = op._build_bddc_tangent_matrix().getValuesCSR()
    assert not op._bddc["predictor_ok"]
    assert rel_err(vals, K_o) <= PLAIN_RTOL
