"""BDDC subdomain pattern, host part (no GPU): element/node selection, local square CSR pattern and
scatter map, Dirichlet diagonals, adjacency, primal vertices and overlap positions, bit for bit
against the reference's ``prepare_bddc_subdomain_pattern`` (golden fixtures ``bddc_*.npz``)."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import golden, golden_files

STRUCTURE_KEYS = ("local_elements", "local_nodes", "local_global_dofs", "local_q_mask", "scatter_map",
                  "constrained_diag_positions", "local_dirichlet_dofs", "local_adjacency_indptr",
                  "local_adjacency_indices", "local_primal_vertices", "local_int_indices", "overlap_local_positions")


def _structure(g, **kw):
    from slope_stability_petsc4py_gb300.bddc import bddc_local_structure

    args = dict(n_q=int(g["n_q"]), overlap_local_int_indices=g["overlap_local_int_indices"],
                adjacency_source=str(g["adjacency_source"]), corner_only_primals=bool(g["corner_only_primals"]))
    args.update(kw)
    return bddc_local_structure(g["coord"], g["elem"], g["q_mask"], tuple(g["owned_node_range"]), **args)


@pytest.mark.parametrize("name", golden_files("bddc_"))
def test_bddc_local_structure_bit_exact_with_reference(name):
    g = golden(name)
    s = _structure(g)
    for key in STRUCTURE_KEYS:
        want, got = np.asarray(g[key]), np.asarray(s[key])
        if want.size == 0 and got.size == 0:
            continue
        assert want.shape == got.shape and np.array_equal(want, got), key
    lp = s["local_matrix_pattern"]
    assert np.array_equal(lp.indptr, g["indptr"]) and np.array_equal(lp.indices, g["indices"])
    if g["local_field_dofs"].size:
        assert np.array_equal(np.stack(s["local_field_dofs"]), g["local_field_dofs"])
    assert np.array_equal(g["local_coord"], g["coord"][:, s["local_nodes"]])


@pytest.mark.parametrize("name", [n for n in golden_files("bddc_") if "empty" not in n])
def test_bddc_other_adjacency_sources_and_primal_modes(name):
    """csr adjacency = the local pattern; topology adjacency contains it (free columns) and is
    symmetric; 'none' is empty; primal vertices are free interface dofs."""
    g = golden(name)
    csr = _structure(g, adjacency_source="csr")
    topo = _structure(g, adjacency_source="topology", corner_only_primals=True)
    none = _structure(g, adjacency_source="none")
    assert np.array_equal(csr["local_adjacency_indptr"], g["indptr"])
    assert none["local_adjacency_indptr"].size == 0 and none["local_adjacency_indices"].size == 0
    ptr, idx = topo["local_adjacency_indptr"], topo["local_adjacency_indices"]
    n = ptr.size - 1
    A = np.zeros((n, n), dtype=bool)
    A[np.repeat(np.arange(n), np.diff(ptr)), idx] = True
    assert (A == A.T).all()
    lp = csr["local_matrix_pattern"]
    B = np.zeros((n, n), dtype=bool)
    B[np.repeat(np.arange(n), np.diff(lp.indptr)), lp.indices] = True
    assert not (B & ~A).any()
    prim = topo["local_primal_vertices"]
    assert np.all(np.diff(prim) > 0) and not np.isin(prim, topo["local_dirichlet_dofs"]).any()


def test_bddc_overlap_positions_reject_missing_points():
    g = golden("bddc_3d_P2_mid.npz")
    with pytest.raises(KeyError):
        ov = g["overlap_local_int_indices"]
        _structure(g, overlap_local_int_indices=ov[ov != g["local_int_indices"][3]])
    with pytest.raises(ValueError):
        _structure(g, adjacency_source="graph")
