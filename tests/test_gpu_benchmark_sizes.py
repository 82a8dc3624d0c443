"""Parity at the sizes of the benchmarked configurations (GPU).

The small-mesh tests pin every kernel; these run the whole Newton iteration of the operator on the
2D P2 (20,000 triangles) and 3D P2 (100,800 tetrahedra) benchmark slopes and compare it with the
oracle's full restatement of the reference's iteration (its own pattern, geometry and elastic
values): stresses, tangents, owned force and CSR values to 1e-12 (plain FP64 form), the CSR pattern,
constrained diagonals and element -> CSR map bit for bit.  The states change between builds so the
shortcuts that only pay at size run as in a Newton solve: the FP32 elastic screen, the elastic
predictor with plastic corrections, the restore of only the rows the previous build changed, and
(3D) the barycentric P2 strain and force.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import PLAIN_RTOL

LAM, R = 1.1, 0.1
# mixed form: its 1e-6 bound on the tangent error; the force (residual) is formed in double-float
MIXED_K_RTOL, MIXED_F_RTOL = 1.0e-6, 1.0e-11


def _rel(torch, a, b) -> float:
    return float(((a - b).abs().max() / b.abs().max().clamp_min(1e-300)).item())


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["2d_p2_homo", "3d_p2_homo"])
def test_newton_iteration_matches_oracle_at_benchmark_size(name, cuda_device):
    import torch

    from oracle.newton_step import OracleNewtonStep
    from slope_stability_petsc4py_gb300 import ConstitutiveOperator, synthetic

    w = synthetic.config_workload(name)
    mesh = w.mesh
    op = ConstitutiveOperator.from_mesh(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, w.specs,
                                        elem_type=mesh.elem_type)
    op.host_outputs = False
    pat = op.owned_tangent_pattern
    states = [w.G + (f * w.amp) * w.V for f in (1.2, 0.9, 1.0)]
    for U in states[:-1]:  # earlier Newton iterates: the last build restores the rows these changed
        op.build_F_K_regularized_all_free(LAM, torch.as_tensor(U, device="cuda"), R)
    U = states[-1]
    U_dev = torch.as_tensor(U, device="cuda")
    F, K = op.build_F_K_regularized_all_free(LAM, U_dev, R)
    torch.cuda.synchronize()

    ref_step = OracleNewtonStep(mesh, w.specs)
    ref = ref_step.step(U, LAM, R)
    p = ref_step.p
    # pattern, constrained diagonals and element -> CSR map bit for bit
    assert np.array_equal(pat.local_matrix_pattern.indptr, p["indptr"])
    assert np.array_equal(pat.local_matrix_pattern.indices, p["indices"])
    assert np.array_equal(pat.constrained_diag_positions, p["constrained_diag_positions"])
    nld = pat.dim * pat.n_p
    se = torch.as_tensor(p["slot_elem"].astype(np.int64), device="cuda")
    cols = torch.as_tensor(p["slot_lrow"].astype(np.int64), device="cuda")[:, None] * nld + \
        torch.arange(nld, device="cuda")[None, :]
    assert torch.equal(pat.device["scatter_map"][se[:, None], cols], torch.as_tensor(p["slot_pos"], device="cuda"))

    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")  # noqa: E731
    S_o, DS_o, F_o, K_o = dev(ref["S"]), dev(ref["DS"]), dev(ref["F"][ref_step.free]), dev(ref["K"])
    plastic = float((op._branch != 0).float().mean().item())
    errs = {"S": _rel(torch, op._S_aos, S_o), "DS": _rel(torch, op._owned_local_DS.aos, DS_o),
            "F_free": _rel(torch, F, F_o), "K": _rel(torch, K.values, K_o)}
    print(f"{name}: {pat.n_local_int:,} points, {pat.nnz:,} nnz, plastic {plastic:.3f}, plain errors",
          {k: f"{v:.2e}" for k, v in errs.items()})
    assert 0.02 < plastic < 0.5  # the states yield: the return mapping's plastic branches run
    assert all(v <= PLAIN_RTOL for v in errs.values()), errs
    # stage by stage: the strain against the oracle's, the return mapping on the GPU's own strain
    from slope_stability_petsc4py_gb300.distributed_tangent import overlap_strain_device

    E_g = overlap_strain_device(pat, U_dev)
    S_gE, DS_gE = ref_step.constitutive(E_g.cpu().numpy(), LAM)
    stages = {"strain": _rel(torch, E_g, dev(ref["E"])), "S": _rel(torch, op._S_aos, dev(S_gE)),
              "DS": _rel(torch, op._owned_local_DS.aos, dev(DS_gE))}
    print(f"{name}: stage errors", {k: f"{v:.2e}" for k, v in stages.items()})
    assert all(v <= PLAIN_RTOL for v in stages.values()), stages
    if pat.dim == 3:
        assert pat.affine_p2 is True  # the barycentric P2 strain and force ran
        op.tangent_form = "mixed"
        op.build_F_K_regularized_all_free(LAM, torch.as_tensor(states[0], device="cuda"), R)
        F, K = op.build_F_K_regularized_all_free(LAM, U_dev, R)
        torch.cuda.synchronize()
        mk, mf = _rel(torch, K.values, K_o), _rel(torch, F, F_o)
        print(f"{name}: mixed tangent error {mk:.2e}, force error {mf:.2e}")
        assert mk <= MIXED_K_RTOL and mf <= MIXED_F_RTOL
