"""Mixed-precision tangent form: error against the FP64 form, per tangent and per Newton step.

The mixed form keeps the return mapping (eigendecomposition, branch tests, plastic multipliers)
and the CSR accumulation in FP64 and takes the plastic-point products B^T (w D B) in FP32 with an
FP64-formed, hi/lo-split D B.  Tolerance of the spec mixed form: 1e-6 relative tangent error.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

MIXED_RTOL = 1.0e-6


def _operator(nx, ny, nz, layered=True, seed=1, elem_type="P2"):
    from slope_stability_petsc4py_gb300 import ConstitutiveOperator, synthetic

    mats = synthetic.MaterialSet.layered(4, seed=seed) if layered else synthetic.MaterialSet.homogeneous()
    mesh = synthetic.slope_mesh_3d(nx, ny, nz, elem_type=elem_type, n_layers=4 if layered else 1)
    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=0.0, young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=20.0, gamma_unsat=20.0) for i in range(mats.c0.size)]
    op = ConstitutiveOperator.from_mesh(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs,
                                        elem_type=elem_type)
    return mesh, mats, op


@pytest.mark.parametrize("elem_type,dims,amp", [("P2", (20, 8, 10), 0.02), ("P4", (10, 4, 5), 0.01)])
def test_mixed_tangent_error_bound(cuda_device, elem_type, dims, amp):
    """P2: FP32 CUDA-core products; P4: the tensor-core (tcgen05 TF32 split) contraction."""
    from slope_stability_petsc4py_gb300 import synthetic

    mesh, mats, op = _operator(*dims, elem_type=elem_type)
    U = synthetic.displacement_field(mesh, mats, amplitude=amp, seed=4)
    op.reduction(1.1)
    op.constitutive_problem_stress_tangent(U)
    plastic = int((op._branch != 0).sum())
    assert plastic > 0
    for r in (0.0, 0.3):
        op.tangent_form = "plain"
        _, _, kp = op.build_K_regularized(r).getValuesCSR()
        kp = kp.copy()
        op.tangent_form = "mixed"
        _, _, km = op.build_K_regularized(r).getValuesCSR()
        err = rel_err(km, kp)
        print(f"{elem_type} r={r}: mixed tangent max-norm relative error {err:.3e} ({plastic} plastic points)")
        assert 0.0 < err <= MIXED_RTOL
        fro = np.linalg.norm(km - kp) / np.linalg.norm(kp)
        assert fro <= MIXED_RTOL


@pytest.mark.parametrize("elem_type,dims", [("P2", (8, 4, 4)), ("P4", (4, 2, 2))])
def test_mixed_form_newton_iterations_unchanged(cuda_device, elem_type, dims):
    from slope_stability_petsc4py_gb300.newton_check import newton_compare, newton_iterations

    mesh, _mats, op = _operator(*dims, elem_type=elem_type)
    lam = 1.0
    it_plain, res_plain, U_plain = newton_iterations(op, mesh, form="plain", lam=lam)
    it_mixed, res_mixed, U_mixed = newton_iterations(op, mesh, form="mixed", lam=lam)
    print(f"{elem_type}: Newton iterations plain {it_plain} (res {res_plain:.2e}), mixed {it_mixed} (res {res_mixed:.2e})")
    assert res_plain < 1e-9 and res_mixed < 1e-9
    assert it_mixed == it_plain
    assert np.linalg.norm(U_mixed - U_plain) <= 1e-8 * np.linalg.norm(U_plain)
    cmp = newton_compare(op, mesh, lam=lam)
    for h in cmp["history"][:-1]:
        print(f"  step {h['it']}: residual {h['residual']:.3e} tangent err {h['tangent_rel_err']:.2e} "
              f"force err {h['force_rel_err']:.2e} update err {h['update_rel_err']:.2e}")
        assert h["tangent_rel_err"] <= MIXED_RTOL
        assert h["force_rel_err"] <= 1e-11
        assert h["update_rel_err"] <= 1e-4


@pytest.mark.parametrize("elem_type,dims,amp", [("P2", (20, 8, 10), 0.02), ("P4", (8, 3, 4), 0.01)])
def test_compensated_strain_and_force_match_fp64(cuda_device, elem_type, dims, amp):
    """The mixed form's strain and force (compensated double-float on the FP32 pipe) against the
    FP64 kernels: max-norm relative error ~1e-13, bounded here by 1e-11."""
    import torch

    from slope_stability_petsc4py_gb300 import synthetic
    from slope_stability_petsc4py_gb300.distributed_tangent import overlap_strain_device, owned_force_device

    mesh, mats, op = _operator(*dims, elem_type=elem_type)
    pat = op.owned_tangent_pattern
    U = synthetic.displacement_field(mesh, mats, amplitude=amp, seed=8)
    E64 = overlap_strain_device(pat, U).cpu().numpy()
    Emx = overlap_strain_device(pat, U, mixed=True).cpu().numpy()
    err_e = rel_err(Emx, E64)
    op.reduction(1.1)
    op.constitutive_problem_stress_tangent(U)
    S = op._S_aos
    F64 = owned_force_device(pat, S).cpu().numpy()
    Fmx = owned_force_device(pat, S, mixed=True).cpu().numpy()
    err_f = rel_err(Fmx, F64)
    print(f"{elem_type}: strain error {err_e:.2e}, force error {err_f:.2e}")
    assert err_e <= 1e-11 and err_f <= 1e-11
    torch.cuda.synchronize()
