"""Mixed-precision tangent form: error against the FP64 form, per tangent and per Newton step.

The mixed form keeps the return mapping's eigendecomposition, branch tests, plastic multipliers
and stresses and the CSR accumulation in FP64; it forms the plastic points' consistent tangent DS,
the strain, the force and the plastic-point products B^T (w D B) in compensated FP32
(double-float) arithmetic.  Tolerance of the mixed form: 1e-6 relative tangent error.
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
    plastic = None
    for r in (0.0, 0.3):
        # each form runs its own return mapping (the mixed one forms the plastic DS compensated)
        op.tangent_form = "plain"
        op.constitutive_problem_stress_tangent(U)
        plastic = int((op._branch != 0).sum())
        assert plastic > 0
        _, _, kp = op.build_K_regularized(r).getValuesCSR()
        kp = kp.copy()
        op.tangent_form = "mixed"
        op.constitutive_problem_stress_tangent(U)
        _, _, km = op.build_K_regularized(r).getValuesCSR()
        err = rel_err(km, kp)
        print(f"{elem_type} r={r}: mixed tangent max-norm relative error {err:.3e} ({plastic} plastic points)")
        assert 0.0 < err <= MIXED_RTOL
        fro = np.linalg.norm(km - kp) / np.linalg.norm(kp)
        assert fro <= MIXED_RTOL


def test_mixed_p2_moment_correction(cuda_device):
    """Straight-sided P2, mixed form: the correction of every plastic element in moment form (FP32
    after the FP64 DS - D_el) against the mixed point-by-point kernel and against the FP64 form, on
    a strongly yielding slope; the split by plastic-point count gives the same tangent."""
    from slope_stability_petsc4py_gb300 import synthetic

    mesh, mats, op = _operator(12, 5, 6)
    U = synthetic.displacement_field(mesh, mats, amplitude=0.08, seed=9)
    op.reduction(1.3)
    assert op.moment_min_points_mixed == 1
    op.tangent_form = "plain"
    op.constitutive_problem_stress_tangent(U)
    per_elem = (np.asarray(op._branch.cpu()).reshape(-1, op.owned_tangent_pattern.n_q) != 0).sum(axis=1)
    assert (per_elem > 0).sum() > 100 and (per_elem == 1).sum() > 0
    kp = op.build_K_regularized(0.2).getValuesCSR()[2].copy()
    assert op.owned_tangent_pattern.affine_p2  # decided at the first tangent build
    op.tangent_form = "mixed"
    out = {}
    for mm in (1, 0, 4):  # every plastic element, none (point by point), split at four points
        op.moment_min_points_mixed = mm
        op.constitutive_problem_stress_tangent(U)
        out[mm] = op.build_K_regularized(0.2).getValuesCSR()[2].copy()
    op.moment_min_points_mixed = 1
    e_mom, e_pt, e_split = rel_err(out[1], kp), rel_err(out[0], kp), rel_err(out[4], kp)
    print(f"P2 mixed tangent error: moment form {e_mom:.3e}, point by point {e_pt:.3e}, split {e_split:.3e}")
    assert 0.0 < e_mom <= MIXED_RTOL and e_pt <= MIXED_RTOL and e_split <= MIXED_RTOL
    assert rel_err(out[1], out[0]) <= MIXED_RTOL


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
    print(f"{elem_type}: strain error {err_e:.2e}, force error {err_f:.2e} (affine kernels {pat.affine})")
    assert pat.affine  # straight-sided tetrahedra: J^{-1} per element and the reference table
    assert err_e <= 1e-11 and err_f <= 1e-11
    torch.cuda.synchronize()


def test_mixed_strain_and_force_on_curved_elements(cuda_device):
    """Mid-edge nodes moved off their edges (curved P2 tetrahedra, gradients no longer J^{-T} ghat):
    the affine check fails and the mixed form reads the per-point gradients instead; errors as above."""
    from slope_stability_petsc4py_gb300 import ConstitutiveOperator, synthetic
    from slope_stability_petsc4py_gb300.distributed_tangent import overlap_strain_device, owned_force_device

    mats = synthetic.MaterialSet.layered(4, seed=1)
    mesh = synthetic.slope_mesh_3d(8, 4, 4, elem_type="P2", n_layers=4)
    coord = mesh.coord.copy()
    n_v = int(mesh.elem[:4].max()) + 1  # vertices first, then the edge nodes
    rng = np.random.default_rng(3)
    interior = np.all(mesh.q_mask[:, n_v:], axis=0)
    coord[:, n_v:][:, interior] += 0.02 * rng.standard_normal((3, int(interior.sum())))
    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=0.0, young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=20.0, gamma_unsat=20.0) for i in range(mats.c0.size)]
    op = ConstitutiveOperator.from_mesh(coord, mesh.elem, mesh.q_mask, mesh.material_id, specs, elem_type="P2")
    pat = op.owned_tangent_pattern
    U = synthetic.displacement_field(mesh, mats, amplitude=0.02, seed=8)
    E64 = overlap_strain_device(pat, U).cpu().numpy()
    Emx = overlap_strain_device(pat, U, mixed=True).cpu().numpy()
    assert pat.affine is False
    assert pat.affine_p2 is False  # the plain form reads the per-point gradients too
    op.reduction(1.1)
    op.constitutive_problem_stress_tangent(U)
    F64 = owned_force_device(pat, op._S_aos).cpu().numpy()
    Fmx = owned_force_device(pat, op._S_aos, mixed=True).cpu().numpy()
    err_e, err_f = rel_err(Emx, E64), rel_err(Fmx, F64)
    print(f"curved P2: strain error {err_e:.2e}, force error {err_f:.2e}")
    assert err_e <= 1e-11 and err_f <= 1e-11


def test_compensated_plastic_ds_matches_fp64(cuda_device):
    """ssp_constitutive_3d_sds_binned_mixed against the FP64 binned return mapping on random trial
    strains over four orders of magnitude: the same branches, bitwise the same stresses, and the
    plastic DS rows within 1e-10 of each row's size."""
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    rng = np.random.default_rng(17)
    n = 400_000
    E = rng.standard_normal((n, 6)) * np.repeat(np.array([1e-4, 1e-3, 3e-3, 1e-2]), n // 4)[:, None]
    young = rng.uniform(1e4, 5e4, n)
    nu = rng.uniform(0.2, 0.45, n)
    shear = young / (2 * (1 + nu))
    lame = young / (3 * (1 - 2 * nu)) - 2 * shear / 3
    phi = np.deg2rad(rng.uniform(20.0, 40.0, n))
    c_bar = 2 * rng.uniform(5.0, 30.0, n) * np.cos(phi)
    sin_phi = np.sin(phi)
    dev = [torch.as_tensor(np.ascontiguousarray(a), device="cuda") for a in (E, c_bar, sin_phi, shear, lame)]
    out = {}
    for entry in ("ssp_constitutive_3d_sds_binned", "ssp_constitutive_3d_sds_binned_mixed"):
        S = torch.empty((n, 6), dtype=torch.float64, device="cuda")
        DS = torch.empty((n, 36), dtype=torch.float64, device="cuda")
        br = torch.empty(n, dtype=torch.int8, device="cuda")
        scratch = torch.empty(3 * n + 4, dtype=torch.int32, device="cuda")
        _lib.call(entry, *[_lib.ptr(a) for a in dev], n, _lib.ptr(S), _lib.ptr(DS), _lib.ptr(br), _lib.ptr(scratch),
                  _lib.stream_handle())
        out[entry] = (S, DS, br)
    _lib.raise_on_device_status()
    S0, DS0, b0 = out["ssp_constitutive_3d_sds_binned"]
    S1, DS1, b1 = out["ssp_constitutive_3d_sds_binned_mixed"]
    assert torch.equal(b0, b1)
    assert torch.equal(S0, S1)
    counts = torch.bincount(b0.long(), minlength=5).cpu().numpy()
    plastic = (b0 >= 1) & (b0 <= 3)
    assert int(plastic.sum()) > 10_000
    err = ((DS1 - DS0).abs().max(dim=1).values / DS0.abs().max(dim=1).values)[plastic]
    same = (DS1 == DS0).all(dim=1)[plastic]
    print(f"branches {counts.tolist()}; plastic DS rows: max rel err {float(err.max()):.3e}, "
          f"median {float(err.median()):.3e}, FP64 fallback (bitwise equal) {float(same.float().mean()):.4f}")
    assert float(err.max()) <= 1e-10
    # the other rows are the FP64 path's own
    assert torch.equal(DS1[~plastic], DS0[~plastic])
