"""The tensor-core path's shared-memory layout, descriptors and tensor-memory read-back.

``ssp_tc_tf32_probe`` runs one 128 x 112 x K tcgen05 TF32 product through exactly the operand
layout and descriptors of the P4 mixed-precision tangent kernel.  Inputs are TF32-representable,
so every product is exact in FP32 and only the FP32 summation rounds."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tf32(x):
    b = np.asarray(x, dtype=np.float32).view(np.uint32)
    return ((b + np.uint32(0x1000)) & np.uint32(0xFFFFE000)).view(np.float32)  # round half away on the magnitude


def _probe(A, B, K, convention):
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    Ad = torch.as_tensor(np.ascontiguousarray(A), device="cuda")
    Bd = torch.as_tensor(np.ascontiguousarray(B), device="cuda")
    D = torch.full((128, 112), np.nan, dtype=torch.float32, device="cuda")
    _lib.call("ssp_tc_tf32_probe", _lib.ptr(Ad), _lib.ptr(Bd), K, convention, _lib.ptr(D), _lib.stream_handle())
    return D.cpu().numpy()


@pytest.mark.parametrize("K", [8, 16, 24])
def test_tf32_tile_layout(cuda_device, K):
    from slope_stability_petsc4py_gb300 import _lib

    rng = np.random.default_rng(K)
    A = _tf32(rng.standard_normal((128, K)))
    B = _tf32(rng.standard_normal((112, K)))
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    errs = {}
    for conv in (0, 1):
        D = _probe(A, B, K, conv)
        errs[conv] = float(np.max(np.abs(D - ref)) / np.max(np.abs(ref))) if np.all(np.isfinite(D)) else np.inf
    print(f"K={K}: relative error, kernel convention {errs[0]:.2e}, swapped {errs[1]:.2e}")
    assert _lib.device_status(clear=True) == 0
    assert errs[0] <= 1e-6


def test_bounded_wait_expires_and_the_context_stays_usable(cuda_device):
    """The expiry path of the tensor-core kernels' bounded mbarrier waits: a wait that nothing
    completes gives up after its limit, sets SSP_DEV_TIMEOUT and frees the tensor memory; the next
    tensor-core build (P4 mixed tangent) runs and matches the FP64 tangent."""
    import torch

    from slope_stability_petsc4py_gb300 import ConstitutiveOperator, _lib, synthetic

    _lib.device_status(clear=True)
    expired = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    _lib.call("ssp_tc_wait_probe", 20000, _lib.ptr(expired), _lib.stream_handle())
    torch.cuda.synchronize()
    assert int(expired.item()) == 1
    assert _lib.device_status(clear=True) & 4  # SSP_DEV_TIMEOUT
    assert _lib.device_status(clear=True) == 0
    with pytest.raises(_lib.SSPError):  # limits outside 1 .. 2e9 clocks are refused before launch
        _lib.call("ssp_tc_wait_probe", 0, _lib.ptr(expired), _lib.stream_handle())

    mats = synthetic.MaterialSet.layered(4, seed=2)
    mesh = synthetic.slope_mesh_3d(4, 2, 2, elem_type="P4", n_layers=4)
    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=0.0, young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=20.0, gamma_unsat=20.0) for i in range(mats.c0.size)]
    op = ConstitutiveOperator.from_mesh(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs, elem_type="P4")
    U = synthetic.displacement_field(mesh, mats, amplitude=0.01, seed=4)
    op.reduction(1.1)
    op.constitutive_problem_stress_tangent(U)
    assert int((op._branch != 0).sum()) > 0
    kp = op.build_K_regularized(0.2).getValuesCSR()[2].copy()
    op.tangent_form = "mixed"
    op.constitutive_problem_stress_tangent(U)
    km = op.build_K_regularized(0.2).getValuesCSR()[2]
    assert np.max(np.abs(km - kp)) <= 1e-6 * np.max(np.abs(kp))
    assert _lib.device_status(clear=True) == 0
