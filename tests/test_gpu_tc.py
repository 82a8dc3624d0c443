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
