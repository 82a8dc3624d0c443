"""Composite regularised builds copy the tangent's starting values on a second stream while the
strain and return mapping run (``_stage_values``).  Over a sequence of states, changes of r,
interleaved tangent builds and host outputs, the results must equal those of builds that copy on
the caller's stream."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _op(mesh, mats, staged):
    from slope_stability_petsc4py_gb300 import ConstitutiveOperator

    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=0.0, young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=20.0, gamma_unsat=20.0) for i in range(mats.c0.size)]
    op = ConstitutiveOperator.from_mesh(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs,
                                        elem_type=mesh.elem_type)
    op.stage_values = staged
    return op


@pytest.mark.parametrize("form,copy,concurrent", [("plain", "kernel", False), ("mixed", "kernel", False),
                                                  ("plain", "memcpy", True), ("mixed", "memcpy", True)])
def test_staged_values_copy_gives_the_same_matrices(cuda_device, form, copy, concurrent):
    """The staged copy of the starting values (by the SM copy kernel or a memcpy; restoring only
    the rows the previous build changed where it can) and the force on a second stream give the
    matrices and forces of one-stream, unstaged builds that copy every starting value, over states
    whose plastic sets grow, shrink and move, with r changes, tangent builds and host outputs."""
    from slope_stability_petsc4py_gb300 import _lib, synthetic

    mats = synthetic.MaterialSet.layered(4, seed=3)
    mesh = synthetic.slope_mesh_3d(12, 5, 6, elem_type="P2", n_layers=4)
    ops = (_op(mesh, mats, True), _op(mesh, mats, False))
    for op in ops:
        op.tangent_form = form
    ops[0].values_copy, ops[0].concurrent_force = copy, concurrent
    ops[1].values_copy, ops[1].concurrent_force, ops[1].incremental_values = "memcpy", False, False
    seq = [(0.010, 1, 0.3, "device"), (0.025, 2, 0.3, "device"), (0.006, 3, 0.3, "tangent"),
           (0.030, 4, 0.5, "device"), (0.015, 5, 0.5, "host"), (0.020, 6, 0.5, "device"), (0.004, 8, 0.3, "device")]
    for amp, seed, r, kind in seq:
        U = synthetic.displacement_field(mesh, mats, amplitude=amp, seed=seed)
        vals, forces = [], []
        for op in ops:
            op.host_outputs = kind == "host"
            if kind == "tangent":
                F, K = op.build_F_K_tangent_all(1.2, U)
            else:
                F, K = op.build_F_K_regularized_all_free(1.2, U, r)
            v = K.getValuesCSR()[2] if kind == "host" else K.values.cpu().numpy()
            vals.append(np.array(v, copy=True))
            forces.append(np.asarray(F.cpu().numpy() if hasattr(F, "cpu") else F, dtype=np.float64).copy())
        err = rel_err(vals[0], vals[1])
        print(f"{kind} amp {amp} r {r}: staged / incremental vs unstaged full-copy values {err:.2e}")
        # the corrections' CSR reductions run in an unspecified order: equal up to rounding
        assert err <= 1e-14
        assert rel_err(forces[0], forces[1]) <= 1e-14
    _lib.raise_on_device_status()


@pytest.mark.parametrize("form,dim", [("plain", 3), ("mixed", 3), ("plain", 2), ("mixed", 2)])
def test_captured_build_replays_match_direct_builds(cuda_device, form, dim):
    """capture_regularized_build: replays on U updated in place give the direct builds' F and K
    (3D P2, and 2D P4 with the binned plane-strain return mapping)."""
    import torch

    from slope_stability_petsc4py_gb300 import _lib, synthetic

    mats = synthetic.MaterialSet.layered(4, seed=3)
    mesh = (synthetic.slope_mesh_3d(12, 5, 6, elem_type="P2", n_layers=4) if dim == 3
            else synthetic.slope_mesh_2d(12, 8, elem_type="P4", n_layers=4))
    cap, ref = _op(mesh, mats, True), _op(mesh, mats, True)
    for op in (cap, ref):
        op.tangent_form, op.host_outputs = form, False
    U0 = synthetic.displacement_field(mesh, mats, amplitude=0.01, seed=1)
    U = torch.as_tensor(U0, device="cuda").clone()
    run = cap.capture_regularized_build(1.2, U, 0.3)
    for amp, seed in ((0.02, 2), (0.005, 3), (0.03, 4)):
        Un = synthetic.displacement_field(mesh, mats, amplitude=amp, seed=seed)
        U.copy_(torch.as_tensor(Un, device="cuda"))
        F, K = run.replay()
        F_ref, K_ref = ref.build_F_K_regularized_all_free(1.2, torch.as_tensor(Un, device="cuda"), 0.3)
        torch.cuda.synchronize()
        err_k = rel_err(K.values.cpu().numpy(), K_ref.values.cpu().numpy())
        err_f = rel_err(F.cpu().numpy(), F_ref.cpu().numpy())
        print(f"amp {amp}: replay vs direct K {err_k:.2e}, F {err_f:.2e}")
        assert err_k <= 1e-14 and err_f <= 1e-14
        assert torch.equal(cap._branch, ref._branch)
    _lib.raise_on_device_status()


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_incremental_host_refresh_gives_full_copies(cuda_device, form):
    """Host outputs: the pinned mirror refreshed row by row (rows of the previous and current
    plastic elements) equals a full device -> host copy, over states whose plastic sets grow,
    shrink and move, with r changes, tangent builds and device-output builds in between."""
    from slope_stability_petsc4py_gb300 import _lib, synthetic

    mats = synthetic.MaterialSet.layered(4, seed=3)
    mesh = synthetic.slope_mesh_3d(12, 5, 6, elem_type="P2", n_layers=4)
    inc, full = _op(mesh, mats, True), _op(mesh, mats, True)
    full.incremental_host_copy = False
    for op in (inc, full):
        op.tangent_form = form
    seq = [(0.010, 1, 0.3, "host"), (0.025, 2, 0.3, "host"), (0.006, 3, 0.3, "host"), (0.030, 4, 0.3, "tangent"),
           (0.015, 5, 0.3, "host"), (0.020, 6, 0.3, "device"), (0.020, 7, 0.3, "host"), (0.004, 8, 0.3, "host"),
           (0.012, 9, 0.5, "host"), (0.018, 10, 0.5, "host")]
    _lib.TRACE = []
    try:
        for amp, seed, r, kind in seq:
            U = synthetic.displacement_field(mesh, mats, amplitude=amp, seed=seed)
            vals = []
            for op in (inc, full):
                op.host_outputs = kind != "device"
                if kind == "tangent":
                    _F, K = op.build_F_K_tangent_all(1.2, U)
                else:
                    _F, K = op.build_F_K_regularized_all_free(1.2, U, r)
                vals.append(np.array(K.getValuesCSR()[2] if op.host_outputs else K.values.cpu().numpy(), copy=True))
            err = rel_err(vals[0], vals[1])
            print(f"{kind} amp {amp} r {r}: incremental vs full host copy {err:.2e}")
            assert err <= 1e-14
        refreshes = sum(1 for name, _a, _b in _lib.TRACE if name.startswith("ssp_copy_rows_out"))
    finally:
        _lib.TRACE = None
    _lib.raise_on_device_status()
    print(f"{refreshes} row-wise refreshes")
    # host builds right after a synced host build with the same r: 2nd, 3rd, 8th and 10th
    assert refreshes >= 4


def test_copy_out_into_pinned_memory(cuda_device):
    """ssp_copy_out / ssp_copy_rows_out into a pinned torch tensor (device-mapped host memory)."""
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    n_rows, per = 1000, 7
    src = torch.randn(n_rows * per, dtype=torch.float64, device="cuda")
    host = torch.zeros(n_rows * per, dtype=torch.float64, pin_memory=True)
    assert _lib.host_writable(host.data_ptr())
    assert not _lib.host_writable(torch.zeros(4, dtype=torch.float64).data_ptr())  # pageable
    _lib.call("ssp_copy_out", _lib.ptr(src), src.numel(), host.data_ptr(), _lib.stream_handle())
    torch.cuda.synchronize()
    assert torch.equal(host, src.cpu())
    host.zero_()
    indptr = torch.arange(0, n_rows * per + 1, per, dtype=torch.int32, device="cuda")
    mark = (torch.arange(n_rows, device="cuda") % 3 == 0).to(torch.uint8)
    _lib.call("ssp_copy_rows_out", _lib.ptr(src), _lib.ptr(indptr), _lib.ptr(mark), n_rows, src.numel(),
              host.data_ptr(), _lib.stream_handle())
    torch.cuda.synchronize()
    rows = mark.cpu().numpy().astype(bool).repeat(per)
    expect = np.where(rows, src.cpu().numpy(), 0.0)
    assert np.array_equal(host.numpy(), expect)
    # ragged rows (0 to 9 values, odd and even starts and ends: scalar heads / tails around the
    # 16-byte body), to the host and device to device
    lengths = np.random.default_rng(3).integers(0, 10, size=997)
    rp = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int32)
    nnz = int(rp[-1])
    src = torch.randn(nnz, dtype=torch.float64, device="cuda")
    mark = torch.as_tensor(np.random.default_rng(4).random(lengths.size) < 0.5, device="cuda").to(torch.uint8)
    indptr = torch.as_tensor(rp, device="cuda")
    sel = np.repeat(mark.cpu().numpy().astype(bool), lengths)
    host = torch.zeros(nnz, dtype=torch.float64, pin_memory=True)
    _lib.call("ssp_copy_rows_out", _lib.ptr(src), _lib.ptr(indptr), _lib.ptr(mark), lengths.size, nnz,
              host.data_ptr(), _lib.stream_handle())
    dev = torch.zeros(nnz, dtype=torch.float64, device="cuda")
    _lib.call("ssp_copy_rows_device", _lib.ptr(src), _lib.ptr(indptr), _lib.ptr(mark), lengths.size, nnz,
              _lib.ptr(dev), _lib.stream_handle())
    dev2 = torch.zeros(nnz, dtype=torch.float64, device="cuda")  # the small grid of a staged restore
    _lib.call("ssp_copy_rows_device_share", _lib.ptr(src), _lib.ptr(indptr), _lib.ptr(mark), lengths.size, nnz,
              _lib.ptr(dev2), 2, _lib.stream_handle())
    torch.cuda.synchronize()
    expect = np.where(sel, src.cpu().numpy(), 0.0)
    assert np.array_equal(host.numpy(), expect)
    assert np.array_equal(dev.cpu().numpy(), expect)
    assert np.array_equal(dev2.cpu().numpy(), expect)
    with pytest.raises(_lib.SSPError):  # 1..8 blocks per SM
        _lib.call("ssp_copy_rows_device_share", _lib.ptr(src), _lib.ptr(indptr), _lib.ptr(mark), lengths.size,
                  nnz, _lib.ptr(dev2), 9, _lib.stream_handle())
    _lib.raise_on_device_status()
