"""Learned branch proposal: kernels against the oracle, training, and what the network gains.

The network (6 -> 32 -> 32 -> 5) is trained on the GPU by the library's own forward/backward
(``ssp_mlp_loss_grad``) and Adam (``ssp_mlp_adam``) kernels on (features, branch) pairs that the
exact return mapping emits over a sequence of continuation states.  The exact kernel still
decides every point, so the learned path must give the plain path's results; its gain is less
branch divergence per warp, hence less time.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import PLAIN_RTOL, rel_err

pytestmark = pytest.mark.gpu


def _strain_batch(n, seed):
    rng = np.random.default_rng(seed)
    E = rng.standard_normal((n, 6)) * np.repeat(np.array([1e-4, 1e-3, 3e-3, 1e-2]), n // 4)[:, None]
    young, nu = 2.0e4, 0.45
    shear = np.full(n, young / (2 * (1 + nu)))
    lame = np.full(n, young / (3 * (1 - 2 * nu))) - 2 * shear / 3
    c_bar = np.full(n, 2 * 8.0 * np.cos(np.deg2rad(35.0)))
    sin_phi = np.full(n, np.sin(np.deg2rad(35.0)))
    return E, c_bar, sin_phi, shear, lame


def test_features_match_oracle(cuda_device, oracle):
    import torch

    from slope_stability_petsc4py_gb300 import learned

    arrs = _strain_batch(20000, 1)
    dev = [torch.as_tensor(a, device="cuda") for a in arrs]
    X = learned.features(*dev).cpu().numpy()
    X_o = oracle.branch_features(*arrs)
    assert np.max(np.abs(X - X_o)) <= 1e-4 * max(1.0, np.max(np.abs(X_o)))


def test_mlp_gradient_matches_oracle(cuda_device, oracle):
    import torch

    from slope_stability_petsc4py_gb300 import learned

    rng = np.random.default_rng(3)
    n = 5000
    X = rng.standard_normal((n, 6)).astype(np.float32)
    y = rng.integers(0, 5, n).astype(np.int8)
    params = learned.init_params(seed=7)
    params[1440:] = rng.standard_normal(5).astype(np.float32) * 0.1
    model = learned.BranchProposal(params)
    loss, grad, hits = model.loss_grad(torch.as_tensor(X, device="cuda"), torch.as_tensor(y, device="cuda"))
    loss_o, grad_o, hits_o = oracle.mlp_loss_grad(params, X, y)
    assert abs(float(loss.item()) - loss_o) <= 1e-4 * abs(loss_o)
    assert rel_err(grad.cpu().numpy(), grad_o) <= 1e-4
    assert int(hits.item()) == hits_o
    # the FP32 prediction is the oracle's argmax
    z, _ = oracle.mlp_forward(params, X)
    Xd = torch.as_tensor(X, device="cuda")
    pred = model.predict(Xd, bf16=False).cpu().numpy()
    margin = np.sort(z, axis=1)[:, -1] - np.sort(z, axis=1)[:, -2]
    sure = margin > 1e-4
    assert np.array_equal(pred[sure], np.argmax(z, axis=1)[sure])
    # BF16 inference: CUDA cores and tensor cores (tcgen05 kind::f16) agree except where BF16
    # rounding makes the top two logits tie (their accumulation orders differ)
    p_cc = model.predict(Xd, bf16=True, tensor_cores=False).cpu().numpy()
    p_tc = model.predict(Xd, bf16=True, tensor_cores=True).cpu().numpy()
    clear = margin > 0.05 * np.maximum(1.0, np.abs(z).max(axis=1))
    assert np.array_equal(p_cc[clear], p_tc[clear])
    assert np.mean(p_cc == p_tc) > 0.99
    assert np.mean(p_tc[clear] == np.argmax(z, axis=1)[clear]) > 0.99


def _trained_model(op, mesh, mats):
    from slope_stability_petsc4py_gb300 import learned, synthetic

    states = []
    for k, lam in enumerate(np.linspace(1.0, 1.4, 10)):  # a strength-reduction sequence
        amp = 0.004 + 0.004 * k  # a widening shear band
        states.append((float(lam), synthetic.displacement_field(mesh, mats, amplitude=amp, seed=11 + k)))
    X, y = learned.collect_training_data(op, states)
    model = learned.BranchProposal(seed=0)
    hist = model.train(X, y, epochs=8, batch=2048, lr=3e-3)
    return model, X, y, hist


def test_training_learns_the_branches_and_gains(cuda_device):
    import torch

    from slope_stability_petsc4py_gb300 import ConstitutiveOperator, _lib, learned, synthetic

    mats = synthetic.MaterialSet.layered(4, seed=2)
    mesh = synthetic.slope_mesh_3d(16, 6, 8, elem_type="P2", n_layers=4)
    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=0.0, young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=20.0, gamma_unsat=20.0) for i in range(4)]
    op = ConstitutiveOperator.from_mesh(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs, elem_type="P2")
    model, X, y, hist = _trained_model(op, mesh, mats)
    counts = np.bincount(y.cpu().numpy(), minlength=5)
    majority = counts.max() / counts.sum()
    acc = model.accuracy(X, y)
    print("training history (loss, acc):", [(round(a, 4), round(b, 4)) for a, b in hist])
    print("branch counts", counts.tolist(), "majority", round(majority, 4), "bf16 accuracy", round(acc, 4))
    assert hist[-1][0] < hist[0][0]
    assert acc > majority + 0.5 * (1.0 - majority)

    # a held-out state: results identical to the plain paths, less divergence per warp
    U = synthetic.displacement_field(mesh, mats, amplitude=0.03, seed=99)
    outs = {}
    for mode in ("unsorted", "binned", "learned"):
        op.return_mapping = mode
        op.branch_model = model
        op.reduction(1.25)
        op.constitutive_problem_stress_tangent(U)
        outs[mode] = (op._S_aos.clone(), op._owned_local_DS.aos.clone(), op._branch.clone())
    # the single-pass kernel and the binned passes: the same branches, results to a few ulps
    assert torch.equal(outs["learned"][2], outs["unsorted"][2])
    assert rel_err(outs["learned"][0].cpu().numpy(), outs["unsorted"][0].cpu().numpy()) <= 1e-14
    assert rel_err(outs["learned"][1].cpu().numpy(), outs["unsorted"][1].cpu().numpy()) <= 1e-14
    assert rel_err(outs["binned"][1].cpu().numpy(), outs["unsorted"][1].cpu().numpy()) <= PLAIN_RTOL
    # the learned path runs the binned path's per-point code in another order: bit-identical results
    for a, b in zip(outs["learned"], outs["binned"]):
        assert torch.equal(a, b)

    br = outs["unsorted"][2]
    n = br.numel()
    scratch = op._scratch
    # the screen's list (point order) and the five proposal bins over it
    listed, bins = learned.proposal_bins(scratch, n)
    counts_l = [b.numel() for b in bins]
    order = torch.cat(bins)
    assert order.numel() == listed.numel()
    assert torch.equal(torch.sort(order).values, torch.sort(listed).values)
    screened = torch.ones(n, dtype=torch.bool, device=br.device)
    screened[listed] = False
    assert (br[screened] == 0).all()
    print(f"listed by the screen {listed.numel()} of {n}, bins {counts_l}")
    mix_natural = learned.warp_branch_mix(br, listed)
    mix_learned = learned.warp_branch_mix(br, order)
    print(f"distinct branches per warp over the listed points: screen order {mix_natural:.3f}, "
          f"learned bins {mix_learned:.3f}")
    assert mix_learned < mix_natural


def test_binning_sources_gain_time_over_the_unsorted_return_mapping(cuda_device):
    """Time of the return mapping on the 100,800-element benchmark slope (1.1 M points) with each
    binning source -- none (unsorted, one divergent pass), the exact screen-decide binning, the
    previous iteration's branches, the trained network's proposal -- with identical results.  Each
    binned form must beat the unsorted pass by at least 5 %."""
    import torch

    from slope_stability_petsc4py_gb300 import ConstitutiveOperator, learned, synthetic

    w = synthetic.config_workload("3d_p2_homo")
    mesh = w.mesh
    op = ConstitutiveOperator.from_mesh(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, w.specs,
                                        elem_type=mesh.elem_type)
    op.host_outputs = False
    train = [(float(lam), torch.as_tensor(w.G + (f * w.amp) * w.V, device="cuda"))
             for lam, f in zip(np.linspace(1.0, 1.3, 6), np.linspace(0.5, 1.6, 6))]
    X, y = learned.collect_training_data(op, train)
    model = learned.BranchProposal(seed=0)
    model.train(X, y, epochs=4, batch=8192, lr=3e-3)
    op.branch_model = model
    U = torch.as_tensor(w.G + (1.05 * w.amp) * w.V, device="cuda")  # a state outside the training set
    op.reduction(1.1)
    times, outs = {}, {}
    for mode in ("unsorted", "binned", "previous", "learned"):
        op.return_mapping = mode
        op.constitutive_problem_stress_tangent(U)  # warm-up (and the previous codes for "previous")
        ts = []
        for _ in range(7):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            op.constitutive_problem_stress_tangent(U)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        times[mode] = float(np.median(ts))
        outs[mode] = (op._S_aos.clone(), op._owned_local_DS.aos.clone(), op._branch.clone())
    print("return mapping, ms:", {k: round(v, 3) for k, v in times.items()},
          "plastic fraction", round(float((outs["binned"][2] != 0).float().mean()), 4))
    for mode in ("binned", "previous", "learned"):
        assert torch.equal(outs[mode][2], outs["unsorted"][2])
        assert rel_err(outs[mode][0].cpu().numpy(), outs["unsorted"][0].cpu().numpy()) <= 1e-14
        assert rel_err(outs[mode][1].cpu().numpy(), outs["unsorted"][1].cpu().numpy()) <= PLAIN_RTOL
        assert times[mode] < 0.95 * times["unsorted"], (mode, times)
