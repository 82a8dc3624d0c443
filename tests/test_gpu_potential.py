"""The potential energy of the Mohr-Coulomb model (the scalar the direct SSR continuation
differences in lambda) through the C ABI and ConstitutiveOperator.potential_energy, against the
reference's fixtures and the oracle."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import PLAIN_RTOL, golden

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _clean_status(cuda_device):
    from slope_stability_petsc4py_gb300 import _lib

    _lib.device_status(clear=True)
    yield
    assert _lib.device_status(clear=True) == 0


def _potential(dim, E_aos, mats, weight=None):
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    n = E_aos.shape[0]
    dv = [_lib.to_device(np.ascontiguousarray(a), torch.float64) for a in (E_aos, *mats)]
    psi = torch.empty(n, dtype=torch.float64, device="cuda")
    br = torch.empty(n, dtype=torch.int8, device="cuda")
    total = part = w = None
    if weight is not None:
        w = _lib.to_device(np.ascontiguousarray(weight), torch.float64)
        part = torch.empty(_lib.POTENTIAL_PARTIALS, dtype=torch.float64, device="cuda")
        total = torch.empty(1, dtype=torch.float64, device="cuda")
    _lib.call("ssp_potential_energy", dim, *[_lib.ptr(a) for a in dv], _lib.ptr(w), n, _lib.ptr(psi), _lib.ptr(br),
              _lib.ptr(part), _lib.ptr(total), _lib.stream_handle())
    out = psi.cpu().numpy(), br.cpu().numpy()
    return out if total is None else out + (float(total.item()),)


@pytest.mark.parametrize("dim", [3, 2])
def test_potential_kernel_matches_reference(oracle, dim):
    """Per-point energy densities against the reference's potential_3D / potential_2D, branches
    against the oracle's, and the weighted sum against a host sum."""
    g = golden("potential.npz")
    E = g["E3"] if dim == 3 else g["E2"]
    fn = oracle.potential_3d if dim == 3 else oracle.potential_2d
    rng = np.random.default_rng(4)
    for key in ("bench", "test"):
        tag = f"{key}_{dim}d"
        mats = tuple(g[f"{tag}_{k}"] for k in ("c_bar", "sin_phi", "shear", "bulk", "lame"))
        ref = g[f"{tag}_psi"]
        w = rng.uniform(0.1, 1.0, ref.size)
        psi, br, total = _potential(dim, E.T, mats, w)
        scale = np.abs(ref).max()
        np.testing.assert_allclose(psi, ref, rtol=1e-10, atol=PLAIN_RTOL * scale)
        _, br_o = fn(E, *mats, with_branch=True)
        assert np.mean(br == br_o) >= 0.995
        assert abs(total - float(np.dot(w, ref))) <= PLAIN_RTOL * float(np.dot(w, np.abs(ref)))


def test_potential_kernel_edge_cases():
    """No points: the total is 0 and nothing else runs; a bad dimension is refused before a launch;
    the sum is the same bit for bit on every call."""
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    part = torch.empty(_lib.POTENTIAL_PARTIALS, dtype=torch.float64, device="cuda")
    total = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
    _lib.call("ssp_potential_energy", 3, None, None, None, None, None, None, _lib.ptr(part), 0, None, None,
              _lib.ptr(part), _lib.ptr(total), _lib.stream_handle())
    assert float(total.item()) == 0.0
    with pytest.raises(_lib.SSPError):
        _lib.call("ssp_potential_energy", 4, None, None, None, None, None, None, None, 0, None, None, None, None,
                  _lib.stream_handle())
    rng = np.random.default_rng(9)
    n = 300_001  # more blocks than partials: the grid-stride path
    E = rng.standard_normal((n, 6)) * 2e-3
    mats = (np.full(n, 8.0), np.full(n, 0.5), np.full(n, 7000.0), np.full(n, 2.0e4), np.full(n, 1.5e4))
    w = rng.uniform(0.1, 1.0, n)
    a = _potential(3, E, mats, w)[2]
    b = _potential(3, E, mats, w)[2]
    assert a == b


def _operator(mesh, mats, et, owned_range):
    from slope_stability_petsc4py_gb300 import ConstitutiveOperator
    from slope_stability_petsc4py_gb300.distributed_tangent import prepare_owned_tangent_pattern
    from slope_stability_petsc4py_gb300.materials import heterogenous_materials

    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=float(mats.psi[i]), young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=20.0, gamma_unsat=20.0) for i in range(mats.c0.size)]
    pat = prepare_owned_tangent_pattern(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs, owned_range,
                                        elem_type=et, include_legacy_scatter=False, keep_slot_metadata=False)
    n_int = mesh.elem.shape[1] * pat.n_q
    c0, phi, psi, shear, bulk, lame, _ = heterogenous_materials(mesh.material_id, np.ones(n_int, bool), pat.n_q, specs)
    op = ConstitutiveOperator(B=None, c0=c0, phi=phi, psi=psi, Davis_type="B", shear=shear, bulk=bulk, lame=lame,
                              WEIGHT=np.zeros(0), n_strain=pat.n_strain, n_int=n_int, dim=pat.dim, q_mask=mesh.q_mask)
    op.set_owned_tangent_pattern(pat, constitutive_mode="overlap")
    return op


@pytest.mark.parametrize("dim,et,dims", [(3, "P2", (8, 4, 5)), (2, "P2", (14, 8))])
def test_operator_potential_energy_against_oracle(oracle, dim, et, dims):
    """ConstitutiveOperator.potential_energy(U) against the oracle chain (strain, energy density,
    weighted sum); two owned node ranges that split the mesh sum to the whole mesh's energy."""
    from slope_stability_petsc4py_gb300 import synthetic

    mats = synthetic.MaterialSet.layered(4, seed=2)
    mesh = (synthetic.slope_mesh_3d(*dims, elem_type=et, n_layers=4) if dim == 3
            else synthetic.slope_mesh_2d(*dims, elem_type=et, n_layers=4))
    U = synthetic.displacement_field(mesh, mats, amplitude=0.05, seed=3)
    op = _operator(mesh, mats, et, (0, mesh.n_nodes))
    with pytest.raises(ValueError):
        op.potential_energy(U)  # no reduction yet
    lam = 1.1
    op.reduction(lam)
    J = op.potential_energy(U)
    assert J == op.potential_energy(U)  # deterministic
    pat = op.owned_tangent_pattern
    idx = pat.local_int_indices
    cb, sp = oracle.reduction(op.c0[idx], op.phi[idx], op.psi[idx], lam, "B")
    u_ov = U.reshape(-1, order="F")[pat.overlap_global_dofs]
    if dim == 3:
        E = oracle.strain_3d(pat.dphi1, pat.dphi2, pat.dphi3, u_ov, pat.overlap_element_dof_lids, pat.n_q).T
        psi = oracle.potential_3d(E, cb, sp, op.shear[idx], op.bulk[idx], op.lame[idx])
    else:
        E = oracle.strain_2d(pat.dphi1, pat.dphi2, u_ov, pat.overlap_element_dof_lids, pat.n_q).T
        psi = oracle.potential_2d(E, cb, sp, op.shear[idx], op.bulk[idx], op.lame[idx])
    w = pat.overlap_assembly_weight
    J_o = float(np.dot(w, psi))
    assert abs(J - J_o) <= PLAIN_RTOL * float(np.dot(w, np.abs(psi)))
    assert op.get_total_time()["potential"] > 0.0
    split = int(np.median(mesh.elem.min(axis=0)))
    parts = []
    for rng in ((0, split), (split, mesh.n_nodes)):
        o = _operator(mesh, mats, et, rng)
        o.reduction(lam)
        parts.append(o.potential_energy(U))
    assert abs(sum(parts) - J) <= PLAIN_RTOL * float(np.dot(w, np.abs(psi)))
    print(f"{dim}D {et}: J = {J:.6e}, split ranks {parts[0]:.4e} + {parts[1]:.4e}")
