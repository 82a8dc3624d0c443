"""Parity of the CUDA hot path with the reference (golden fixtures) and with the oracle.

Every comparison is a max-norm relative error at the plain-path tolerance (1e-12) unless stated;
CSR indices and maps are compared bit for bit.  All calls go through the C ABI (directly or via
the package's drop-in functions, which are thin ctypes wrappers)."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import PLAIN_RTOL, golden, golden_files, rel_err

pytestmark = pytest.mark.gpu

MATERIAL = {"c0": 15.0, "phi": 30.0, "psi": 0.0, "young": 10000.0, "poisson": 0.33, "gamma_sat": 19.0,
            "gamma_unsat": 19.0}


@pytest.fixture(autouse=True)
def _clean_status(cuda_device):
    from slope_stability_petsc4py_gb300 import _lib

    _lib.device_status(clear=True)
    yield
    assert _lib.device_status(clear=True) == 0


def _dev(a, dtype=None):
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    return _lib.to_device(np.ascontiguousarray(a), dtype or torch.float64)


def _constitutive(E, args, tangent=True, kernel="ssp_constitutive_3d_sds"):
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    n = E.shape[0]
    Ed = _dev(E)
    A = [_dev(a) for a in args]
    S = torch.empty((n, 6), dtype=torch.float64, device="cuda")
    if tangent:
        DS = torch.empty((n, 36), dtype=torch.float64, device="cuda")
        _lib.call(kernel, _lib.ptr(Ed), *[_lib.ptr(a) for a in A], n, _lib.ptr(S), _lib.ptr(DS), _lib.stream_handle())
        return S.cpu().numpy(), DS.cpu().numpy()
    _lib.call("ssp_constitutive_3d_s", _lib.ptr(Ed), *[_lib.ptr(a) for a in A], n, _lib.ptr(S), _lib.stream_handle())
    return S.cpu().numpy()


def test_constitutive_3d_matches_reference_c_kernel():
    g = golden("constitutive_3d.npz")
    for tag in ("bench_l1.0", "bench_l1.3", "test_l1.0", "test_l1.3"):
        args = [g[f"{tag}_{k}"] for k in ("c_bar", "sin_phi", "shear", "bulk", "lame")]
        S, DS = _constitutive(g["E"], args)
        assert rel_err(S, g[f"{tag}_S_c"]) <= PLAIN_RTOL
        assert rel_err(DS, g[f"{tag}_DS_c"]) <= PLAIN_RTOL
        # the stress-only kernel yields the same stresses bit for bit
        assert np.array_equal(_constitutive(g["E"], args, tangent=False), S)
        # the tangent is exactly symmetric
        D = DS.reshape(-1, 6, 6)
        assert np.array_equal(D, np.transpose(D, (0, 2, 1)))


def test_constitutive_3d_matches_oracle_on_many_points(oracle):
    rng = np.random.default_rng(2024)
    n = 200_000
    E = rng.standard_normal((n, 6)) * np.repeat(np.array([1e-4, 1e-3, 3e-3, 1e-2]), n // 4)[:, None]
    young, nu = 2.0e4, 0.49
    shear = np.full(n, young / (2 * (1 + nu)))
    bulk = np.full(n, young / (3 * (1 - 2 * nu)))
    lame = bulk - 2 * shear / 3
    c_bar, sin_phi = oracle.reduction(np.full(n, 6.0), np.full(n, np.deg2rad(45.0)), np.zeros(n), 1.1, "B")
    args = [c_bar, sin_phi, shear, bulk, lame]
    S, DS = _constitutive(E, args)
    S_o, DS_o = oracle.constitutive_3d(E, *args)
    assert rel_err(S, S_o) <= PLAIN_RTOL
    assert rel_err(DS, DS_o) <= PLAIN_RTOL


def test_binned_return_mapping_matches_single_pass_and_oracle(oracle):
    """Two-pass, branch-binned kernel == single-pass kernel == oracle, on points of every branch."""
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    rng = np.random.default_rng(77)
    n = 150_000
    E = rng.standard_normal((n, 6)) * np.repeat(np.array([1e-4, 1e-3, 3e-3]), n // 3)[:, None]
    g = golden("constitutive_3d.npz")
    E = np.vstack([E, g["E"]])
    n = E.shape[0]
    young, nu = 2.0e4, 0.49
    shear = np.full(n, young / (2 * (1 + nu)))
    lame = np.full(n, young / (3 * (1 - 2 * nu))) - 2 * shear / 3
    c_bar, sin_phi = oracle.reduction(np.full(n, 6.0), np.full(n, np.deg2rad(45.0)), np.zeros(n), 1.1, "B")
    Ed, cb, sp, G, L = (_dev(a) for a in (E, c_bar, sin_phi, shear, lame))
    outs = {}
    for mode in ("single", "binned"):
        S = torch.empty((n, 6), dtype=torch.float64, device="cuda")
        DS = torch.empty((n, 36), dtype=torch.float64, device="cuda")
        br = torch.empty(n, dtype=torch.int8, device="cuda")
        if mode == "single":
            _lib.call("ssp_constitutive_sds_branch", 3, _lib.ptr(Ed), _lib.ptr(cb), _lib.ptr(sp), _lib.ptr(G), _lib.ptr(L),
                      n, _lib.ptr(S), _lib.ptr(DS), _lib.ptr(br), _lib.stream_handle())
        else:
            scratch = torch.full((3 * n + 4,), -7, dtype=torch.int32, device="cuda")
            _lib.call("ssp_constitutive_3d_sds_binned", _lib.ptr(Ed), _lib.ptr(cb), _lib.ptr(sp), _lib.ptr(G),
                      _lib.ptr(L), n, _lib.ptr(S), _lib.ptr(DS), _lib.ptr(br), _lib.ptr(scratch), _lib.stream_handle())
            listed, n_smooth, n_left, n_right = (int(v) for v in scratch[:4].cpu().numpy())
            b = br.cpu().numpy()
            lst = scratch[4:4 + listed].cpu().numpy()
            assert int((b != 0).sum()) <= listed <= n  # every plastic point went through the full path
            assert np.unique(lst).size == listed and set(np.flatnonzero(b != 0)) <= set(lst.tolist())
            assert [n_smooth, n_left, n_right] == [int((b == k).sum()) for k in (1, 2, 3)]
        outs[mode] = (S.cpu().numpy(), DS.cpu().numpy(), br.cpu().numpy())
    assert np.array_equal(outs["single"][2], outs["binned"][2])
    seen = set(np.unique(outs["binned"][2]).tolist())
    assert {0, 1, 4} <= seen and seen & {2, 3}
    # the same FP64 formulas compiled in two kernels (FMA contraction may differ): a few ulps
    assert rel_err(outs["binned"][0], outs["single"][0]) <= 1e-14
    assert rel_err(outs["binned"][1], outs["single"][1]) <= 1e-14
    S_o, DS_o = oracle.constitutive_3d(E, c_bar, sin_phi, shear, shear, lame)
    assert rel_err(outs["binned"][0], S_o) <= PLAIN_RTOL
    assert rel_err(outs["binned"][1], DS_o) <= PLAIN_RTOL


def test_branch_labels_match_tangent_structure():
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    g = golden("constitutive_3d.npz")
    tag = "bench_l1.0"
    args = [g[f"{tag}_{k}"] for k in ("c_bar", "sin_phi", "shear", "lame")]
    n = g["E"].shape[0]
    Ed = _dev(g["E"])
    A = [_dev(a) for a in args]
    S = torch.empty((n, 6), dtype=torch.float64, device="cuda")
    br = torch.empty(n, dtype=torch.int8, device="cuda")
    _lib.call("ssp_constitutive_3d_branch", _lib.ptr(Ed), *[_lib.ptr(a) for a in A], n, _lib.ptr(S), _lib.ptr(br),
              _lib.stream_handle())
    b = br.cpu().numpy()
    DS = g[f"{tag}_DS_c"].reshape(-1, 6, 6)
    assert set(np.unique(b)) <= {0, 1, 2, 3, 4}
    assert np.all(np.abs(DS[b == 4]).max(initial=0.0) == 0.0)  # apex: zero tangent
    assert np.allclose(DS[b == 0][:, 0, 1], g[f"{tag}_lame"][b == 0])  # elastic: lame off-diagonal
    assert rel_err(S.cpu().numpy(), g[f"{tag}_S_c"]) <= PLAIN_RTOL


def test_constitutive_2d_matches_reference_numpy():
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    g = golden("constitutive_2d.npz")
    for tag in ("l1.0", "l1.2"):
        n = g["E"].shape[1]
        Ed = _dev(g["E"].T)
        A = [_dev(g[f"{tag}_{k}"]) for k in ("c_bar", "sin_phi", "shear", "bulk", "lame")]
        S = torch.empty((n, 4), dtype=torch.float64, device="cuda")
        DS = torch.empty((n, 9), dtype=torch.float64, device="cuda")
        _lib.call("ssp_constitutive_2d", _lib.ptr(Ed), *[_lib.ptr(a) for a in A], n, _lib.ptr(S), _lib.ptr(DS),
                  _lib.stream_handle())
        assert rel_err(S.cpu().numpy().T, g[f"{tag}_S"]) <= PLAIN_RTOL
        assert rel_err(DS.cpu().numpy().T, g[f"{tag}_DS"]) <= PLAIN_RTOL


def test_binned_2d_return_mapping_matches_single_pass_and_reference():
    """ssp_constitutive_2d_sds_binned (elastic points first, plastic branches on the listed points):
    the reference's fixture at 1e-12, and against the single-pass kernel the same branch codes and
    S, DS within a few ulps (the same source in two kernels may contract multiply-adds differently),
    on the fixture's points and on 200k random points over four strain magnitudes."""
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    def run(entry, E, args):
        n = E.shape[0]
        Ed = _dev(E)
        A = [_dev(a) for a in args]
        S = torch.empty((n, 4), dtype=torch.float64, device="cuda")
        DS = torch.empty((n, 9), dtype=torch.float64, device="cuda")
        br = torch.empty(n, dtype=torch.int8, device="cuda")
        if entry == "ssp_constitutive_2d_sds_binned":
            scratch = torch.empty(n + 1, dtype=torch.int32, device="cuda")
            _lib.call(entry, _lib.ptr(Ed), *[_lib.ptr(a) for a in A], n, _lib.ptr(S), _lib.ptr(DS), _lib.ptr(br),
                      _lib.ptr(scratch), _lib.stream_handle())
        else:
            _lib.call(entry, 2, _lib.ptr(Ed), *[_lib.ptr(a) for a in A], n, _lib.ptr(S), _lib.ptr(DS), _lib.ptr(br),
                      _lib.stream_handle())
        return S, DS, br

    g = golden("constitutive_2d.npz")
    for tag in ("l1.0", "l1.2"):
        args = [g[f"{tag}_{k}"] for k in ("c_bar", "sin_phi", "shear", "lame")]
        S, DS, br = run("ssp_constitutive_2d_sds_binned", np.ascontiguousarray(g["E"].T), args)
        assert rel_err(S.cpu().numpy().T, g[f"{tag}_S"]) <= PLAIN_RTOL
        assert rel_err(DS.cpu().numpy().T, g[f"{tag}_DS"]) <= PLAIN_RTOL
        S1, DS1, br1 = run("ssp_constitutive_sds_branch", np.ascontiguousarray(g["E"].T), args)
        assert torch.equal(br, br1)
        assert rel_err(S.cpu().numpy(), S1.cpu().numpy()) <= 1e-14 and rel_err(DS.cpu().numpy(), DS1.cpu().numpy()) <= 1e-14
    rng = np.random.default_rng(21)
    n = 200_000
    E = rng.standard_normal((n, 3)) * np.repeat(np.array([1e-4, 1e-3, 3e-3, 1e-2]), n // 4)[:, None]
    young, nu = rng.uniform(1e4, 5e4, n), rng.uniform(0.2, 0.45, n)
    shear = young / (2 * (1 + nu))
    lame = young / (3 * (1 - 2 * nu)) - 2 * shear / 3
    phi = np.deg2rad(rng.uniform(20.0, 45.0, n))
    args = [2 * rng.uniform(5.0, 30.0, n) * np.cos(phi), np.sin(phi), shear, lame]
    a = run("ssp_constitutive_2d_sds_binned", E, args)
    b = run("ssp_constitutive_sds_branch", E, args)
    counts = torch.bincount(a[2].long(), minlength=5).cpu().numpy()
    assert (counts > 100).all(), counts  # every branch occurs
    assert torch.equal(a[2], b[2])
    for x, y in zip(a[:2], b[:2]):
        assert rel_err(x.cpu().numpy(), y.cpu().numpy()) <= 1e-14  # max-norm over all points, as in 3D
        rows = (x - y).abs().amax(dim=1) / y.abs().amax(dim=1).clamp_min(1e-300)
        assert float(rows.max()) <= PLAIN_RTOL  # and every point within the parity tolerance


def test_reduction_matches_reference():
    from slope_stability_petsc4py_gb300 import reduction

    g = golden("reduction.npz")
    for dav in ("A", "B", "C"):
        for lam in (0.8, 1.0, 1.35):
            cb, sp = reduction(g["c0"], g["phi"], g["psi"], lam, dav)
            assert rel_err(cb, g[f"{dav}_{lam}_c_bar"]) <= 1e-14
            assert rel_err(sp, g[f"{dav}_{lam}_sin_phi"]) <= 1e-14
    with pytest.raises(ValueError):
        reduction(g["c0"], g["phi"], g["psi"], -1.0, "A")


def _pattern(g, **kw):
    from slope_stability_petsc4py_gb300 import prepare_owned_tangent_pattern

    return prepare_owned_tangent_pattern(g["coord"], g["elem"], g["q_mask"], np.zeros(g["elem"].shape[1], np.int64),
                                         [MATERIAL] if g["coord"].shape[0] == 3 else [dict(MATERIAL, c0=6.0, phi=45.0,
                                                                                           young=2.0e4, poisson=0.49,
                                                                                           gamma_sat=20.0,
                                                                                           gamma_unsat=20.0)],
                                         tuple(int(v) for v in g["owned_node_range"]), elem_type=str(g["elem_type"]), **kw)


@pytest.mark.parametrize("name", golden_files("pattern_"))
def test_pattern_geometry_and_elastic_values(name):
    g = golden(name)
    pat = _pattern(g)
    assert np.array_equal(pat.local_matrix_pattern.indptr, g["indptr"])
    assert np.array_equal(pat.local_matrix_pattern.indices, g["indices"])
    assert np.array_equal(pat.scatter_map, g["scatter_map"])
    assert np.array_equal(pat.slot_pos, g["slot_pos"])
    assert np.array_equal(pat.constrained_diag_positions, g["constrained_diag_positions"])
    assert rel_err(pat.dphi1, g["dphi1"]) <= PLAIN_RTOL
    assert rel_err(pat.dphi2, g["dphi2"]) <= PLAIN_RTOL
    assert rel_err(pat.dphi3, g["dphi3"]) <= PLAIN_RTOL
    assert rel_err(pat.overlap_assembly_weight, g["weight"]) <= PLAIN_RTOL
    assert rel_err(pat.elastic_values, g["elastic_values"]) <= PLAIN_RTOL
    assert np.all(pat.elastic_values[pat.constrained_diag_positions] == 1.0)


@pytest.mark.parametrize("name", golden_files("overlap_operator_"))
def test_overlap_operator_and_reference_elastic_rows(name):
    """include_overlap_B=True gives the reference's sparse strain operator; a reference
    OwnedElasticRows passed as elastic_rows gives its projected elastic values; overlap_B applied to
    the overlap displacements equals the strain kernel."""
    from types import SimpleNamespace

    from scipy.sparse import csr_matrix

    from slope_stability_petsc4py_gb300 import assemble_overlap_strain, prepare_owned_tangent_pattern

    g = golden(name)
    dim = g["q_mask"].shape[0]
    mat = {"c0": 6.0, "phi": 45.0, "psi": 0.0, "young": 2.0e4, "poisson": 0.49, "gamma_sat": 20.0, "gamma_unsat": 20.0}
    owned = tuple(int(v) for v in g["owned_node_range"])
    L = csr_matrix((g["L_data"], g["L_indices"], g["L_indptr"]), shape=tuple(g["L_shape"]))
    rows = SimpleNamespace(owned_node_range=owned, owned_row_range=(dim * owned[0], dim * owned[1]), local_matrix=L)
    pat = prepare_owned_tangent_pattern(g["coord"], g["elem"], g["q_mask"], np.zeros(g["elem"].shape[1], np.int64),
                                        [mat], owned, elem_type="P2", include_overlap_B=True, elastic_rows=rows)
    assert np.array_equal(pat.elastic_values, g["elastic_values"])
    assert pat.timings["elastic_pattern_reused"] == 1.0
    B = pat.overlap_B
    ref = csr_matrix((g["B_data"], g["B_indices"], g["B_indptr"]), shape=tuple(g["B_shape"]))
    # the same matrix to the gradients' rounding: the reference keeps roundoff-sized gradients
    # (down to 1e-33 here) as stored entries and drops exact zeros, so which of those entries are
    # stored follows the last bits of the gradients (bit for bit from the reference's own
    # gradients: tests/test_lib_cpu.py)
    assert B.shape == ref.shape
    assert abs(B - ref).max() <= PLAIN_RTOL * abs(ref).max()
    U = np.random.default_rng(3).standard_normal(g["q_mask"].shape)
    E = assemble_overlap_strain(pat, U)
    u_ov = U.reshape(-1, order="F")[pat.overlap_global_dofs]
    assert rel_err(np.asarray(B @ u_ov).reshape(pat.n_strain, -1, order="F"), E) <= PLAIN_RTOL
    with pytest.raises(ValueError):
        prepare_owned_tangent_pattern(g["coord"], g["elem"], g["q_mask"], np.zeros(g["elem"].shape[1], np.int64),
                                      [mat], (0, owned[1]), elem_type="P2", elastic_rows=rows)


@pytest.mark.parametrize("name", golden_files("pattern_"))
def test_assembly_matches_reference(name):
    from slope_stability_petsc4py_gb300 import (assemble_overlap_strain, assemble_owned_force_from_local_stress,
                                                assemble_owned_tangent_values)

    g = golden(name)
    pat = _pattern(g)
    for kernel in ("rows", "legacy", "rows_gather"):
        vals = assemble_owned_tangent_values(pat, g["ds"], kernel=kernel)
        assert rel_err(vals, g["rows_c"]) <= PLAIN_RTOL, kernel
        assert np.all(vals[pat.constrained_diag_positions] == 1.0)
    assert rel_err(assemble_overlap_strain(pat, g["U"]), g["strain_c"]) <= PLAIN_RTOL
    assert rel_err(assemble_owned_force_from_local_stress(pat, g["stress"]), g["force_c"]) <= PLAIN_RTOL


@pytest.mark.parametrize("name", golden_files("pattern_"))
def test_symmetric_tangent_kernel(name, oracle):
    import torch

    from slope_stability_petsc4py_gb300.distributed_tangent import tangent_values_device

    g = golden(name)
    pat = _pattern(g)
    ds = g["ds"].T.reshape(-1, 6, 6)
    ds = 0.5 * (ds + np.transpose(ds, (0, 2, 1)))
    ds_aos = np.ascontiguousarray(ds.reshape(-1, 36))
    want = oracle.tangent_scatter(3, g["dphi1"], g["dphi2"], g["dphi3"], ds_aos, g["weight"], g["scatter_map"],
                                  int(g["n_q"]), pat.nnz)
    want[pat.constrained_diag_positions] = 1.0
    got_sym = tangent_values_device(pat, _dev(ds_aos), symmetric=True).cpu().numpy()
    got_gen = tangent_values_device(pat, _dev(ds_aos), symmetric=False).cpu().numpy()
    assert rel_err(got_sym, want) <= PLAIN_RTOL
    assert rel_err(got_gen, want) <= PLAIN_RTOL
    torch.cuda.synchronize()


@pytest.mark.parametrize("name", golden_files("pattern_"))
def test_constitutive_operator_matches_reference(name):
    from slope_stability_petsc4py_gb300 import ConstitutiveOperator

    g = golden(name)
    pat = _pattern(g)
    n_int = g["mat_c0"].size
    op = ConstitutiveOperator(B=None, c0=g["mat_c0"], phi=g["mat_phi"], psi=g["mat_psi"], Davis_type="B",
                              shear=g["mat_shear"], bulk=g["mat_bulk"], lame=g["mat_lame"], WEIGHT=np.ones(n_int),
                              n_strain=6, n_int=n_int, dim=3, q_mask=g["q_mask"])
    op.set_owned_tangent_pattern(pat, tangent_kernel="rows", constitutive_mode="overlap")
    op.reduction(float(g["op_lambda"]))
    S = op.constitutive_problem_stress_tangent(g["op_U"])
    assert S.shape == g["op_S"].shape
    assert rel_err(np.asarray(S), g["op_S"]) <= PLAIN_RTOL
    assert rel_err(np.asarray(op._owned_local_DS), g["op_DS"]) <= PLAIN_RTOL
    assert rel_err(op.build_F_local(), g["op_F"]) <= PLAIN_RTOL
    assert rel_err(op.build_F_free_local(), g["op_F_free"]) <= PLAIN_RTOL
    K = op._build_owned_tangent_matrix()
    _, _, kv = K.getValuesCSR()
    assert rel_err(kv, g["op_K"]) <= PLAIN_RTOL
    Kr = op.build_K_regularized(float(g["op_r"]))
    _, cols, kr = Kr.getValuesCSR()
    assert np.array_equal(cols, g["indices"])
    assert rel_err(kr, g["op_Kr"]) <= PLAIN_RTOL
    h1 = Kr.handle
    assert op.build_K_regularized(float(g["op_r"])).handle == h1  # in-place update, stable handle
    S_only = op.constitutive_problem_stress(g["op_U"])
    assert rel_err(np.asarray(S_only), g["op_S_only"]) <= PLAIN_RTOL
    assert set(op.get_total_time()) >= {"reduction", "stress", "stress_tangent", "build_F", "build_tangent_local"}


def test_operator_accepts_caller_tangent_like_reference():
    """A caller may assign _owned_local_DS directly (tests/test_distributed_tangent_rows.py:308-321)."""
    from slope_stability_petsc4py_gb300 import ConstitutiveOperator, assemble_owned_tangent_matrix

    g = golden("pattern_tet2_P2.npz")
    pat = _pattern(g)
    n_int = pat.n_local_int
    op = ConstitutiveOperator(B=None, c0=np.zeros(n_int), phi=np.zeros(n_int), psi=np.zeros(n_int), Davis_type="B",
                              shear=np.ones(n_int), bulk=np.ones(n_int), lame=np.ones(n_int), WEIGHT=np.ones(n_int),
                              n_strain=6, n_int=n_int, dim=3, q_mask=g["q_mask"])
    op.set_owned_tangent_pattern(pat, tangent_kernel="rows", constitutive_mode="overlap")
    rng = np.random.default_rng(404)
    ds1, ds2 = rng.standard_normal((36, n_int)), rng.standard_normal((36, n_int))
    op._owned_local_DS = ds1
    m1 = op._build_owned_tangent_matrix()
    op._owned_local_DS = ds2
    m2 = op._build_owned_tangent_matrix()
    assert m1.handle == m2.handle
    rows, cols, vals = m2.getValuesCSR()
    ref = assemble_owned_tangent_matrix(pat, ds2)
    assert np.array_equal(rows, ref.indptr) and np.array_equal(cols, ref.indices)
    assert rel_err(vals, ref.data) <= 1e-11


@pytest.mark.parametrize("name", golden_files("pattern2d_"))
def test_2d_assembly_matches_reference(name, oracle):
    from slope_stability_petsc4py_gb300 import (assemble_overlap_strain, assemble_owned_force_from_local_stress,
                                                assemble_owned_tangent_values)

    g = golden(name)
    pat = _pattern(g)
    assert np.array_equal(pat.scatter_map, g["scatter_map"])
    assert rel_err(pat.dphi1, g["dphi1"]) <= PLAIN_RTOL
    assert rel_err(pat.elastic_values, g["elastic_values"]) <= PLAIN_RTOL
    assert rel_err(assemble_owned_tangent_values(pat, g["ds"], kernel="legacy"), g["legacy_py"]) <= PLAIN_RTOL
    assert rel_err(assemble_overlap_strain(pat, g["U"]), g["strain_py"]) <= PLAIN_RTOL
    assert rel_err(assemble_owned_force_from_local_stress(pat, g["stress"]), g["force_py"]) <= PLAIN_RTOL


@pytest.mark.parametrize("et,dims", [("P1", (24, 12)), ("P2", (14, 8)), ("P4", (7, 4))])
def test_2d_operator_against_oracle_on_slope(oracle, et, dims):
    """Plane strain on a layered synthetic slope: strain -> S/DS -> F -> regularised K through the
    operator, against the oracle chain (P4: the reference's 15-node triangles and basis table);
    then the mixed form's tangent against the FP64 one."""
    from slope_stability_petsc4py_gb300 import ConstitutiveOperator, synthetic
    from slope_stability_petsc4py_gb300.distributed_tangent import _PatternBuild

    mats = synthetic.MaterialSet.layered(4, seed=2)
    mesh = synthetic.slope_mesh_2d(*dims, elem_type=et, n_layers=4)
    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=float(mats.psi[i]), young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=20.0, gamma_unsat=20.0) for i in range(mats.c0.size)]
    op = ConstitutiveOperator.from_mesh(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs, elem_type=et)
    U = synthetic.displacement_field(mesh, mats, amplitude=0.05, seed=3)
    pat = op.owned_tangent_pattern
    lam, r = 1.1, 0.25
    op.reduction(lam)
    op.constitutive_problem_stress_tangent(U)
    idx = pat.local_int_indices
    cb, sp = oracle.reduction(op.c0[idx], op.phi[idx], op.psi[idx], lam, "B")
    u_ov = U.reshape(-1, order="F")[pat.overlap_global_dofs]
    E = oracle.strain_2d(pat.dphi1, pat.dphi2, u_ov, pat.overlap_element_dof_lids, pat.n_q)
    S, DS = oracle.constitutive_2d(E.T, cb, sp, op.shear[idx], op.bulk[idx], op.lame[idx])
    plastic = np.mean(np.abs(DS[1] - op.lame[idx]) > 1e-9 * op.lame[idx])
    assert 0.02 < plastic < 0.8
    assert rel_err(np.asarray(op._owned_local_S), S) <= PLAIN_RTOL
    assert rel_err(np.asarray(op._owned_local_DS), DS) <= PLAIN_RTOL
    F = op.build_F_local()
    f_ov = oracle.overlap_force_2d(pat.dphi1, pat.dphi2, np.ascontiguousarray(S[:3].T), pat.overlap_assembly_weight,
                                   pat.overlap_element_dof_lids, pat.n_q, pat.overlap_global_dofs.size)
    F_o = f_ov[pat.owned_local_overlap_dofs]
    F_o[~pat.owned_free_mask] = 0.0
    assert rel_err(F, F_o) <= PLAIN_RTOL
    _, _, kv = op.build_K_regularized(r).getValuesCSR()
    kv = kv.copy()
    pb = _PatternBuild(mesh.elem, mesh.q_mask, (0, mesh.n_nodes))
    scatter = pb.get("scatter_map")
    pb.close()
    K_o = oracle.tangent_scatter(2, pat.dphi1, pat.dphi2, None, np.ascontiguousarray(DS.T), pat.overlap_assembly_weight,
                                 scatter, pat.n_q, pat.nnz)
    K_o[pat.constrained_diag_positions] = 1.0
    K_o = (1.0 - r) * K_o + r * pat.elastic_values
    assert rel_err(kv, K_o) <= PLAIN_RTOL
    op.tangent_form = "mixed"
    op.constitutive_problem_stress_tangent(U)
    _, _, km = op.build_K_regularized(r).getValuesCSR()
    err = rel_err(km, kv)
    print(f"2D {et}: plastic fraction {plastic:.3f}, mixed tangent error {err:.3e}")
    assert err <= 1.0e-6


def _slope_operator(et, nx, ny, nz, materials=None, lam=1.1):
    from slope_stability_petsc4py_gb300 import ConstitutiveOperator, synthetic

    mesh = synthetic.slope_mesh_3d(nx, ny, nz, elem_type=et, n_layers=4 if materials is not None else 1)
    mats = materials or synthetic.MaterialSet.homogeneous()
    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=float(mats.psi[i]), young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=20.0, gamma_unsat=20.0) for i in range(mats.c0.size)]
    op = ConstitutiveOperator.from_mesh(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs, elem_type=et)
    U = synthetic.displacement_field(mesh, mats, amplitude=0.05, seed=3)
    return mesh, op, U


@pytest.mark.parametrize("et,dims", [("P2", (12, 5, 6)), ("P4", (4, 2, 2))])
def test_operator_against_oracle_on_slope(oracle, et, dims):
    """Strain -> S/DS -> F -> K on a heterogeneous synthetic slope, against the oracle chain."""
    from slope_stability_petsc4py_gb300 import synthetic

    mesh, op, U = _slope_operator(et, *dims, materials=synthetic.MaterialSet.layered(4, seed=1))
    pat = op.owned_tangent_pattern
    op.reduction(1.1)
    op.constitutive_problem_stress_tangent(U)
    idx = pat.local_int_indices
    cb, sp = oracle.reduction(op.c0[idx], op.phi[idx], op.psi[idx], 1.1, "B")
    u_ov = U.reshape(-1, order="F")[pat.overlap_global_dofs]
    n_q = pat.n_q
    E = oracle.strain_3d(pat.dphi1, pat.dphi2, pat.dphi3, u_ov, pat.overlap_element_dof_lids, n_q)
    S, DS = oracle.constitutive_3d(E, cb, sp, op.shear[idx], op.bulk[idx], op.lame[idx])
    plastic = np.mean(np.abs(DS[:, 1] - op.lame[idx]) > 1e-9 * op.lame[idx])
    assert 0.05 < plastic < 0.6
    assert rel_err(np.asarray(op._owned_local_S), S.T) <= PLAIN_RTOL
    assert rel_err(np.asarray(op._owned_local_DS), DS.T) <= PLAIN_RTOL
    F = op.build_F_local()
    from slope_stability_petsc4py_gb300.distributed_tangent import _PatternBuild

    pb = _PatternBuild(mesh.elem, mesh.q_mask, (0, mesh.n_nodes))
    slots = {k: pb.get(k) for k in ("row_slot_ptr", "slot_elem", "slot_lrow", "slot_pos", "scatter_map")}
    pb.close()
    F_o = oracle.force_rows_3d(pat.dphi1, pat.dphi2, pat.dphi3, S, pat.overlap_assembly_weight, slots["row_slot_ptr"],
                               slots["slot_elem"], slots["slot_lrow"], n_q)
    F_o[~pat.owned_free_mask] = 0.0
    assert rel_err(F, F_o) <= PLAIN_RTOL
    r = 0.25
    _, _, kv = op.build_K_regularized(r).getValuesCSR()
    K_o = oracle.tangent_rows_3d(pat.dphi1, pat.dphi2, pat.dphi3, DS, pat.overlap_assembly_weight, slots["row_slot_ptr"],
                                 slots["slot_elem"], slots["slot_lrow"], slots["slot_pos"], n_q, pat.nnz)
    K_o[pat.constrained_diag_positions] = 1.0
    K_o = (1.0 - r) * K_o + r * pat.elastic_values
    assert rel_err(kv, K_o) <= PLAIN_RTOL


def test_p2_affine_strain_and_force_match_gradient_kernels():
    """The plain form's regrouped P2 strain and force (J^{-1} per element, barycentric basis) that
    the operator runs on straight-sided tetrahedra, against the per-point-gradient kernels of the
    reference's arithmetic on the same inputs; a partial owned node range (rows of only some of
    the overlap elements' dofs)."""
    import torch

    from slope_stability_petsc4py_gb300 import _lib, synthetic
    from slope_stability_petsc4py_gb300.distributed_tangent import (
        _p2_affine_inputs,
        _u_overlap_device,
        overlap_strain_device,
        owned_force_device,
        prepare_owned_tangent_pattern,
    )

    mesh = synthetic.slope_mesh_3d(16, 6, 8, elem_type="P2", n_layers=4)
    mats = synthetic.MaterialSet.layered(4, seed=5)
    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=0.0, young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=20.0, gamma_unsat=20.0) for i in range(mats.c0.size)]
    U = synthetic.displacement_field(mesh, mats, amplitude=0.03, seed=6)
    for rng in ((0, mesh.n_nodes), (mesh.n_nodes // 3, 2 * mesh.n_nodes // 3)):
        pat = prepare_owned_tangent_pattern(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs, rng,
                                            elem_type="P2", include_legacy_scatter=False, keep_slot_metadata=False)
        d = _p2_affine_inputs(pat)
        assert d is not None and pat.affine_p2
        E = overlap_strain_device(pat, U)
        u_ov = _u_overlap_device(pat, U)
        n_el, n = int(pat.overlap_elements.size), pat.n_local_int
        E_g = torch.empty_like(E)
        st = _lib.stream_handle()
        _lib.call("ssp_assemble_overlap_strain_3d", _lib.ptr(d["dphi1"]), _lib.ptr(d["dphi2"]), _lib.ptr(d["dphi3"]),
                  _lib.ptr(u_ov), int(u_ov.numel()), _lib.ptr(d["dof_lids"]), n, n_el, pat.n_p, pat.n_q,
                  _lib.ptr(E_g), st)
        err_e = rel_err(E.cpu().numpy(), E_g.cpu().numpy())
        S = torch.randn((n, 6), dtype=torch.float64, device="cuda")
        F = owned_force_device(pat, S)
        F_g = torch.empty_like(F)
        _lib.call("ssp_assemble_force_element", 3, _lib.ptr(d["dphi1"]), _lib.ptr(d["dphi2"]), _lib.ptr(d["dphi3"]),
                  _lib.ptr(S), _lib.ptr(d["weight"]), _lib.ptr(d["elem_row"]), n_el, pat.n_p, pat.n_q, int(F.numel()),
                  _lib.ptr(F_g), st)
        err_f = rel_err(F.cpu().numpy(), F_g.cpu().numpy())
        print(f"P2 affine, owned range {rng}: strain {err_e:.2e}, force {err_f:.2e}")
        assert err_e <= 1e-13 and err_f <= 1e-13


@pytest.mark.parametrize("et,dims", [("P4", (6, 3, 3)), ("P1", (24, 10, 12))])
def test_affine_fp64_strain_and_force_match_gradient_kernels(oracle, et, dims):
    """The plain form's J^{-1} strain and force for straight-sided P1 / P4 tetrahedra (reference
    gradient table in shared memory instead of per-point gradients) against the per-point-gradient
    kernels and the oracle, on a full and a partial owned node range."""
    import torch

    from slope_stability_petsc4py_gb300 import _lib, synthetic
    from slope_stability_petsc4py_gb300.distributed_tangent import (
        _affine_fp64_inputs,
        _u_overlap_device,
        overlap_strain_device,
        owned_force_device,
        prepare_owned_tangent_pattern,
    )

    mesh = synthetic.slope_mesh_3d(*dims, elem_type=et, n_layers=4)
    mats = synthetic.MaterialSet.layered(4, seed=5)
    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=0.0, young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=20.0, gamma_unsat=20.0) for i in range(mats.c0.size)]
    U = synthetic.displacement_field(mesh, mats, amplitude=0.03, seed=6)
    for rng in ((0, mesh.n_nodes), (mesh.n_nodes // 3, 2 * mesh.n_nodes // 3)):
        pat = prepare_owned_tangent_pattern(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs, rng,
                                            elem_type=et, include_legacy_scatter=False, keep_slot_metadata=True,
                                            include_overlap_B=False)
        d = _affine_fp64_inputs(pat)
        assert d is not None and pat.affine_fp64
        E = overlap_strain_device(pat, U)
        u_ov = _u_overlap_device(pat, U)
        n_el, n = int(pat.overlap_elements.size), pat.n_local_int
        E_g = torch.empty_like(E)
        st = _lib.stream_handle()
        _lib.call("ssp_assemble_overlap_strain_3d", _lib.ptr(d["dphi1"]), _lib.ptr(d["dphi2"]), _lib.ptr(d["dphi3"]),
                  _lib.ptr(u_ov), int(u_ov.numel()), _lib.ptr(d["dof_lids"]), n, n_el, pat.n_p, pat.n_q,
                  _lib.ptr(E_g), st)
        err_e = rel_err(E.cpu().numpy(), E_g.cpu().numpy())
        S = torch.randn((n, 6), dtype=torch.float64, device="cuda")
        F = owned_force_device(pat, S)
        F_g = torch.empty_like(F)
        _lib.call("ssp_assemble_force_element", 3, _lib.ptr(d["dphi1"]), _lib.ptr(d["dphi2"]), _lib.ptr(d["dphi3"]),
                  _lib.ptr(S), _lib.ptr(d["weight"]), _lib.ptr(d["elem_row"]), n_el, pat.n_p, pat.n_q, int(F.numel()),
                  _lib.ptr(F_g), st)
        err_f = rel_err(F.cpu().numpy(), F_g.cpu().numpy())
        # and the oracle's restatement of the reference's row kernels on the same gradients
        E_o = oracle.strain_3d(pat.dphi1, pat.dphi2, pat.dphi3, u_ov.cpu().numpy(), pat.overlap_element_dof_lids,
                               pat.n_q)
        F_o = oracle.force_rows_3d(pat.dphi1, pat.dphi2, pat.dphi3, S.cpu().numpy(), pat.overlap_assembly_weight,
                                   pat.row_slot_ptr, pat.slot_elem, pat.slot_lrow, pat.n_q)
        F_o[~pat.owned_free_mask] = 0.0
        err_eo, err_fo = rel_err(E.cpu().numpy(), E_o), rel_err(F.cpu().numpy(), F_o)
        print(f"{et} affine, owned range {rng}: strain {err_e:.2e} / oracle {err_eo:.2e}, "
              f"force {err_f:.2e} / oracle {err_fo:.2e}")
        assert max(err_e, err_f) <= 1e-13 and max(err_eo, err_fo) <= PLAIN_RTOL


def test_p2_moment_correction_matches_point_by_point(oracle):
    """The plain tangent of straight-sided P2 elements with the plastic correction in moment form
    (every plastic element, and the default split by plastic-point count) against the
    point-by-point correction and against the oracle's rows tangent, on a strongly yielding slope."""
    from slope_stability_petsc4py_gb300 import ConstitutiveOperator, synthetic

    mats = synthetic.MaterialSet.layered(4, seed=2)
    mesh = synthetic.slope_mesh_3d(12, 5, 6, elem_type="P2", n_layers=4)
    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=0.0, young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=20.0, gamma_unsat=20.0) for i in range(mats.c0.size)]
    op = ConstitutiveOperator.from_mesh(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs, elem_type="P2")
    U = synthetic.displacement_field(mesh, mats, amplitude=0.08, seed=9)
    op.reduction(1.3)
    split = op.moment_min_points
    assert split > 1
    out = {}
    for mp in (0, 1, split):
        op.moment_min_points = mp
        op.constitutive_problem_stress_tangent(U)
        kt = op._build_owned_tangent_matrix().getValuesCSR()[2].copy()
        kr = op.build_K_regularized(0.2).getValuesCSR()[2].copy()
        out[mp] = (kt, kr)
    pat = op.owned_tangent_pattern
    assert pat.affine_p2
    per_elem = (np.asarray(op._branch.cpu()).reshape(-1, pat.n_q) != 0).sum(axis=1)
    assert (per_elem >= split).sum() > 50 and ((per_elem > 0) & (per_elem < split)).sum() > 0
    for mp in (1, split):
        assert rel_err(out[mp][0], out[0][0]) <= 1e-13
        assert rel_err(out[mp][1], out[0][1]) <= 1e-13
    DS = np.ascontiguousarray(np.asarray(op._owned_local_DS).T)
    K_o = oracle.tangent_scatter(3, pat.dphi1, pat.dphi2, pat.dphi3, DS, pat.overlap_assembly_weight,
                                 _p2_scatter_map(pat), pat.n_q, pat.nnz)
    K_o[pat.constrained_diag_positions] = 1.0
    assert rel_err(out[1][0], K_o) <= PLAIN_RTOL


def _p2_scatter_map(pat):
    return pat.device["scatter_map"].cpu().numpy()


def test_large_mesh_properties():
    """At a benchmark-like size: symmetric == general kernel, K symmetric, linear in DS."""
    import torch

    from slope_stability_petsc4py_gb300.distributed_tangent import tangent_values_device

    mesh, op, U = _slope_operator("P2", 30, 10, 20)  # ~36k tets, ~400k points
    pat = op.owned_tangent_pattern
    op.reduction(1.0)
    op.constitutive_problem_stress_tangent(U)
    ds = op._owned_local_DS.aos
    k_sym = tangent_values_device(pat, ds, symmetric=True)
    k_gen = tangent_values_device(pat, ds, symmetric=False)
    assert rel_err(k_sym.cpu().numpy(), k_gen.cpu().numpy()) <= 1e-13
    # elastic predictor + plastic correction (the operator's path) == direct sum over all points
    k_direct = tangent_values_device(pat, ds, symmetric=True).cpu().numpy()
    Kf = op._build_owned_tangent_matrix().to_scipy()
    assert op._branch is not None and int((op._branch != 0).sum()) > 0
    assert rel_err(Kf.data, k_direct) <= 1e-13
    r = 0.3
    _, _, kr = op.build_K_regularized(r).getValuesCSR()
    assert rel_err(kr, (1.0 - r) * k_direct + r * pat.elastic_values) <= 1e-13
    # K restricted to free rows/cols is symmetric (every row is owned here)
    free = np.flatnonzero(pat.owned_free_mask)
    Kff = Kf[free][:, free]
    assert abs(Kff - Kff.T).max() <= 1e-12 * abs(Kff).max()
    # linearity in DS
    ds2 = ds * 0.5 + 1.0
    lhs = tangent_values_device(pat, (ds + 2.0 * ds2).contiguous(), finish=False)
    rhs = tangent_values_device(pat, ds, finish=False) + 2.0 * tangent_values_device(pat, ds2.contiguous(), finish=False)
    assert rel_err(lhs.cpu().numpy(), rhs.cpu().numpy()) <= 1e-12
    torch.cuda.synchronize()


def test_screened_return_mapping_options_and_elastic_fill(oracle):
    """ssp_constitutive_3d_sds_screened: with SSP_RM_PLASTIC_DS_ONLY the rows of the points that
    return elastic are left untouched and every other output equals the full run bit for bit;
    ssp_fill_elastic_ds then completes DS bit for bit; the three binning sources agree."""
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    rng = np.random.default_rng(17)
    n = 60_000
    E = rng.standard_normal((n, 6)) * np.repeat([1e-4, 1e-3, 3e-3], n // 3)[:, None]
    young, nu, phi = 2.0e4, 0.35, np.deg2rad(35.0)
    shear = np.full(n, young / (2 * (1 + nu)))
    lame = np.full(n, young / (3 * (1 - 2 * nu))) - 2 * shear / 3
    args = [_dev(a) for a in (E, np.full(n, 12.0 * np.cos(phi)), np.full(n, np.sin(phi)), shear, lame)]
    scratch = torch.empty(8 * n + 12, dtype=torch.int32, device="cuda")

    def run(bins, source, options):
        S = torch.full((n, 6), float("nan"), dtype=torch.float64, device="cuda")
        DS = torch.full((n, 36), float("nan"), dtype=torch.float64, device="cuda")
        br = torch.full((n,), -1, dtype=torch.int8, device="cuda")
        _lib.call("ssp_constitutive_3d_sds_screened", *[_lib.ptr(a) for a in args], n, _lib.ptr(S), _lib.ptr(DS),
                  _lib.ptr(br), _lib.ptr(scratch), bins, source, options, _lib.stream_handle())
        return S, DS, br

    S0, DS0, b0 = run(_lib.BINS_EXACT, None, 0)
    assert not torch.isnan(DS0).any() and (b0 >= 0).all()
    el = b0 == 0
    assert 0 < int(el.sum()) < n
    S1, DS1, b1 = run(_lib.BINS_EXACT, None, _lib.RM_PLASTIC_DS_ONLY)
    assert torch.equal(S1, S0) and torch.equal(b1, b0)
    assert torch.equal(DS1[~el], DS0[~el])
    assert torch.isnan(DS1[el]).any()  # the rows of the points the screen finished were not written
    _lib.call("ssp_fill_elastic_ds", 3, _lib.ptr(b1), _lib.ptr(args[3]), _lib.ptr(args[4]), n, _lib.ptr(DS1),
              _lib.stream_handle())
    assert torch.equal(DS1, DS0)
    prev = b0.clone()
    for bins, source in ((_lib.BINS_GIVEN, _lib.ptr(prev)),):
        S2, DS2, b2 = run(bins, source, 0)
        assert torch.equal(S2, S0) and torch.equal(DS2, DS0) and torch.equal(b2, b0)
    Sm, DSm, bm = run(_lib.BINS_EXACT, None, _lib.RM_COMPENSATED_DS | _lib.RM_PLASTIC_DS_ONLY)
    assert torch.equal(bm, b0) and torch.equal(Sm, S0)
    pl = (b0 >= 1) & (b0 <= 3)  # smooth face and edges (an apex point's DS is zero)
    err = ((DSm[pl] - DS0[pl]).abs().max(dim=1).values / DS0[pl].abs().max(dim=1).values).max()
    assert float(err) <= 1e-10  # the compensated plastic DS, as ssp_constitutive_3d_sds_binned_mixed
    with pytest.raises(_lib.SSPError):
        run(7, None, 0)
    S_o, DS_o = oracle.constitutive_3d(E, *[a.cpu().numpy() for a in args[1:3]], shear, np.zeros(n), lame)
    assert rel_err(S0.cpu().numpy(), S_o) <= PLAIN_RTOL and rel_err(DS0.cpu().numpy(), DS_o) <= PLAIN_RTOL


def test_operator_lazy_elastic_rows_match_full_rows():
    """The operator's default (elastic DS rows written only when read) gives the same DS, tangent
    and regularised values as writing every row in the return mapping."""
    mesh, op, U = _slope_operator("P2", 8, 4, 4)
    op.reduction(1.1)
    outs = {}
    for lazy in (False, True):
        op.lazy_elastic_ds = lazy
        op.constitutive_problem_stress_tangent(U)
        kt = op._build_owned_tangent_matrix().getValuesCSR()[2].copy()
        kr = op.build_K_regularized(0.25).getValuesCSR()[2].copy()
        outs[lazy] = (np.asarray(op._owned_local_DS), kt, kr)
    assert np.array_equal(outs[False][0], outs[True][0])  # DS bit for bit
    # the CSR values are sums of FP64 reductions in no fixed order: equal to rounding
    assert rel_err(outs[True][1], outs[False][1]) <= 1e-14
    assert rel_err(outs[True][2], outs[False][2]) <= 1e-14


def test_device_resident_operator_path():
    """CUDA-tensor inputs keep every result on the device."""
    import torch

    mesh, op, U = _slope_operator("P2", 6, 3, 3)
    op.host_outputs = False
    Ud = torch.as_tensor(U, device="cuda")
    op.reduction(1.2)
    F_free, K = op.build_F_K_regularized_reduced_free(Ud, 0.1)
    assert isinstance(F_free, torch.Tensor) and F_free.is_cuda
    assert K.values.is_cuda
    op.host_outputs = True
    F_free_h = op.build_F_free_local()
    # the element force kernel sums with atomics, so repeated calls agree to rounding only
    assert rel_err(F_free.cpu().numpy(), F_free_h) <= 1e-14


def _yield_parts(E, shear, lame, sin_phi):
    """g with f = g - c_bar (exact eigenvalues), the invariant bound h >= g and the size of f's terms."""
    t = E.copy()
    t[:, 3:] *= 0.5
    M = np.zeros((E.shape[0], 3, 3))
    for (i, j), k in {(0, 0): 0, (1, 1): 1, (2, 2): 2, (0, 1): 3, (1, 2): 4, (0, 2): 5}.items():
        M[:, i, j] = M[:, j, i] = t[:, k]
    ev = np.linalg.eigvalsh(M)
    I1 = t[:, :3].sum(axis=1)
    s = sin_phi
    g = 2 * shear * ((1 + s) * ev[:, 2] - (1 - s) * ev[:, 0]) + 2 * lame * s * I1
    dev = 2 * np.sqrt(((ev[:, :, None] - ev[:, None, :]) ** 2).sum(axis=(1, 2)) / 36.0) * np.sqrt(3 + s * s)  # 2 sqrt(J2/3)
    h = 2 * shear * (dev + 2 * s * I1 / 3) + 2 * lame * s * I1
    size = 2 * shear * (dev + np.abs(I1)) + 2 * np.abs(lame * s * I1)
    return g, h, size


def test_elastic_screen_near_yield_and_screen_threshold(oracle):
    """Points straddling the yield surface and the invariant screen's threshold: every point the
    kernels call elastic is elastic for the reference formula, and results match the oracle away
    from the yield surface itself (|f| > 1e-7 of its terms, where any two FP64 evaluations agree)."""
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    rng = np.random.default_rng(5)
    young, nu, c0, phi = 2.0e4, 0.3, 10.0, np.deg2rad(32.0)
    shear, lame = young / (2 * (1 + nu)), young * nu / ((1 + nu) * (1 - 2 * nu))
    sin_phi = np.sin(phi)
    c_bar = 2 * c0 * np.cos(phi)
    dirs = [rng.standard_normal((3000, 6))]
    # deviators at the Lode angle that maximises the trial yield function (where the bound is tight)
    a = np.arctan2(np.sqrt(3.0), sin_phi)
    th = a - np.pi / 3
    d = np.array([np.cos(th), np.cos(th - 2 * np.pi / 3), np.cos(th + 2 * np.pi / 3)])
    for k in range(600):
        Rq, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        T = Rq @ np.diag(d + rng.uniform(-0.5, 0.5)) @ Rq.T
        dirs.append(np.array([[T[0, 0], T[1, 1], T[2, 2], 2 * T[0, 1], 2 * T[1, 2], 2 * T[0, 2]]]))
    rep = rng.standard_normal((300, 2))  # repeated eigenvalues
    dirs.append(np.column_stack([rep[:, 0], rep[:, 0], rep[:, 1], np.zeros((300, 3))]))
    D = np.vstack(dirs)
    repeated_dir = np.zeros(D.shape[0], dtype=bool)
    repeated_dir[-300:] = True
    g1, h1, size1 = _yield_parts(D, shear, lame, sin_phi)
    pts, rep_tag = [], []
    mult = np.array([1 - 1e-2, 1 - 1e-5, 1 - 1e-8, 1 + 1e-8, 1 + 1e-5, 1 + 1e-2])
    ok = g1 > 0
    for m in mult:  # around the yield surface
        pts.append(D[ok] * (c_bar / g1[ok] * m)[:, None])
        rep_tag.append(repeated_dir[ok])
    # the screen's threshold: bound = -1e-4 size with the kernel's size = 2G (dev + 3 max|t|) +
    # 2|lambda s I1| + c_bar (dev and I1 scale with the strain, c_bar does not)
    tD = D.copy()
    tD[:, 3:] *= 0.5
    dev1 = (h1 - 2 * lame * sin_phi * tD[:, :3].sum(1)) / (2 * shear) - 2 * sin_phi * tD[:, :3].sum(1) / 3
    size_k = 2 * shear * (dev1 + 3 * np.abs(tD).max(1)) + 2 * np.abs(lame * sin_phi * tD[:, :3].sum(1))
    ok = h1 + 1e-4 * size_k > 0
    alpha_s = c_bar * (1 - 1e-4) / (h1[ok] + 1e-4 * size_k[ok])
    # the screen's FP32 noise is ~4e-6 of size; beyond 1e-4 the yield surface is reached
    for m in (1 - 3e-5, 1 - 1e-6, 1 - 1e-7, 1.0, 1 + 1e-7, 1 + 1e-6, 1 + 3e-5):
        pts.append(D[ok] * (alpha_s * m)[:, None])
        rep_tag.append(repeated_dir[ok])
    E = np.vstack(pts)
    repeated = np.concatenate(rep_tag)
    n = E.shape[0]
    full = lambda v: np.full(n, v)  # noqa: E731
    args = (full(c_bar), full(sin_phi), full(shear), full(lame))
    Ed, cb, sp, G, L = (_dev(x) for x in (E,) + args)
    outs = {}
    for mode in ("single", "binned"):
        S = torch.empty((n, 6), dtype=torch.float64, device="cuda")
        DS = torch.empty((n, 36), dtype=torch.float64, device="cuda")
        br = torch.empty(n, dtype=torch.int8, device="cuda")
        if mode == "single":
            _lib.call("ssp_constitutive_sds_branch", 3, _lib.ptr(Ed), _lib.ptr(cb), _lib.ptr(sp), _lib.ptr(G),
                      _lib.ptr(L), n, _lib.ptr(S), _lib.ptr(DS), _lib.ptr(br), _lib.stream_handle())
        else:
            scratch = torch.empty(3 * n + 4, dtype=torch.int32, device="cuda")
            _lib.call("ssp_constitutive_3d_sds_binned", _lib.ptr(Ed), _lib.ptr(cb), _lib.ptr(sp), _lib.ptr(G),
                      _lib.ptr(L), n, _lib.ptr(S), _lib.ptr(DS), _lib.ptr(br), _lib.ptr(scratch), _lib.stream_handle())
        outs[mode] = (S.cpu().numpy(), DS.cpu().numpy(), br.cpu().numpy())
    br = outs["binned"][2]
    assert np.array_equal(outs["single"][2], br)
    el = br == 0  # elastic points: the same arithmetic in both kernels, screened or not
    assert np.array_equal(outs["single"][0][el], outs["binned"][0][el])
    assert np.array_equal(outs["single"][1][el], outs["binned"][1][el])
    g, h, size = _yield_parts(E, shear, lame, sin_phi)
    f = g - c_bar
    # the reference's trigonometric eigenvalues carry up to ~1e-8 sqrt(Q) of rounding near repeated
    # roots, so decisions are compared where |f| exceeds 1e-7 of its terms (the screen's margin is 1e-4)
    tol = 1e-7 * (size + c_bar)
    assert np.all(f[el] <= tol[el])  # never elastic where the reference yields
    assert np.all(br[f < -tol] == 0) and np.all(br[f > tol] != 0)
    S_o, DS_o = oracle.constitutive_3d(E, *args[:3], args[2], args[3])
    clear = np.abs(f) > tol
    # away from the surface, and (for plastic points) with distinct eigenvalues: the plastic
    # tangent of exactly repeated principal strains is rounding-sensitive in any FP64 evaluation
    well = clear & (el | ~repeated)
    for mode in ("single", "binned"):
        assert rel_err(outs[mode][0][well], S_o[well]) <= PLAIN_RTOL
        assert rel_err(outs[mode][1][well], DS_o[well]) <= PLAIN_RTOL
    thr = np.zeros(n, dtype=bool)
    thr[-7 * int(ok.sum()):] = True  # the points around the screen's threshold
    assert np.all(br[thr] == 0)
    print(f"{n} points, {int(well.sum())} compared with the oracle, elastic {float(np.mean(el)):.3f}")
