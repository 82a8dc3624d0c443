"""Generate the golden fixtures in this folder from the reference implementation itself.

Run where a reference checkout is available (it is read, never modified), naming it by the
environment variable ``SSP_REFERENCE_ROOT``:

    SSP_REFERENCE_ROOT=<reference checkout> python tests/golden/make_golden.py [generator ...]

What it does:

1. compiles the reference's own C kernels (``src/slope_stability/cython/*.c``) from their
   sources through ``oracle/Makefile`` (target ``ref``) and calls them through ctypes;
2. imports the reference Python package with stand-ins for the modules this container lacks
   (petsc4py, mpi4py, h5py, meshio, matplotlib); the paths used here never touch them;
3. evaluates the reference on small seeded inputs and stores inputs and outputs as ``.npz``.

The fixtures pin the oracle (``oracle/``) and the CUDA path to the reference's results.
"""

from __future__ import annotations

import ctypes
import importlib
import os
import sys
import types
from pathlib import Path
from unittest import mock

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
REF_ROOT = Path(os.environ.get("SSP_REFERENCE_ROOT", ""))
sys.path.insert(0, str(REPO))

from oracle import oracle_py  # noqa: E402

MATERIAL = {"c0": 15.0, "phi": 30.0, "psi": 0.0, "young": 10000.0, "poisson": 0.33,
            "gamma_sat": 19.0, "gamma_unsat": 19.0}


def import_reference():
    os.environ["PYTHONDONTWRITEBYTECODE"] = "1"
    sys.dont_write_bytecode = True
    for name in ("petsc4py", "petsc4py.PETSc", "mpi4py", "mpi4py.MPI", "h5py", "meshio",
                 "matplotlib", "matplotlib.pyplot", "pyvista"):
        sys.modules.setdefault(name, mock.MagicMock())
    sys.path.insert(0, str(REF_ROOT / "src"))
    mods = {
        "dt": importlib.import_module("slope_stability.fem.distributed_tangent"),
        "problem": importlib.import_module("slope_stability.constitutive.problem"),
        "reduction": importlib.import_module("slope_stability.constitutive.reduction"),
        "simplex": importlib.import_module("slope_stability.core.simplex_lagrange"),
        "assembly": importlib.import_module("slope_stability.fem.assembly"),
    }
    return mods


def compiled_kernels_module(libref):
    """A stand-in for the reference's Cython module that calls its compiled C kernels."""
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int32)

    def d(a):
        return a.ctypes.data_as(dp)

    def sds(E, c, s, g, k, l):
        n = E.shape[0]
        S = np.empty((n, 6))
        DS = np.empty((n, 36))
        libref.constitutive_problem_3d_sds_batch_c(d(E), d(c), d(s), d(g), d(k), d(l), n, d(S), d(DS))
        return S, DS

    def s_only(E, c, s, g, k, l):
        n = E.shape[0]
        S = np.empty((n, 6))
        libref.constitutive_problem_3d_s_batch_c(d(E), d(c), d(s), d(g), d(k), d(l), n, d(S))
        return S

    def strain(d1, d2, d3, u, dof, n_q):
        n_el = dof.shape[0]
        out = np.empty((n_el * n_q, 6))
        libref.assemble_overlap_strain_3d_c(d(d1), d(d2), d(d3), d(u), dof.ctypes.data_as(ip), d1.shape[0], n_el,
                                            d1.shape[1], n_q, d(out))
        return out

    def force(d1, d2, d3, S, w, rp, se, sl, n_q):
        n_rows = rp.size - 1
        out = np.zeros(n_rows)
        libref.assemble_force_3d_rows_c(d(d1), d(d2), d(d3), d(S), d(w), rp.ctypes.data_as(ip), se.ctypes.data_as(ip),
                                        sl.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), d1.shape[0], n_rows,
                                        se.size, d1.shape[1], n_q, d(out))
        return out

    def rows(d1, d2, d3, ds, w, rp, se, sl, sp, n_q, nnz):
        out = np.zeros(nnz)
        libref.assemble_tangent_values_3d_rows_c(d(d1), d(d2), d(d3), d(ds), d(w), rp.ctypes.data_as(ip),
                                                 se.ctypes.data_as(ip), sl.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                                 sp.ctypes.data_as(ip), d1.shape[0], rp.size - 1, se.size, d1.shape[1],
                                                 n_q, nnz, d(out))
        return out

    def legacy(d1, d2, d3, ds, w, sm, nnz):
        out = np.zeros(nnz)
        n_el = sm.shape[0]
        libref.assemble_tangent_values_3d_p2_c(d(d1), d(d2), d(d3), d(ds), d(w), sm.ctypes.data_as(ip), d1.shape[0],
                                               n_el, d1.shape[1], d1.shape[0] // max(n_el, 1), nnz, d(out))
        return out

    m = types.ModuleType("reference_compiled_kernels")
    m.constitutive_problem_3d_sds = sds
    m.constitutive_problem_3d_s = s_only
    m.assemble_overlap_strain_3d = strain
    m.assemble_force_3d_rows = force
    m.assemble_tangent_values_3d_rows = rows
    m.assemble_tangent_values_3d = legacy
    return m


def elevated_tetra_mesh(simplex, order, tet4, vertices):
    tuples = simplex.tetra_lagrange_node_tuples(int(order))
    cmap, pts = {}, []
    elem = np.empty((len(tuples), tet4.shape[1]), dtype=np.int64)
    for e in range(tet4.shape[1]):
        verts = vertices[:, tet4[:, e]]
        for li, counts in enumerate(tuples):
            p = verts @ (np.asarray(counts, dtype=np.float64) / order)
            key = tuple(np.round(p, 12).tolist())
            if key not in cmap:
                cmap[key] = len(pts)
                pts.append(p)
            elem[li, e] = cmap[key]
    return np.column_stack(pts), elem


def pattern_arrays(pat):
    out = {
        "indptr": np.asarray(pat.local_matrix_pattern.indptr, dtype=np.int32),
        "indices": np.asarray(pat.local_matrix_pattern.indices, dtype=np.int32),
        "scatter_map": pat.scatter_map,
        "row_slot_ptr": pat.row_slot_ptr,
        "slot_elem": pat.slot_elem,
        "slot_lrow": pat.slot_lrow,
        "slot_pos": pat.slot_pos,
        "constrained_diag_positions": pat.constrained_diag_positions,
        "elastic_values": pat.elastic_values,
        "dphi1": pat.dphi1,
        "dphi2": pat.dphi2,
        "weight": pat.overlap_assembly_weight,
        "overlap_elements": pat.overlap_elements,
        "overlap_nodes": pat.overlap_nodes,
        "overlap_global_dofs": pat.overlap_global_dofs,
        "overlap_element_dof_lids": pat.overlap_element_dof_lids,
        "owned_local_overlap_dofs": pat.owned_local_overlap_dofs,
        "owned_free_mask": pat.owned_free_mask,
        "local_int_indices": pat.local_int_indices,
        "n_q": np.int64(pat.n_q),
        "n_p": np.int64(pat.n_p),
    }
    if pat.dim == 3:
        out["dphi3"] = pat.dphi3
    return out


def material_fields(n_int):
    young, nu = MATERIAL["young"], MATERIAL["poisson"]
    shear = young / (2.0 * (1.0 + nu))
    bulk = young / (3.0 * (1.0 - 2.0 * nu))
    lame = bulk - 2.0 * shear / 3.0
    return {
        "c0": np.full(n_int, MATERIAL["c0"]),
        "phi": np.full(n_int, np.deg2rad(MATERIAL["phi"])),
        "psi": np.full(n_int, np.deg2rad(MATERIAL["psi"])),
        "shear": np.full(n_int, shear),
        "bulk": np.full(n_int, bulk),
        "lame": np.full(n_int, lame),
    }


def mesh_cases(simplex):
    verts = np.array([[0.0, 1.0, 0.0, 0.0, 1.0], [0.0, 0.0, 1.0, 0.0, 1.0], [0.0, 0.0, 0.0, 1.0, 1.0]])
    one = np.array([[0], [1], [2], [3]], dtype=np.int64)
    two = np.array([[0, 1], [1, 2], [2, 3], [3, 4]], dtype=np.int64)
    cases = {}
    for et, order in (("P1", 1), ("P2", 2), ("P4", 4)):
        cases[f"tet1_{et}"] = (et, *elevated_tetra_mesh(simplex, order, one, verts), False, None, None)
    for et, order in (("P2", 2), ("P4", 4)):
        cases[f"tet2_{et}"] = (et, *elevated_tetra_mesh(simplex, order, two, verts), False, None, None)
    cases["tet1_P4_constrained"] = ("P4", *elevated_tetra_mesh(simplex, 4, one, verts), True, None, None)
    # four-element chain of curved-ish vertices (tests/test_owned_constitutive_exchange.py:44-65)
    t = np.arange(1, 8, dtype=np.float64)
    chain_v = np.vstack((t, 0.1 * t * t, 0.01 * t * t * t))
    chain = np.vstack([np.arange(i, i + 4, dtype=np.int64) for i in range(4)])
    cases["chain_P2"] = ("P2", *elevated_tetra_mesh(simplex, 2, chain, chain_v), False, None, None)
    # a small slope block with a Dirichlet base and a partial owned node range
    from slope_stability_petsc4py_gb300 import synthetic

    m = synthetic.slope_mesh_3d(3, 2, 2, depth=6.0, elem_type="P2")
    n_nodes = m.coord.shape[1]
    cases["slope_P2_partial"] = ("P2", m.coord, m.elem, "mask", (n_nodes // 3, 2 * n_nodes // 3), m.q_mask)
    m4 = synthetic.slope_mesh_3d(2, 1, 1, depth=6.0, elem_type="P4")
    cases["slope_P4_partial"] = ("P4", m4.coord, m4.elem, "mask", (0, 12), m4.q_mask)
    return cases


def gen_patterns(ref, kern):
    dt, problem = ref["dt"], ref["problem"]
    for name, (et, coord, elem, constrain, owned, qm) in mesh_cases(ref["simplex"]).items():
        if isinstance(constrain, str):
            q_mask = np.asarray(qm, dtype=bool)
        else:
            q_mask = np.ones((3, coord.shape[1]), dtype=bool)
            if constrain:
                q_mask[:, 0] = False
        owned = owned or (0, coord.shape[1])
        mat_id = np.zeros(elem.shape[1], dtype=np.int64)
        full = tuple(owned) == (0, coord.shape[1])
        pat = dt.prepare_owned_tangent_pattern(coord, elem, q_mask, mat_id, [MATERIAL], owned, elem_type=et,
                                               include_unique=full)
        rng = np.random.default_rng(101)
        n_loc = pat.local_int_indices.size
        ds = rng.standard_normal((36, n_loc))
        U = rng.standard_normal((3, coord.shape[1]))
        stress = rng.standard_normal((6, n_loc))
        rows_py = dt.assemble_owned_tangent_values(pat, ds, use_compiled=False, kernel="rows")
        legacy_py = dt.assemble_owned_tangent_values(pat, ds, use_compiled=False, kernel="legacy")
        dt._kernels = kern
        rows_c = dt.assemble_owned_tangent_values(pat, ds, use_compiled=True, kernel="rows")
        legacy_c = dt.assemble_owned_tangent_values(pat, ds, use_compiled=True, kernel="legacy")
        strain_c = dt.assemble_overlap_strain(pat, U, use_compiled=True)
        force_c = dt.assemble_owned_force_from_local_stress(pat, stress, use_compiled=True)
        dt._kernels = None
        strain_py = dt.assemble_overlap_strain(pat, U, use_compiled=False)
        force_py = dt.assemble_owned_force_from_local_stress(pat, stress, use_compiled=False)
        # full constitutive operator, production settings (overlap mode, compiled kernels)
        n_int_global = elem.shape[1] * pat.n_q
        mf = material_fields(n_int_global)
        builder = problem.ConstitutiveOperator(B=None, c0=mf["c0"], phi=mf["phi"], psi=mf["psi"], Davis_type="B",
                                               shear=mf["shear"], bulk=mf["bulk"], lame=mf["lame"],
                                               WEIGHT=np.ones(n_int_global), n_strain=6, n_int=n_int_global, dim=3,
                                               q_mask=q_mask)
        builder.set_owned_tangent_pattern(pat, use_compiled=True, tangent_kernel="rows", constitutive_mode="overlap",
                                          use_compiled_constitutive=True)
        dt._kernels = kern
        problem._kernels = kern
        lam = 1.1
        scale = 2.0e-3
        U_op = scale * U
        builder.reduction(lam)
        S_op = np.asarray(builder.constitutive_problem_stress_tangent(U_op)).copy()
        DS_op = np.asarray(builder._owned_local_DS).copy()
        F_op = np.asarray(builder.build_F_local()).copy()
        F_free_op = np.asarray(builder.build_F_free_local()).copy()
        K_op = dt.assemble_owned_tangent_values(pat, DS_op, use_compiled=True, kernel="rows")
        r = 0.3
        Kr_op = (1.0 - r) * K_op + r * pat.elastic_values
        S_only = np.asarray(builder.constitutive_problem_stress(U_op)).copy()
        dt._kernels = None
        problem._kernels = None
        np.savez_compressed(
            HERE / f"pattern_{name}.npz",
            elem_type=np.array(et), coord=coord, elem=elem, q_mask=q_mask, owned_node_range=np.asarray(owned),
            ds=ds, U=U, stress=stress,
            rows_py=rows_py, legacy_py=legacy_py, rows_c=rows_c, legacy_c=legacy_c,
            strain_c=strain_c, strain_py=strain_py, force_c=force_c, force_py=force_py,
            op_lambda=lam, op_U=U_op, op_r=r, op_S=S_op, op_DS=DS_op, op_F=F_op, op_F_free=F_free_op,
            op_K=K_op, op_Kr=Kr_op, op_S_only=S_only,
            **{f"mat_{k}": v for k, v in mf.items()},
            **pattern_arrays(pat),
        )
        print("pattern", name, pat.local_matrix_pattern.nnz, "nnz")


def constitutive_points(rng, n_random=800):
    """Strain points spanning the branches plus hand-made edge cases, E (n, 6) engineering."""
    pts = []
    for scale in (1e-5, 1e-4, 1e-3, 3e-3, 1e-2):
        pts.append(rng.standard_normal((n_random // 5, 6)) * scale)
    edge = [
        np.zeros(6),                                   # zero strain: Q = 0
        np.array([1e-3, 1e-3, 1e-3, 0, 0, 0]),         # hydrostatic compression-free expansion: Q = 0
        np.array([-2e-3, -2e-3, -2e-3, 0, 0, 0]),      # hydrostatic compression
        np.array([5e-3, 5e-3, 5e-3, 0, 0, 0]),         # large hydrostatic tension -> apex
        np.array([2e-3, 0, 0, 0, 0, 0]),               # uniaxial: repeated eigenvalues (0, 0)
        np.array([0, 0, -3e-3, 0, 0, 0]),              # uniaxial compression
        np.array([1e-3, 1e-3, -2e-3, 0, 0, 0]),        # e1 == e2 (triaxial extension)
        np.array([2e-3, -1e-3, -1e-3, 0, 0, 0]),       # e2 == e3 (triaxial compression)
        np.array([0, 0, 0, 4e-3, 0, 0]),               # pure shear
        np.array([1e-3, -1e-3, 0, 2e-3, 1e-3, -1e-3]),
        np.array([3e-3, 1e-3, -2e-3, 1e-3, -2e-3, 5e-4]),
    ]
    return np.vstack(pts + [np.vstack(edge)])


def gen_constitutive(kern, problem, libref):
    rng = np.random.default_rng(7)
    E = constitutive_points(rng)
    n = E.shape[0]
    out = {"E": E}
    # two material sets: the benchmark's (c=6, phi=45, nu=0.49) and the tests' (c=15, phi=30, nu=0.33)
    sets = {"bench": (6.0, 45.0, 2.0e4, 0.49), "test": (15.0, 30.0, 1.0e4, 0.33)}
    red = importlib.import_module("slope_stability.constitutive.reduction")
    for key, (c0, phi, young, nu) in sets.items():
        for lam in (1.0, 1.3):
            shear = young / (2.0 * (1.0 + nu))
            bulk = young / (3.0 * (1.0 - 2.0 * nu))
            lame = bulk - 2.0 * shear / 3.0
            c_bar, sin_phi = red.reduction(np.full(n, c0), np.full(n, np.deg2rad(phi)), np.zeros(n), lam, "B")
            g, k, l = np.full(n, shear), np.full(n, bulk), np.full(n, lame)
            S_c, DS_c = kern.constitutive_problem_3d_sds(np.ascontiguousarray(E), c_bar, sin_phi, g, k, l)
            S_only = kern.constitutive_problem_3d_s(np.ascontiguousarray(E), c_bar, sin_phi, g, k, l)
            S_np, DS_np = problem.constitutive_problem_3D(E.T, c_bar, sin_phi, g, k, l, return_tangent=True)
            tag = f"{key}_l{lam}"
            out.update({f"{tag}_c_bar": c_bar, f"{tag}_sin_phi": sin_phi, f"{tag}_shear": g, f"{tag}_bulk": k,
                        f"{tag}_lame": l, f"{tag}_S_c": S_c, f"{tag}_DS_c": DS_c, f"{tag}_S_only_c": S_only,
                        f"{tag}_S_np": S_np.T.copy(), f"{tag}_DS_np": DS_np.T.copy()})
    np.savez_compressed(HERE / "constitutive_3d.npz", **out)
    print("constitutive_3d", n, "points")


def gen_constitutive_2d(problem, red):
    rng = np.random.default_rng(11)
    pts = [rng.standard_normal((300, 3)) * s for s in (1e-4, 1e-3, 3e-3, 1e-2)]
    edge = np.array([[0, 0, 0], [1e-3, 1e-3, 0], [-1e-3, -1e-3, 0], [5e-3, 5e-3, 0], [2e-3, 0, 0],
                     [0, -3e-3, 0], [0, 0, 4e-3], [1e-3, -1e-3, 2e-3], [-1e-3, -2e-3, 0], [1e-3, 2e-3, 1e-4]])
    E = np.vstack(pts + [edge]).T.copy()  # (3, n)
    n = E.shape[1]
    out = {"E": E}
    for lam in (1.0, 1.2):
        young, nu = 2.0e4, 0.49
        shear = young / (2.0 * (1.0 + nu))
        bulk = young / (3.0 * (1.0 - 2.0 * nu))
        lame = bulk - 2.0 * shear / 3.0
        c_bar, sin_phi = red.reduction(np.full(n, 6.0), np.full(n, np.deg2rad(45.0)), np.zeros(n), lam, "B")
        S, DS = problem.constitutive_problem_2D(E, c_bar, sin_phi, np.full(n, shear), np.full(n, bulk),
                                                np.full(n, lame), return_tangent=True)
        tag = f"l{lam}"
        out.update({f"{tag}_c_bar": c_bar, f"{tag}_sin_phi": sin_phi, f"{tag}_shear": np.full(n, shear),
                    f"{tag}_bulk": np.full(n, bulk), f"{tag}_lame": np.full(n, lame), f"{tag}_S": S, f"{tag}_DS": DS})
    np.savez_compressed(HERE / "constitutive_2d.npz", **out)
    print("constitutive_2d", n, "points")


def gen_potential(problem, red):
    """The reference's potential_3D / potential_2D (the energy the direct SSR continuation
    differences in lambda) on the constitutive test points, two material sets."""
    rng = np.random.default_rng(19)
    E3 = constitutive_points(rng).T.copy()  # (6, n)
    E2 = np.hstack([rng.standard_normal((3, 250)) * s for s in (1e-4, 1e-3, 3e-3, 1e-2)]
                   + [np.array([[0, 0, 0], [1e-3, 1e-3, 0], [-1e-3, -1e-3, 0], [2e-3, -1e-3, 0], [0, 0, 4e-3],
                                [5e-3, 5e-3, 0], [-1e-3, -2e-3, 0]], dtype=np.float64).T])
    out = {"E3": E3, "E2": E2}
    for key, (c0, phi, young, nu, lam) in {"bench": (6.0, 45.0, 2.0e4, 0.49, 1.1),
                                           "test": (15.0, 30.0, 1.0e4, 0.33, 1.3)}.items():
        shear = young / (2.0 * (1.0 + nu))
        bulk = young / (3.0 * (1.0 - 2.0 * nu))
        lame = bulk - 2.0 * shear / 3.0
        for dim, E in ((3, E3), (2, E2)):
            n = E.shape[1]
            c_bar, sin_phi = red.reduction(np.full(n, c0), np.full(n, np.deg2rad(phi)), np.zeros(n), lam, "B")
            mats = (c_bar, sin_phi, np.full(n, shear), np.full(n, bulk), np.full(n, lame))
            psi = (problem.potential_3D if dim == 3 else problem.potential_2D)(E, *mats)
            tag = f"{key}_{dim}d"
            out.update({f"{tag}_c_bar": c_bar, f"{tag}_sin_phi": sin_phi, f"{tag}_shear": mats[2],
                        f"{tag}_bulk": mats[3], f"{tag}_lame": mats[4], f"{tag}_psi": psi})
    np.savez_compressed(HERE / "potential.npz", **out)
    print("potential", E3.shape[1], "3D points,", E2.shape[1], "2D points")


def gen_reduction(red):
    rng = np.random.default_rng(3)
    n = 64
    c0 = rng.uniform(1.0, 20.0, n)
    phi = np.deg2rad(rng.uniform(15.0, 45.0, n))
    psi = np.deg2rad(rng.uniform(0.0, 15.0, n))
    out = {"c0": c0, "phi": phi, "psi": psi}
    for dav in ("A", "B", "C"):
        for lam in (0.8, 1.0, 1.35):
            cb, sp = red.reduction(c0, phi, psi, lam, dav)
            out[f"{dav}_{lam}_c_bar"] = cb
            out[f"{dav}_{lam}_sin_phi"] = sp
    np.savez_compressed(HERE / "reduction.npz", **out)
    print("reduction")


def gen_pattern_2d(ref):
    dt = ref["dt"]
    from slope_stability_petsc4py_gb300 import synthetic

    m = synthetic.slope_mesh_2d(4, 3, elem_type="P2")
    n_nodes = m.coord.shape[1]
    mat = {"c0": 6.0, "phi": 45.0, "psi": 0.0, "young": 2.0e4, "poisson": 0.49, "gamma_sat": 20.0,
           "gamma_unsat": 20.0}
    for tag, owned in (("full", (0, n_nodes)), ("partial", (n_nodes // 4, 3 * n_nodes // 4))):
        pat = dt.prepare_owned_tangent_pattern(m.coord, m.elem, m.q_mask, np.zeros(m.elem.shape[1], np.int64), [mat],
                                               owned, elem_type="P2", include_unique=(tag == "full"))
        rng = np.random.default_rng(5)
        n_loc = pat.local_int_indices.size
        ds = rng.standard_normal((9, n_loc))
        U = rng.standard_normal((2, n_nodes))
        stress = rng.standard_normal((3, n_loc))
        legacy_py = dt.assemble_owned_tangent_values(pat, ds, use_compiled=False, kernel="legacy")
        strain_py = dt.assemble_overlap_strain(pat, U, use_compiled=False)
        force_py = dt.assemble_owned_force_from_local_stress(pat, stress, use_compiled=False)
        np.savez_compressed(HERE / f"pattern2d_{tag}.npz", elem_type=np.array("P2"), coord=m.coord, elem=m.elem,
                            q_mask=m.q_mask, owned_node_range=np.asarray(owned), ds=ds, U=U, stress=stress,
                            legacy_py=legacy_py, strain_py=strain_py, force_py=force_py, **pattern_arrays(pat))
        print("pattern2d", tag, pat.local_matrix_pattern.nnz, "nnz")


def gen_pattern_2d_p4(ref):
    """2D P4 (15-node triangles) on the reference's own slope generator (``mesh/slope_2d.py:351-376``,
    node order of ``mesh/textmesh_2d.py:116-184``); dphi come from the reference's basis table."""
    dt = ref["dt"]
    slope_2d = importlib.import_module("slope_stability.mesh.slope_2d")
    m = slope_2d.generate_homogeneous_slope_mesh_2d(elem_type="P4", h=5.0)
    coord, elem = np.asarray(m.coord, dtype=np.float64), np.asarray(m.elem, dtype=np.int64)
    q_mask = np.asarray(m.q_mask, dtype=bool)
    n_nodes = coord.shape[1]
    mat = {"c0": 6.0, "phi": 45.0, "psi": 0.0, "young": 2.0e4, "poisson": 0.49, "gamma_sat": 20.0,
           "gamma_unsat": 20.0}
    for tag, owned in (("P4_full", (0, n_nodes)), ("P4_partial", (n_nodes // 3, 2 * n_nodes // 3))):
        pat = dt.prepare_owned_tangent_pattern(coord, elem, q_mask, np.zeros(elem.shape[1], np.int64), [mat], owned,
                                               elem_type="P4", include_unique=(tag == "P4_full"))
        rng = np.random.default_rng(13)
        n_loc = pat.local_int_indices.size
        ds = rng.standard_normal((9, n_loc))
        U = rng.standard_normal((2, n_nodes))
        stress = rng.standard_normal((3, n_loc))
        legacy_py = dt.assemble_owned_tangent_values(pat, ds, use_compiled=False, kernel="legacy")
        strain_py = dt.assemble_overlap_strain(pat, U, use_compiled=False)
        force_py = dt.assemble_owned_force_from_local_stress(pat, stress, use_compiled=False)
        np.savez_compressed(HERE / f"pattern2d_{tag}.npz", elem_type=np.array("P4"), coord=coord, elem=elem,
                            q_mask=q_mask, owned_node_range=np.asarray(owned), ds=ds, U=U, stress=stress,
                            legacy_py=legacy_py, strain_py=strain_py, force_py=force_py, **pattern_arrays(pat))
        print("pattern2d", tag, pat.local_matrix_pattern.nnz, "nnz")


BDDC_KEYS = ("local_nodes", "local_elements", "local_coord", "local_q_mask", "local_global_dofs", "elastic_values",
             "local_assembly_weight", "dphi1", "dphi2", "dphi3", "local_int_indices", "overlap_local_positions",
             "scatter_map", "local_dirichlet_dofs", "constrained_diag_positions", "local_adjacency_indptr",
             "local_adjacency_indices", "local_primal_vertices", "owned_coord")


def bddc_cases():
    """(name, elem_type, coord, elem, q_mask, owned range, adjacency_source, corner_only_primals)."""
    from slope_stability_petsc4py_gb300 import synthetic

    slope_2d = importlib.import_module("slope_stability.mesh.slope_2d")
    def owner_range(elem, lo, hi):
        # elements belong to the subdomain owning their smallest node: cut at owner quantiles
        owners = np.sort(np.min(elem, axis=0))
        return int(owners[int(lo * (owners.size - 1))]), int(owners[int(hi * (owners.size - 1))])

    out = []
    m = synthetic.slope_mesh_3d(3, 2, 2, depth=6.0, elem_type="P2")
    n = m.coord.shape[1]
    out.append(("3d_P2_mid", "P2", m.coord, m.elem, m.q_mask, owner_range(m.elem, 0.3, 0.7), "csr", True))
    out.append(("3d_P2_all", "P2", m.coord, m.elem, m.q_mask, (0, n), "topology", False))
    out.append(("3d_P2_empty", "P2", m.coord, m.elem, m.q_mask, (n - 5, n), "csr", True))
    m4 = synthetic.slope_mesh_3d(2, 1, 1, depth=6.0, elem_type="P4")
    out.append(("3d_P4_head", "P4", m4.coord, m4.elem, m4.q_mask, owner_range(m4.elem, 0.0, 0.6), "topology", True))
    m2 = synthetic.slope_mesh_2d(4, 3, elem_type="P2")
    out.append(("2d_P2_tail", "P2", m2.coord, m2.elem, m2.q_mask, owner_range(m2.elem, 0.5, 1.0), "none", True))
    r4 = slope_2d.generate_homogeneous_slope_mesh_2d(elem_type="P4", h=5.0)
    e4 = np.asarray(r4.elem, dtype=np.int64)
    out.append(("2d_P4_mid", "P4", np.asarray(r4.coord, dtype=np.float64), e4, np.asarray(r4.q_mask, dtype=bool),
                owner_range(e4, 0.25, 0.75), "csr", False))
    return out


def gen_bddc(ref, kern):
    """BDDC subdomain patterns and tangent values (``fem/distributed_tangent.py:1178-1434``)."""
    dt = ref["dt"]
    for name, et, coord, elem, q_mask, owned, adj, corners in bddc_cases():
        dim = coord.shape[0]
        mat_id = (np.arange(elem.shape[1]) % 2).astype(np.int64)
        mats = [MATERIAL, dict(MATERIAL, young=2.0 * MATERIAL["young"], poisson=0.3)]
        owned_pat = dt.prepare_owned_tangent_pattern(coord, elem, q_mask, mat_id, mats, owned, elem_type=et,
                                                     include_unique=False)
        dt._kernels = kern  # the production path: elastic values through the compiled 3D kernel
        pat = dt.prepare_bddc_subdomain_pattern(coord, elem, q_mask, mat_id, mats, owned, elem_type=et,
                                                overlap_local_int_indices=owned_pat.local_int_indices,
                                                adjacency_source=adj, corner_only_primals=corners)
        ns = 6 if dim == 3 else 3
        rng = np.random.default_rng(17)
        ds = rng.standard_normal((ns * ns, pat.local_int_indices.size))
        dt._kernels = None
        values_py = dt.assemble_bddc_subdomain_tangent_values(pat, ds, use_compiled=False)
        extra = {}
        if dim == 3:
            dt._kernels = kern
            extra["values_c"] = dt.assemble_bddc_subdomain_tangent_values(pat, ds, use_compiled=True)
            dt._kernels = None
        np.savez_compressed(
            HERE / f"bddc_{name}.npz", elem_type=np.array(et), coord=coord, elem=elem, q_mask=q_mask,
            owned_node_range=np.asarray(owned), material_identifier=mat_id, adjacency_source=np.array(adj),
            corner_only_primals=np.array(corners), overlap_local_int_indices=owned_pat.local_int_indices, ds=ds,
            values_py=values_py, indptr=np.asarray(pat.local_matrix_pattern.indptr, dtype=np.int32),
            indices=np.asarray(pat.local_matrix_pattern.indices, dtype=np.int32),
            local_field_dofs=np.stack(pat.local_field_dofs) if pat.local_field_dofs[0].size else np.zeros((dim, 0), np.int32),
            n_p=np.int64(pat.n_p), n_q=np.int64(pat.n_q),
            **{k: np.asarray(getattr(pat, k)) for k in BDDC_KEYS}, **extra,
        )
        print("bddc", name, pat.local_matrix_pattern.nnz, "nnz", pat.local_elements.size, "elements")


def gmsh_like_tet4_mesh(seed=23):
    """A tet4 box mesh numbered the way a mesh file may be: shuffled vertex ids, shuffled element
    order, rotated vertex order per tet; boundary triangles labelled by box face (1: x=0, 2: x=max,
    3: z=0, 4: z=max, 5: y=0, 6: top) and two material ids."""
    from itertools import combinations

    from slope_stability_petsc4py_gb300 import synthetic

    rng = np.random.default_rng(seed)
    m = synthetic.slope_mesh_3d(3, 2, 2, depth=6.0, elem_type="P1")
    n_v = m.coord.shape[1]
    perm = rng.permutation(n_v)
    coord = np.empty_like(m.coord)
    coord[:, perm] = m.coord
    tet = perm[m.elem][:, rng.permutation(m.elem.shape[1])]
    rot = rng.integers(0, 4, tet.shape[1])
    tet = np.stack([np.roll(tet[:, e], rot[e]) for e in range(tet.shape[1])], axis=1)
    faces = {}
    for e in range(tet.shape[1]):
        for f in combinations(range(4), 3):
            key = tuple(sorted(tet[list(f), e]))
            faces[key] = (faces.get(key, (0, None))[0] + 1, tet[list(f), e])
    tris, labels = [], []
    x_max, z_max = coord[0].max(), coord[2].max()
    for key, (count, local) in faces.items():
        if count != 1:
            continue
        c = coord[:, list(key)]
        if np.all(c[0] < 1e-9):
            lab = 1
        elif np.all(c[0] > x_max - 1e-9):
            lab = 2
        elif np.all(c[2] < 1e-9):
            lab = 3
        elif np.all(c[2] > z_max - 1e-9):
            lab = 4
        elif np.all(c[1] < 1e-9):
            lab = 5
        else:
            lab = 6
        tris.append(local)
        labels.append(lab)
    order = rng.permutation(len(tris))
    tri = np.stack(tris, axis=1)[:, order]
    boundary = np.asarray(labels, dtype=np.int64)[order]
    material = (np.arange(tet.shape[1]) % 3).astype(np.int64)
    return coord, tet.astype(np.int64), tri.astype(np.int64), boundary, material


def gen_mesh_io(ref):
    """Tet4 -> tet10 / tet35 elevation and Dirichlet masks of the reference's gmsh loader
    (``io.py:61-93, 216-398``) on a file-like numbered tet4 mesh."""
    io = importlib.import_module("slope_stability.io")
    coord, tet, tri, boundary, material = gmsh_like_tet4_mesh()
    out = {"coord": coord, "tet4": tet, "tri3": tri, "boundary": boundary, "material": material}
    where = Path("/tmp/not_a_mesh_family/mesh.msh")  # outside the reference's meshes: default labels
    for order, fn in ((2, io._elevate_tet4_mesh_to_tet10), (4, io._elevate_tet4_mesh_to_tet35)):
        c, e, s = fn(coord, tet, tri)
        out[f"coord_p{order}"], out[f"elem_p{order}"], out[f"surf_p{order}"] = c, e, s
        for bt in (0, 1):
            out[f"q_mask_p{order}_bt{bt}"] = io._build_dirichlet_mask(3, c.shape[1], s, boundary, path=where,
                                                                     boundary_type=bt)
    out["q_mask_p1_bt0"] = io._build_dirichlet_mask(3, coord.shape[1], tri, boundary, path=where, boundary_type=0)
    field = {"boundary_0": np.array([11, 2]), "boundary_1": np.array([12, 2]), "material_0": np.array([7, 3]),
             "material_1": np.array([8, 3]), "other": np.array([9, 3])}
    out["physical_tags"] = np.array([12, 11, 11, 12], dtype=np.int64)
    out["physical_mapped"] = io._map_physical_ids(out["physical_tags"], field, 2, "boundary")
    np.savez_compressed(HERE / "mesh_io.npz", **out)
    print("mesh_io", tet.shape[1], "tets", tri.shape[1], "boundary triangles")


def gen_overlap_operator(ref):
    """The reference's overlap strain operator (``overlap_B``, include_overlap_B=True) and its
    ``OwnedElasticRows`` with the elastic values it projects onto the owned pattern, on a partially
    owned 3D P2 slope and a partially owned 2D P2 slope."""
    dt = ref["dt"]
    from slope_stability.fem.distributed_elastic import assemble_owned_elastic_rows

    from slope_stability_petsc4py_gb300 import synthetic

    mat = {"c0": 6.0, "phi": 45.0, "psi": 0.0, "young": 2.0e4, "poisson": 0.49, "gamma_sat": 20.0,
           "gamma_unsat": 20.0}
    for tag, m in (("3d", synthetic.slope_mesh_3d(3, 2, 2, depth=6.0, elem_type="P2")),
                   ("2d", synthetic.slope_mesh_2d(4, 3, elem_type="P2"))):
        n_nodes = m.coord.shape[1]
        owned = (n_nodes // 3, 2 * n_nodes // 3)
        mat_id = np.zeros(m.elem.shape[1], np.int64)
        rows = assemble_owned_elastic_rows(m.coord, m.elem, m.q_mask, mat_id, [mat], owned, elem_type="P2")
        pat = dt.prepare_owned_tangent_pattern(m.coord, m.elem, m.q_mask, mat_id, [mat], owned, elem_type="P2",
                                               include_unique=False, include_overlap_B=True, elastic_rows=rows)
        B, L = pat.overlap_B, rows.local_matrix.tocsr()
        np.savez_compressed(HERE / f"overlap_operator_{tag}.npz", coord=m.coord, elem=m.elem, q_mask=m.q_mask,
                            owned_node_range=np.asarray(owned), B_data=B.data, B_indices=B.indices,
                            B_indptr=B.indptr, B_shape=np.asarray(B.shape), L_data=L.data, L_indices=L.indices,
                            L_indptr=L.indptr, L_shape=np.asarray(L.shape), **pattern_arrays(pat))
        print("overlap_operator", tag, B.nnz, "B nnz", L.nnz, "elastic-row nnz")


GENERATORS = ("constitutive_3d", "constitutive_2d", "reduction", "patterns", "pattern_2d", "pattern_2d_p4", "bddc",
              "mesh_io", "potential", "overlap_operator")


def main(which=GENERATORS):
    """``python tests/golden/make_golden.py [generator ...]`` (default: all of GENERATORS)."""
    if not (REF_ROOT / "src" / "slope_stability").is_dir():
        raise SystemExit("set SSP_REFERENCE_ROOT to a reference checkout")
    oracle_py.build(ref=True)
    libref = oracle_py.ref_lib()
    assert libref is not None, "reference kernels did not build"
    ref = import_reference()
    kern = compiled_kernels_module(libref)
    if "constitutive_3d" in which:
        gen_constitutive(kern, ref["problem"], libref)
    if "constitutive_2d" in which:
        gen_constitutive_2d(ref["problem"], ref["reduction"])
    if "reduction" in which:
        gen_reduction(ref["reduction"])
    if "patterns" in which:
        gen_patterns(ref, kern)
    if "pattern_2d" in which:
        gen_pattern_2d(ref)
    if "pattern_2d_p4" in which:
        gen_pattern_2d_p4(ref)
    if "bddc" in which:
        gen_bddc(ref, kern)
    if "mesh_io" in which:
        gen_mesh_io(ref)
    if "potential" in which:
        gen_potential(ref["problem"], ref["reduction"])
    if "overlap_operator" in which:
        gen_overlap_operator(ref)


if __name__ == "__main__":
    main(tuple(sys.argv[1:]) or GENERATORS)
