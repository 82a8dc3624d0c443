"""Python side of the oracle: ctypes access to the C restatement plus NumPy restatements.

TEST INFRASTRUCTURE ONLY.  The product package never imports this module; it is the
oracle used by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py``.

Restated reference routines (paths relative to the reference project root):

* ``constitutive_2d``      -- src/slope_stability/constitutive/problem.py:143-475
* ``potential_2d``, ``potential_3d`` -- src/slope_stability/constitutive/problem.py:1029-1190
* ``reduction``            -- src/slope_stability/constitutive/reduction.py:14-78
* ``geometry``             -- src/slope_stability/fem/assembly.py:50-136 (2D), :139-245 (3D)
* ``owned_pattern``        -- src/slope_stability/fem/distributed_tangent.py:297-478, 937-1175
  (structural CSR, row maps, element->CSR scatter map, row-slot metadata, overlap dofs); pure
  Python, for small meshes
* ``owned_pattern_c``      -- the same pattern (without the legacy scatter map) through the C
  restatement ``orc_pattern_build`` in ``oracle.c``, for meshes of millions of elements
* ``geometry_3d_c``        -- src/slope_stability/fem/assembly.py:139-245 through ``orc_geometry_3d``
* the C functions in ``oracle.c`` (see its header) for the 3D kernels.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
REF_LIB_PATH = HERE / "_ref" / "libref.so"

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_up = ctypes.POINTER(ctypes.c_uint8)


def build(ref: bool = False) -> None:
    targets = ["all"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", str(HERE), *targets], check=True)


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            build()
        _LIB = ctypes.CDLL(str(LIB_PATH))
        _LIB.orc_mc3d_point.restype = None
    return _LIB


def nofma_lib():
    """The C restatement compiled without fused multiply-adds (-ffp-contract=off)."""
    path = HERE / "_build" / "liboracle_nofma.so"
    if not path.exists():
        build()
    return ctypes.CDLL(str(path))


def ref_lib():
    """The reference's own C kernels compiled from its sources (only where it is mounted)."""
    if not REF_LIB_PATH.exists():
        return None
    return ctypes.CDLL(str(REF_LIB_PATH))


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def num_threads() -> int:
    lib().orc_num_threads.restype = ctypes.c_int
    return int(lib().orc_num_threads())


def set_num_threads(n: int) -> None:
    """OpenMP threads of the C restatement's kernels (omp_set_num_threads)."""
    lib().orc_set_num_threads(ctypes.c_int(int(n)))


_PATTERN_ARRAYS = (("overlap_elements", np.int64), ("overlap_nodes", np.int64), ("overlap_element_dof_lids", np.int32),
                   ("indptr", np.int32), ("indices", np.int32), ("constrained_diag_positions", np.int32),
                   ("row_slot_ptr", np.int32), ("slot_elem", np.int32), ("slot_lrow", np.uint8),
                   ("slot_pos", np.int32))


def owned_pattern_c(elem, q_mask, owned_node_range):
    """``owned_pattern`` through the C restatement (no legacy scatter map), as a dict of arrays."""
    L = lib()
    L.orc_pattern_build.restype = ctypes.c_void_p
    elem = np.asarray(elem, dtype=np.int64)
    q_mask = np.asarray(q_mask, dtype=bool)
    dim, n_nodes = q_mask.shape
    n_p, n_elem = elem.shape
    nld = dim * n_p
    elem_em = np.ascontiguousarray(elem.T)
    free = np.ascontiguousarray(q_mask.reshape(-1, order="F").astype(np.uint8))
    n0, n1 = (int(v) for v in owned_node_range)
    h = L.orc_pattern_build(ctypes.c_int(dim), ctypes.c_int64(n_nodes), ctypes.c_int(n_p), ctypes.c_int64(n_elem),
                            elem_em.ctypes.data_as(ctypes.c_void_p), free.ctypes.data_as(ctypes.c_void_p),
                            ctypes.c_int64(n0), ctypes.c_int64(n1))
    if not h:
        raise MemoryError("orc_pattern_build failed (allocation, or an index beyond int32)")
    try:
        sz = np.zeros(6, dtype=np.int64)
        L.orc_pattern_sizes(ctypes.c_void_p(h), sz.ctypes.data_as(ctypes.c_void_p))
        n_ov, n_ovn, n_rows, nnz, n_slots, n_cd = (int(v) for v in sz)
        shapes = {"overlap_elements": (n_ov,), "overlap_nodes": (n_ovn,), "overlap_element_dof_lids": (n_ov, nld),
                  "indptr": (n_rows + 1,), "indices": (nnz,), "constrained_diag_positions": (n_cd,),
                  "row_slot_ptr": (n_rows + 1,), "slot_elem": (n_slots,), "slot_lrow": (n_slots,),
                  "slot_pos": (n_slots, nld)}
        out = {}
        for k, (name, dt) in enumerate(_PATTERN_ARRAYS):
            a = np.empty(shapes[name], dtype=dt)
            if a.size:
                L.orc_pattern_copy(ctypes.c_void_p(h), ctypes.c_int(k), a.ctypes.data_as(ctypes.c_void_p))
            out[name] = a
    finally:
        L.orc_pattern_free(ctypes.c_void_p(h))
    nodes = out["overlap_nodes"]
    lid = np.full(n_nodes, -1, dtype=np.int64)
    lid[nodes] = np.arange(nodes.size)
    gdofs = lambda v: (dim * np.repeat(v, dim) + np.tile(np.arange(dim), v.size)).astype(np.int64)  # noqa: E731
    out["overlap_global_dofs"] = gdofs(nodes)
    out["owned_local_overlap_dofs"] = gdofs(lid[np.arange(n0, n1)])
    out["owned_free_mask"] = free[dim * n0:dim * n1].astype(bool)
    return out


def elastic_ds(dim, shear, bulk, lame):
    """Per-point elastic D blocks (n, n_s*n_s), each column-major, of build_elastic_stiffness_matrix
    (src/slope_stability/fem/assembly.py:281-302): K vol + 2G (I_half - vol/3) in 3D,
    lame vol + 2G diag(1, 1, 1/2) in 2D."""
    shear, bulk, lame = (np.asarray(a, dtype=np.float64).ravel() for a in (shear, bulk, lame))
    if dim == 3:
        iota = np.array([1.0, 1.0, 1.0, 0.0, 0.0, 0.0])
        vol = np.outer(iota, iota)
        ident = np.diag([1.0, 1.0, 1.0, 0.5, 0.5, 0.5]) - vol / 3.0
        coeff = bulk
    else:
        iota = np.array([1.0, 1.0, 0.0])
        vol = np.outer(iota, iota)
        ident = np.diag([1.0, 1.0, 0.5])
        coeff = lame
    return np.ascontiguousarray(coeff[:, None] * vol.reshape(-1, order="F")[None, :]
                                + 2.0 * shear[:, None] * ident.reshape(-1, order="F")[None, :])


def scatter_from_slots(p, n_ld):
    """The element -> CSR scatter map (distributed_tangent.py:328-366) from row-slot metadata: row
    slot (element e, local dof a) holds exactly scatter[e, a*n_ld : (a+1)*n_ld] (the reference's own
    test pins slot_pos to the scatter map, tests/test_distributed_tangent_rows.py:135-153)."""
    n_ov = p["overlap_elements"].size
    scatter = np.full((n_ov, n_ld * n_ld), -1, dtype=np.int32)
    rows = p["slot_elem"].astype(np.int64)
    cols = p["slot_lrow"].astype(np.int64)[:, None] * n_ld + np.arange(n_ld)[None, :]
    scatter[rows[:, None], cols] = p["slot_pos"]
    return scatter


def geometry_3d_c(coord, elem, dhat, wf):
    """3D ``geometry`` through the C restatement: dphi1..3 (n_int, n_p) and weights (n_int,).
    ``elem`` is (n_p, n_el) node ids, ``dhat`` (3, n_p, n_q)."""
    coord = _c(coord, np.float64)
    elem_em = np.ascontiguousarray(np.asarray(elem, dtype=np.int64).T)
    dhat = _c(dhat, np.float64)
    wf = _c(wf, np.float64)
    n_el, n_p = elem_em.shape
    n_q = dhat.shape[2]
    d = [np.empty((n_el * n_q, n_p)) for _ in range(3)]
    w = np.empty(n_el * n_q)
    vp = ctypes.c_void_p
    lib().orc_geometry_3d(coord.ctypes.data_as(vp), ctypes.c_int64(coord.shape[1]), elem_em.ctypes.data_as(vp),
                          ctypes.c_int64(n_el), ctypes.c_int(n_p), ctypes.c_int(n_q), dhat.ctypes.data_as(vp),
                          wf.ctypes.data_as(vp), *[x.ctypes.data_as(vp) for x in d], w.ctypes.data_as(vp))
    return d, w


# --------------------------------------------------------------------------- 3D kernels


def constitutive_3d(E, c_bar, sin_phi, shear, bulk, lame, *, tangent=True, library=None):
    """AoS E (n, 6) -> S (n, 6) [, DS (n, 36)] through the C restatement (or ``library``,
    which may be the reference's own compiled kernels)."""
    E = _c(E, np.float64)
    n = E.shape[0]
    args = [_c(a, np.float64) for a in (c_bar, sin_phi, shear, bulk, lame)]
    S = np.empty((n, 6))
    DS = np.empty((n, 36)) if tangent else None
    L = library or lib()
    if hasattr(L, "orc_constitutive_3d"):  # this restatement (or its no-FMA build)
        L.orc_constitutive_3d(_d(E), *[_d(a) for a in args], ctypes.c_int(n), _d(S),
                              _d(DS) if tangent else None)
    elif tangent:
        L.constitutive_problem_3d_sds_batch_c(_d(E), *[_d(a) for a in args], ctypes.c_int(n), _d(S), _d(DS))
    else:
        L.constitutive_problem_3d_s_batch_c(_d(E), *[_d(a) for a in args], ctypes.c_int(n), _d(S))
    return (S, DS) if tangent else S


def strain_3d(dphi1, dphi2, dphi3, u_overlap, dof_lids, n_q, library=None):
    d1, d2, d3 = (_c(a, np.float64) for a in (dphi1, dphi2, dphi3))
    dof = _c(dof_lids, np.int32)
    u = _c(u_overlap, np.float64)
    n_elem, nld = dof.shape
    n_p = nld // 3
    E = np.empty((n_elem * n_q, 6))
    (library or lib()).orc_strain_3d(_d(d1), _d(d2), _d(d3), _d(u), _i(dof), n_elem, n_p, n_q, _d(E))
    return E


def force_rows_3d(dphi1, dphi2, dphi3, S, w, row_slot_ptr, slot_elem, slot_lrow, n_q, library=None):
    d1, d2, d3 = (_c(a, np.float64) for a in (dphi1, dphi2, dphi3))
    S = _c(S, np.float64)
    w = _c(w, np.float64)
    rp, se = _c(row_slot_ptr, np.int32), _c(slot_elem, np.int32)
    sl = _c(slot_lrow, np.uint8)
    n_rows = rp.size - 1
    F = np.zeros(n_rows)
    (library or lib()).orc_force_rows_3d(_d(d1), _d(d2), _d(d3), _d(S), _d(w), _i(rp), _i(se),
                            sl.ctypes.data_as(_up), n_rows, d1.shape[1], n_q, _d(F))
    return F


def tangent_rows_3d(dphi1, dphi2, dphi3, DS, w, row_slot_ptr, slot_elem, slot_lrow, slot_pos, n_q, nnz, library=None):
    d1, d2, d3 = (_c(a, np.float64) for a in (dphi1, dphi2, dphi3))
    DS, w = _c(DS, np.float64), _c(w, np.float64)
    rp, se, sp = _c(row_slot_ptr, np.int32), _c(slot_elem, np.int32), _c(slot_pos, np.int32)
    sl = _c(slot_lrow, np.uint8)
    out = np.zeros(int(nnz))
    (library or lib()).orc_tangent_rows_3d(_d(d1), _d(d2), _d(d3), _d(DS), _d(w), _i(rp), _i(se),
                              sl.ctypes.data_as(_up), _i(sp), rp.size - 1, d1.shape[1], n_q, _d(out))
    return out


def tangent_scatter(dim, dphi1, dphi2, dphi3, DS, w, scatter_map, n_q, nnz):
    d1, d2 = _c(dphi1, np.float64), _c(dphi2, np.float64)
    d3 = _c(dphi3, np.float64) if dim == 3 else np.zeros(1)
    DS, w, sm = _c(DS, np.float64), _c(w, np.float64), _c(scatter_map, np.int32)
    n_p = d1.shape[1]
    nld = dim * n_p
    ns = 6 if dim == 3 else 3
    work = np.empty(nld * nld + 2 * ns * nld)
    out = np.zeros(int(nnz))
    lib().orc_tangent_scatter(dim, _d(d1), _d(d2), _d(d3), _d(DS), _d(w), _i(sm), sm.shape[0], n_p, n_q,
                              _d(out), _d(work))
    return out


def strain_2d(dphi1, dphi2, u_overlap, dof_lids, n_q):
    d1, d2 = _c(dphi1, np.float64), _c(dphi2, np.float64)
    dof, u = _c(dof_lids, np.int32), _c(u_overlap, np.float64)
    E = np.empty((dof.shape[0] * n_q, 3))
    lib().orc_strain_2d(_d(d1), _d(d2), _d(u), _i(dof), dof.shape[0], d1.shape[1], n_q, _d(E))
    return E


def overlap_force_2d(dphi1, dphi2, S, w, dof_lids, n_q, n_overlap_dofs):
    d1, d2 = _c(dphi1, np.float64), _c(dphi2, np.float64)
    S, w, dof = _c(S, np.float64), _c(w, np.float64), _c(dof_lids, np.int32)
    out = np.zeros(int(n_overlap_dofs))
    lib().orc_overlap_force_2d(_d(d1), _d(d2), _d(S), _d(w), _i(dof), dof.shape[0], d1.shape[1], n_q, _d(out))
    return out


# --------------------------------------------------------------------------- NumPy restatements


def reduction(c0, phi, psi, lam, davis_type="A"):
    """Davis-type strength reduction -> (c_bar, sin_phi)."""
    c0, phi, psi = (np.asarray(a, dtype=np.float64) for a in (c0, phi, psi))
    if lam <= 0:
        raise ValueError("lambda must be positive")
    t = str(davis_type).upper()
    if t == "A":
        beta = np.cos(phi) * np.cos(psi) / (1.0 - np.sin(phi) * np.sin(psi))
        c_l = beta * c0 / lam
        phi_l = np.arctan(beta * np.tan(phi) / lam)
    elif t == "B":
        c1 = c0 / lam
        phi1 = np.arctan(np.tan(phi) / lam)
        psi1 = np.arctan(np.tan(psi) / lam)
        beta = np.cos(phi1) * np.cos(psi1) / (1.0 - np.sin(phi1) * np.sin(psi1))
        c_l = beta * c1
        phi_l = np.arctan(beta * np.tan(phi1))
    elif t == "C":
        c1 = c0 / lam
        phi1 = np.arctan(np.tan(phi) / lam)
        beta = np.where(phi1 > psi, np.cos(phi1) * np.cos(psi) / (1.0 - np.sin(phi1) * np.sin(psi)), 1.0)
        c_l = beta * c1
        phi_l = np.arctan(beta * np.tan(phi1))
    else:
        raise ValueError("unknown Davis type")
    return 2.0 * c_l * np.cos(phi_l), np.sin(phi_l)


def _outer9(a, b):
    """Column-major 3x3 outer products a_i b_j at k = i + 3 j, for columns of (3, n)."""
    return (a[:, None, :] * b[None, :, :]).reshape(9, -1, order="F")


def constitutive_2d(E, c_bar, sin_phi, shear, bulk, lame, tangent=True):
    """Plane-strain Mohr-Coulomb return mapping, E (3, n) -> S (4, n) [, DS (9, n)]."""
    E = np.asarray(E, dtype=np.float64)
    n = E.shape[1]
    c, s, G, lam = (np.asarray(a, dtype=np.float64).ravel() for a in (c_bar, sin_phi, shear, lame))
    e11, e22, g12 = E
    tr2 = e11 + e22
    rad = np.sqrt((e11 - e22) ** 2 + g12 ** 2)
    ev0 = np.stack((0.5 * (tr2 + rad), 0.5 * (tr2 - rad), np.zeros(n)))
    act = rad != 0.0
    P0 = np.zeros((4, n))
    with np.errstate(divide="ignore", invalid="ignore"):
        P0[0] = np.where(act, (e11 - ev0[1]) / rad, 1.0)
        P0[1] = np.where(act, (e22 - ev0[1]) / rad, 1.0)
        P0[2] = np.where(act, (g12 / 2.0) / rad, 0.0)
    P1 = np.vstack((np.ones((2, n)), np.zeros((2, n)))) - P0
    P2 = np.vstack((np.zeros((3, n)), np.ones((1, n))))
    dP0 = np.zeros((9, n))
    a, b = P0[:3], P1[:3]
    halfI = np.array([1.0, 1.0, 0.5])
    with np.errstate(divide="ignore", invalid="ignore"):
        for j in range(3):
            for i in range(3):
                v = (halfI[i] if i == j else 0.0) - a[i] * a[j] - b[i] * b[j]
                dP0[i + 3 * j] = np.where(act, v / rad, 0.0)
    eig = [ev0[0].copy(), ev0[1].copy(), ev0[2].copy()]
    P = [P0.copy(), P1.copy(), P2.copy()]
    dP = [dP0.copy(), -dP0, np.zeros((9, n))]
    t2 = (ev0[0] >= ev0[2]) & (ev0[2] > ev0[1])
    t3 = ev0[2] > ev0[0]
    src0 = [(ev0[0], P0, dP0), (ev0[1], P1, -dP0), (ev0[2], P2, np.zeros((9, n)))]
    # order (0,2,1) where t2, (2,0,1) where t3
    for k, (o2, o3) in enumerate(((0, 2), (2, 0), (1, 1))):
        for mask, origin in ((t2, o2), (t3, o3)):
            eig[k][mask] = src0[origin][0][mask]
            P[k][:, mask] = src0[origin][1][:, mask]
            dP[k][:, mask] = src0[origin][2][:, mask]
    e1, e2, e3 = eig
    tr = e1 + e2 + e3
    f_tr = 2.0 * G * ((1.0 + s) * e1 - (1.0 - s) * e3) + 2.0 * lam * s * tr - c
    g_sl = (e1 - e2) / (1.0 + s)
    g_sr = (e2 - e3) / (1.0 - s)
    g_la = (e1 + e2 - 2.0 * e3) / (3.0 - s)
    g_ra = (2.0 * e1 - e2 - e3) / (3.0 + s)
    d_s = 4.0 * lam * s ** 2 + 2.0 * G * (1.0 + s) ** 2 + 2.0 * G * (1.0 - s) ** 2
    d_l = 4.0 * lam * s ** 2 + G * (1.0 + s) ** 2 + 2.0 * G * (1.0 - s) ** 2
    d_r = 4.0 * lam * s ** 2 + 2.0 * G * (1.0 + s) ** 2 + G * (1.0 - s) ** 2
    l_s = f_tr / d_s
    l_l = (G * ((1.0 + s) * (e1 + e2) - 2.0 * (1.0 - s) * e3) + 2.0 * lam * s * tr - c) / d_l
    l_r = (G * (2.0 * (1.0 + s) * e1 - (1.0 - s) * (e2 + e3)) + 2.0 * lam * s * tr - c) / d_r

    iota4 = np.array([1.0, 1.0, 0.0, 1.0])
    vol3 = np.outer(iota4[:3], iota4[:3]).reshape(-1, order="F")
    id3 = np.diag([1.0, 1.0, 0.5]).reshape(-1, order="F")
    Etr = np.vstack((E, np.zeros((1, n))))
    S = np.zeros((4, n))
    DS = np.zeros((9, n))
    el = f_tr <= 0.0
    S[:, el] = lam[el] * (np.outer(iota4, iota4) @ Etr[:, el]) + 2.0 * G[el] * (np.diag([1.0, 1.0, 0.5, 1.0]) @ Etr[:, el])
    DS[:, el] = vol3[:, None] * lam[el] + 2.0 * id3[:, None] * G[el]
    vol_term = vol3[:, None] * lam[None, :]
    bm = np.array([1.0, 1.0, 0.0])[:, None]

    sm = (l_s <= np.minimum(g_sl, g_sr)) & ~el
    sig1 = lam * tr + 2.0 * G * e1 - l_s * (2.0 * lam * s + 2.0 * G * (1.0 + s))
    sig2 = lam * tr + 2.0 * G * e2 - l_s * (2.0 * lam * s)
    sig3 = lam * tr + 2.0 * G * e3 - l_s * (2.0 * lam * s - 2.0 * G * (1.0 - s))
    S[:, sm] = (sig1 * P[0] + sig2 * P[1] + sig3 * P[2])[:, sm]
    q6 = 2.0 * G * (1.0 + s) * P[0][:3] - 2.0 * G * (1.0 - s) * P[2][:3] + bm * (2.0 * lam * s)
    ds_s = (sig1 * dP[0] + sig2 * dP[1] + sig3 * dP[2] + vol_term
            + 2.0 * G * (_outer9(P[0][:3], P[0][:3]) + _outer9(P[1][:3], P[1][:3]) + _outer9(P[2][:3], P[2][:3]))
            - _outer9(q6, q6) / d_s)
    DS[:, sm] = ds_s[:, sm]

    lm = (g_sl < g_sr) & (l_l >= g_sl) & (l_l <= g_la) & ~(el | sm)
    s1 = lam * tr + G * (e1 + e2) - l_l * (2.0 * lam * s + G * (1.0 + s))
    s3 = lam * tr + 2.0 * G * e3 - l_l * (2.0 * lam * s - 2.0 * G * (1.0 - s))
    P12 = P[0] + P[1]
    S[:, lm] = (s1 * P12 + s3 * P[2])[:, lm]
    q6 = G * (1.0 + s) * P12[:3] - 2.0 * G * (1.0 - s) * P[2][:3] + bm * (2.0 * lam * s)
    ds_l = (s1 * (dP[0] + dP[1]) + s3 * dP[2] + vol_term + G * _outer9(P12[:3], P12[:3])
            + 2.0 * G * _outer9(P[2][:3], P[2][:3]) - _outer9(q6, q6) / d_l)
    DS[:, lm] = ds_l[:, lm]

    rm = (g_sl > g_sr) & (l_r >= g_sr) & (l_r <= g_ra) & ~(el | sm)
    s1 = lam * tr + 2.0 * G * e1 - l_r * (2.0 * lam * s + 2.0 * G * (1.0 + s))
    s3 = lam * tr + G * (e2 + e3) - l_r * (2.0 * lam * s - G * (1.0 - s))
    P23 = P[1] + P[2]
    S[:, rm] = (s1 * P[0] + s3 * P23)[:, rm]
    q6 = 2.0 * G * (1.0 + s) * P[0][:3] - G * (1.0 - s) * P23[:3] + bm * (2.0 * lam * s)
    ds_r = (s1 * dP[0] + s3 * (dP[1] + dP[2]) + vol_term + 2.0 * G * _outer9(P[0][:3], P[0][:3])
            + G * _outer9(P23[:3], P23[:3]) - _outer9(q6, q6) / d_r)
    DS[:, rm] = ds_r[:, rm]

    ap = ~(el | sm | lm | rm)
    S[:, ap] = iota4[:, None] * (c[ap] / (2.0 * s[ap]))[None, :]
    DS[:, ap] = 0.0
    return (S, DS) if tangent else S


def _np_safe_denominator(d):
    """The reference's guard: a denominator below 1e-15 in magnitude becomes +-1e-15."""
    return np.where(np.abs(d) < 1.0e-15, np.sign(d + 1.0e-15) * 1.0e-15, d)


def _mc_potential(e1, e2, e3, tr, c, s, G, K, lam, d_s, d_l, d_r):
    """Branch selection and energy shared by the 2D and 3D potentials (the reference's
    src/slope_stability/constitutive/problem.py:1075-1108 and :1158-1190)."""
    f_tr = 2.0 * G * ((1.0 + s) * e1 - (1.0 - s) * e3) + 2.0 * (lam * s) * tr - c
    g_sl = (e1 - e2) / np.maximum(1.0e-15, 1.0 + s)
    g_sr = (e2 - e3) / np.maximum(1.0e-15, 1.0 - s)
    g_la = (e1 + e2 - 2.0 * e3) / np.maximum(1.0e-15, 3.0 - s)
    g_ra = (2.0 * e1 - e2 - e3) / np.maximum(1.0e-15, 3.0 + s)
    d_a = 4.0 * K * s ** 2
    l_s = f_tr / _np_safe_denominator(d_s)
    l_l = (G * ((1.0 + s) * (e1 + e2) - 2.0 * (1.0 - s) * e3) + 2.0 * lam * s * tr - c) / _np_safe_denominator(d_l)
    l_r = (G * (2.0 * (1.0 + s) * e1 - (1.0 - s) * (e2 + e3)) + 2.0 * lam * s * tr - c) / _np_safe_denominator(d_r)
    l_a = (2.0 * K * s * tr - c) / _np_safe_denominator(d_a)
    vol = 0.5 * lam * tr ** 2
    el = f_tr <= 0.0
    sm = (l_s <= np.minimum(g_sl, g_sr)) & ~el
    lm = (g_sl < g_sr) & (l_l >= g_sl) & (l_l <= g_la) & ~(el | sm)
    rm = (g_sl > g_sr) & (l_r >= g_sr) & (l_r <= g_ra) & ~(el | sm)
    elastic = vol + G * (e1 ** 2 + e2 ** 2 + e3 ** 2)
    psi = 0.5 * K * tr ** 2 - 0.5 * d_a * l_a ** 2
    psi = np.where(rm, vol + G * (e1 ** 2 + 0.5 * (e2 + e3) ** 2) - 0.5 * d_r * l_r ** 2, psi)
    psi = np.where(lm, vol + G * (e3 ** 2 + 0.5 * (e1 + e2) ** 2) - 0.5 * d_l * l_l ** 2, psi)
    psi = np.where(sm, elastic - 0.5 * d_s * l_s ** 2, psi)
    psi = np.where(el, elastic, psi)
    branch = np.select([el, sm, lm, rm], [0, 1, 2, 3], 4).astype(np.int8)
    return psi, branch


def potential_3d(E, c_bar, sin_phi, shear, bulk, lame, *, with_branch=False):
    """Mohr-Coulomb potential energy density, E (6, n) -> Psi (n,)  (the reference's
    ``potential_3D``, src/slope_stability/constitutive/problem.py:1111-1190).

    As the reference does: the invariants take E's rows 3, 4, 5 as the tensor entries
    (12), (13), (23) without halving the engineering shears, while E is ordered
    [11, 22, 33, 12, 23, 13] -- so I3 pairs e22 with gamma_23 and e11 with gamma_13 -- and the
    eigenvalues come from the trigonometric formula with the 1e-15 guard on sqrt(Q^3)."""
    E = np.asarray(E, dtype=np.float64)
    c, s, G, K, lam = (np.asarray(a, dtype=np.float64).ravel() for a in (c_bar, sin_phi, shear, bulk, lame))
    e11, e22, e33, r3, r4, r5 = E
    I1 = e11 + e22 + e33
    I2 = e11 * e22 + e11 * e33 + e22 * e33 - r3 * r3 - r4 * r4 - r5 * r5
    I3 = e11 * e22 * e33 - e33 * r3 * r3 - e22 * r4 * r4 - e11 * r5 * r5 + 2.0 * r3 * r4 * r5
    Q = np.maximum(0.0, (I1 * I1 - 3.0 * I2) / 9.0)
    R = (-2.0 * I1 ** 3 + 9.0 * I1 * I2 - 27.0 * I3) / 54.0
    theta = np.zeros_like(Q)
    on = Q > 0
    with np.errstate(divide="ignore", invalid="ignore"):
        theta[on] = np.arccos(np.clip(R[on] / np.maximum(1.0e-15, np.sqrt(Q[on] ** 3)), -1.0, 1.0)) / 3.0
    rq = np.sqrt(Q)
    e1 = -2.0 * rq * np.cos(theta + 2.0 * np.pi / 3.0) + I1 / 3.0
    e2 = -2.0 * rq * np.cos(theta - 2.0 * np.pi / 3.0) + I1 / 3.0
    e3 = -2.0 * rq * np.cos(theta) + I1 / 3.0
    d_s = 4.0 * lam * s ** 2 + 4.0 * G * (1.0 + s ** 2)
    d_l = 4.0 * lam * s ** 2 + G * (1.0 + s) * (1.0 + s) + 2.0 * G * (1.0 - s) * (1.0 - s)
    d_r = 4.0 * lam * s ** 2 + 2.0 * G * (1.0 + s) * (1.0 + s) + G * (1.0 - s) * (1.0 - s)
    with np.errstate(divide="ignore", invalid="ignore"):
        psi, br = _mc_potential(e1, e2, e3, I1, c, s, G, K, lam, d_s, d_l, d_r)
    return (psi, br) if with_branch else psi


def potential_2d(E, c_bar, sin_phi, shear, bulk, lame, *, with_branch=False):
    """Plane-strain potential energy density, E (3, n) -> Psi (n,)  (the reference's
    ``potential_2D``, src/slope_stability/constitutive/problem.py:1029-1108).

    As the reference's arrays do (its sorted eigenvalues alias the unsorted ones, so the
    reordering overwrites before it reads): where the in-plane eigenvalues straddle the
    out-of-plane zero (e_a >= 0 > e_b) the sorted triple is (e_a, 0, 0), and where both are
    negative it is (0, 0, 0); otherwise (e_a, e_b, 0)."""
    E = np.asarray(E, dtype=np.float64)
    c, s, G, K, lam = (np.asarray(a, dtype=np.float64).ravel() for a in (c_bar, sin_phi, shear, bulk, lame))
    e11, e22, g12 = E
    tr2 = e11 + e22
    rad = np.sqrt((e11 - e22) ** 2 + g12 * g12)
    ea, eb = (tr2 + rad) / 2.0, (tr2 - rad) / 2.0
    straddle = (ea >= 0.0) & (0.0 > eb)
    negative = 0.0 > ea
    e1 = np.where(negative, 0.0, ea)
    e2 = np.where(straddle | negative, 0.0, eb)
    e3 = np.zeros_like(ea)
    tr = e1 + e2 + e3
    d_s = 4.0 * lam * s ** 2 + 2.0 * G * (1.0 + s) ** 2 + 2.0 * G * (1.0 - s) ** 2
    d_l = 4.0 * lam * s ** 2 + G * (1.0 + s) ** 2 + 2.0 * G * (1.0 - s) ** 2
    d_r = 4.0 * lam * s ** 2 + 2.0 * G * (1.0 + s) ** 2 + G * (1.0 - s) ** 2
    with np.errstate(divide="ignore", invalid="ignore"):
        psi, br = _mc_potential(e1, e2, e3, tr, c, s, G, K, lam, d_s, d_l, d_r)
    return (psi, br) if with_branch else psi


def geometry(coord, elem, dim, dhat, wf):
    """dphi (dim arrays of shape (n_int, n_p)) and weights (n_int,) of every quadrature point.

    ``dhat`` is (dim, n_p, n_q) reference gradients, ``wf`` the rule's weights."""
    coord = np.asarray(coord, dtype=np.float64)
    elem = np.asarray(elem, dtype=np.int64)
    n_p, n_e = elem.shape
    n_q = dhat.shape[2]
    X = coord[:, elem]  # (dim, n_p, n_e)
    # J[r][c] = sum_a X[c, a, e] * dhat[r, a, q]
    J = np.einsum("cae,raq->eqrc", X, dhat)
    if dim == 3:
        j11, j12, j13 = J[..., 0, 0], J[..., 0, 1], J[..., 0, 2]
        j21, j22, j23 = J[..., 1, 0], J[..., 1, 1], J[..., 1, 2]
        j31, j32, j33 = J[..., 2, 0], J[..., 2, 1], J[..., 2, 2]
        det = j11 * (j22 * j33 - j23 * j32) - j12 * (j21 * j33 - j23 * j31) + j13 * (j21 * j32 - j22 * j31)
        inv = 1.0 / det
        h1, h2, h3 = (np.transpose(dhat[r], (1, 0))[None, :, :] for r in range(3))  # (1, q, a)
        c = lambda v: v[..., None]  # noqa: E731
        d1 = (c(j22 * j33 - j23 * j32) * h1 - c(j12 * j33 - j13 * j32) * h2 + c(j12 * j23 - j13 * j22) * h3) * c(inv)
        d2 = (-c(j21 * j33 - j23 * j31) * h1 + c(j11 * j33 - j13 * j31) * h2 - c(j11 * j23 - j13 * j21) * h3) * c(inv)
        d3 = (c(j21 * j32 - j22 * j31) * h1 - c(j11 * j32 - j12 * j31) * h2 + c(j11 * j22 - j12 * j21) * h3) * c(inv)
        w = (np.asarray(wf)[None, :] * np.abs(det)).reshape(-1)
        return [d.reshape(n_e * n_q, n_p) for d in (d1, d2, d3)], w
    j11, j12, j21, j22 = J[..., 0, 0], J[..., 0, 1], J[..., 1, 0], J[..., 1, 1]
    det = j11 * j22 - j12 * j21
    h1, h2 = (np.transpose(dhat[r], (1, 0))[None, :, :] for r in range(2))
    c = lambda v: v[..., None]  # noqa: E731
    d1 = c(j22 / det) * h1 + c(-j12 / det) * h2
    d2 = c(-j21 / det) * h1 + c(j11 / det) * h2
    w = (np.abs(det) * np.asarray(wf)[None, :]).reshape(-1)
    return [d.reshape(n_e * n_q, n_p) for d in (d1, d2)], w


def owned_pattern(elem, q_mask, owned_node_range):
    """Structural owned-row CSR, scatter map and row-slot metadata, as plain dict of arrays."""
    elem = np.asarray(elem, dtype=np.int64)
    q_mask = np.asarray(q_mask, dtype=bool)
    dim, n_nodes = q_mask.shape
    n_p = elem.shape[0]
    nld = dim * n_p
    n0, n1 = (int(v) for v in owned_node_range)
    row0, row1 = dim * n0, dim * n1
    n_rows = row1 - row0
    free = q_mask.reshape(-1, order="F")
    ov_el = np.flatnonzero(np.any((elem >= n0) & (elem < n1), axis=0))
    ov_nodes = np.unique(elem[:, ov_el].reshape(-1, order="F")) if ov_el.size else np.empty(0, np.int64)
    lid = np.full(n_nodes, -1, dtype=np.int64)
    lid[ov_nodes] = np.arange(ov_nodes.size)
    gdofs = lambda nodes: (dim * np.repeat(nodes, dim) + np.tile(np.arange(dim), nodes.size))  # noqa: E731
    dof_lids = np.stack([gdofs(lid[elem[:, e]]) for e in ov_el]).astype(np.int32) if ov_el.size else np.empty((0, nld), np.int32)
    cols = [set() for _ in range(n_rows)]
    for e in ov_el:
        dofs = gdofs(elem[:, e])
        fc = [int(v) for v in dofs if free[v]]
        for r in dofs:
            if row0 <= r < row1 and free[r]:
                cols[r - row0].update(fc)
    for lr in range(n_rows):
        if not free[row0 + lr]:
            cols[lr] = {row0 + lr}
    indptr = np.zeros(n_rows + 1, dtype=np.int32)
    chunks = []
    for lr in range(n_rows):
        arr = np.asarray(sorted(cols[lr]), dtype=np.int32)
        chunks.append(arr)
        indptr[lr + 1] = indptr[lr] + arr.size
    indices = np.concatenate(chunks) if chunks else np.empty(0, np.int32)
    lookup = [{int(cc): int(indptr[lr]) + k for k, cc in enumerate(chunks[lr])} for lr in range(n_rows)]
    owned_free = free[row0:row1]
    cdiag = np.asarray([lookup[lr][row0 + lr] for lr in range(n_rows) if not owned_free[lr]], dtype=np.int32)
    scatter = np.full((ov_el.size, nld * nld), -1, dtype=np.int32)
    counts = np.zeros(n_rows, dtype=np.int64)
    for k, e in enumerate(ov_el):
        dofs = gdofs(elem[:, e])
        for a, r in enumerate(dofs):
            if not (row0 <= r < row1) or not owned_free[r - row0]:
                continue
            counts[r - row0] += 1
            for b, cc in enumerate(dofs):
                if free[cc]:
                    scatter[k, a * nld + b] = lookup[r - row0][int(cc)]
    rsp = np.zeros(n_rows + 1, dtype=np.int64)
    rsp[1:] = np.cumsum(counts)
    n_slots = int(rsp[-1])
    slot_elem = np.empty(n_slots, np.int32)
    slot_lrow = np.empty(n_slots, np.uint8)
    slot_pos = np.full((n_slots, nld), -1, np.int32)
    wp = rsp[:-1].copy()
    for k, e in enumerate(ov_el):
        dofs = gdofs(elem[:, e])
        for a, r in enumerate(dofs):
            if not (row0 <= r < row1) or not owned_free[r - row0]:
                continue
            sidx = wp[r - row0]
            wp[r - row0] += 1
            slot_elem[sidx] = k
            slot_lrow[sidx] = a
            slot_pos[sidx] = scatter[k, a * nld:(a + 1) * nld]
    owned_lids = lid[np.arange(n0, n1)]
    return {
        "overlap_elements": ov_el.astype(np.int64),
        "overlap_nodes": ov_nodes.astype(np.int64),
        "overlap_global_dofs": gdofs(ov_nodes).astype(np.int64),
        "overlap_element_dof_lids": dof_lids,
        "owned_local_overlap_dofs": gdofs(owned_lids).astype(np.int64),
        "owned_free_mask": owned_free.copy(),
        "indptr": indptr,
        "indices": indices,
        "constrained_diag_positions": cdiag,
        "scatter_map": scatter,
        "row_slot_ptr": rsp.astype(np.int32),
        "slot_elem": slot_elem,
        "slot_lrow": slot_lrow,
        "slot_pos": slot_pos,
    }


# --------------------------------------------------------------------------- learned branch proposal
# (no reference counterpart: the oracle for the product's MLP kernels, in float64)

MLP_SHAPES = (("W1", (32, 6)), ("b1", (32,)), ("W2", (32, 32)), ("b2", (32,)), ("W3", (5, 32)), ("b3", (5,)))


def mlp_unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, o = {}, 0
    for name, shape in MLP_SHAPES:
        k = int(np.prod(shape))
        out[name] = p[o:o + k].reshape(shape)
        o += k
    return out


def mlp_forward(p, X):
    w = mlp_unpack(p)
    X = np.asarray(X, dtype=np.float64)
    a1 = X @ w["W1"].T + w["b1"]
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ w["W2"].T + w["b2"]
    h2 = np.maximum(a2, 0.0)
    z = h2 @ w["W3"].T + w["b3"]
    return z, (X, a1, h1, a2, h2)


def mlp_loss_grad(p, X, y):
    """Summed softmax cross-entropy, its gradient (flat, kernel layout) and the argmax hits."""
    w = mlp_unpack(p)
    z, (X, a1, h1, a2, h2) = mlp_forward(p, X)
    y = np.asarray(y, dtype=np.int64)
    zmax = z.max(axis=1, keepdims=True)
    ez = np.exp(z - zmax)
    prob = ez / ez.sum(axis=1, keepdims=True)
    loss = float(np.sum(np.log(ez.sum(axis=1)) + zmax[:, 0] - z[np.arange(len(y)), y]))
    g3 = prob.copy()
    g3[np.arange(len(y)), y] -= 1.0
    g2 = (g3 @ w["W3"]) * (a2 > 0)
    g1 = (g2 @ w["W2"]) * (a1 > 0)
    grads = {"W3": g3.T @ h2, "b3": g3.sum(0), "W2": g2.T @ h1, "b2": g2.sum(0), "W1": g1.T @ X, "b1": g1.sum(0)}
    flat = np.concatenate([grads[name].ravel() for name, _ in MLP_SHAPES])
    hits = int(np.sum(np.argmax(z, axis=1) == y))
    return loss, flat, hits


def branch_features(E, c_bar, sin_phi, shear, lame):
    """Float64 restatement of the proposal network's input features (for checking the kernel)."""
    E = np.asarray(E, dtype=np.float64)
    t = E.copy()
    t[:, 3:] *= 0.5
    I1 = t[:, 0] + t[:, 1] + t[:, 2]
    d = t[:, :3] - I1[:, None] / 3.0
    J2 = 0.5 * np.sum(d * d, axis=1) + np.sum(t[:, 3:] ** 2, axis=1)
    J3 = (d[:, 0] * d[:, 1] * d[:, 2] + 2 * t[:, 3] * t[:, 4] * t[:, 5] - d[:, 0] * t[:, 4] ** 2
          - d[:, 1] * t[:, 5] ** 2 - d[:, 2] * t[:, 3] ** 2)
    k = 2.0 * shear / c_bar
    with np.errstate(divide="ignore", invalid="ignore"):
        lode = np.where(J2 > 0, 2.598076211 * J3 / (J2 * np.sqrt(J2)), 0.0)
    lode = np.clip(lode, -1.0, 1.0)
    lr = lame / shear
    slog = lambda x: np.sign(x) * np.log1p(np.abs(x))  # noqa: E731
    return np.stack([slog(k * np.sqrt(J2)), slog(k * I1), slog(lr * sin_phi * k * I1), lode, sin_phi,
                     lr / (lr + 2.0)], axis=1)


def have_reference_checkout() -> bool:
    """Whether the reference's kernel sources are where ``oracle/Makefile`` looks for them
    (``SSP_REFERENCE_ROOT``, or the recipe's default)."""
    r = subprocess.run(["make", "-s", "-C", str(HERE), "have-ref"], capture_output=True)
    return r.returncode == 0
