"""Quadrature rules and reference-element basis gradients of the supported simplex elements.

The rules and node orderings must be the reference's, value for value, because every
tangent and force entry is a sum over these points and weights:

* quadrature: ``src/slope_stability/fem/quadrature.py:7-126`` (the tables below restate its
  constants, including the truncated decimals and the negative centroid weight of the
  11-point tetrahedron rule);
* basis gradients: ``src/slope_stability/fem/basis.py:9-206`` and the generic barycentric
  construction of ``src/slope_stability/core/simplex_lagrange.py:95-161`` for P4.

Only small host tables live here; the per-point geometry (``dphi``, weights) is computed on
the GPU by the ``ssp_geometry_*`` kernels.
"""

from __future__ import annotations

from functools import lru_cache

import numpy as np

from .synthetic import tet_node_tuples, tri_node_tuples

N_NODES = {(2, "P1"): 3, (2, "P2"): 6, (2, "P4"): 15, (3, "P1"): 4, (3, "P2"): 10, (3, "P4"): 35}


def quadrature(dim: int, elem_type: str) -> tuple[np.ndarray, np.ndarray]:
    """Reference-element points ``xi`` (dim, n_q) and weights ``wf`` (n_q,)."""
    et = elem_type.upper()
    if dim == 2:
        if et == "P1":
            return np.array([[1 / 3], [1 / 3]]), np.array([0.5])
        if et == "P2":
            a, b, c, d = 0.1012865073235, 0.7974269853531, 0.4701420641051, 0.0597158717898
            xi = np.array([[a, b, a, c, c, d, 1 / 3], [a, a, b, d, c, c, 1 / 3]])
            wf = np.array([0.1259391805448] * 3 + [0.1323941527885] * 3 + [0.225]) / 2
            return xi, wf
        if et == "P4":
            # 12-point rule: two 3-point orbits and one 6-point orbit (quadrature.py:28-51)
            a1, b1 = 0.063089014491502, 0.873821971016996
            a2, b2 = 0.249286745170910, 0.501426509658179
            p, q, r = 0.310352451033785, 0.053145049844816, 0.636502499121399
            xi = np.array(
                [
                    [a1, a1, b1, a2, a2, b2, p, p, q, q, r, r],
                    [a1, b1, a1, a2, b2, a2, q, r, p, r, p, q],
                ]
            )
            wf = np.array([0.050844906370207] * 3 + [0.116786275726379] * 3 + [0.082851075618374] * 6) / 2
            return xi, wf
    if dim == 3:
        if et == "P1":
            return np.array([[0.25], [0.25], [0.25]]), np.array([1 / 6])
        if et == "P2":
            s, l, u, v = 0.0714285714285714, 0.785714285714286, 0.399403576166799, 0.100596423833201
            xi = np.array(
                [
                    [1 / 4, s, l, s, s, u, v, v, u, u, v],
                    [1 / 4, s, s, l, s, v, u, v, u, v, u],
                    [1 / 4, s, s, s, l, v, v, u, v, u, u],
                ]
            )
            wf = np.array([-0.013155555555555] + [0.007622222222222] * 4 + [0.024888888888888] * 6)
            return xi, wf
        if et == "P4":
            a, b = 0.3561913862225449, 0.2146028712591517
            c, d = 0.8779781243961660, 0.0406739585346113
            e, f = 0.0329863295731731, 0.3223378901422757
            g, h, k = 0.2696723314583159, 0.0636610018750175, 0.6030056647916491
            xi = np.array(
                [
                    [a, b, b, b, c, d, d, d, e, f, f, f, g, h, h, k, h, h, h, g, k, h, g, k],
                    [b, b, b, a, d, d, d, c, f, f, f, e, h, g, h, h, k, h, g, k, h, k, h, g],
                    [b, b, a, b, d, d, c, d, f, f, e, f, h, h, g, h, h, k, k, h, g, g, k, h],
                ]
            )
            wf = np.array(
                [0.0399227502581679] * 4 + [0.0100772110553207] * 4 + [0.0553571815436544] * 4
                + [0.0482142857142857] * 12
            ) / 6.0
            return xi, wf
    raise ValueError(f"unsupported element {dim}D {elem_type!r}")


def _lagrange_factor(order: int, degree: int, lam: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """prod_{m<degree} (order*lam - m)/(m+1) and its derivative in lam."""
    if degree == 0:
        return np.ones_like(lam), np.zeros_like(lam)
    fac = [(order * lam - m) / (m + 1) for m in range(degree)]
    val = np.ones_like(lam)
    for f in fac:
        val = val * f
    der = np.zeros_like(lam)
    for m in range(degree):
        term = np.full_like(lam, order / (m + 1))
        for n, f in enumerate(fac):
            if n != m:
                term = term * f
        der = der + term
    return val, der


def _tet_lagrange_grads(order: int, xi: np.ndarray) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    bary = (1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2])
    tuples = tet_node_tuples(order)
    n_q = xi.shape[1]
    out = [np.empty((len(tuples), n_q)) for _ in range(3)]
    for idx, counts in enumerate(tuples):
        vals, ders = zip(*(_lagrange_factor(order, c, l) for l, c in zip(bary, counts)))
        dl = []
        for dv in range(4):
            term = ders[dv]
            for fv in range(4):
                if fv != dv:
                    term = term * vals[fv]
            dl.append(term)
        for ax in range(3):
            out[ax][idx] = dl[ax + 1] - dl[0]
    return out[0], out[1], out[2]


def _tri_lagrange(order: int, xi: np.ndarray) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Values and (xi1, xi2) derivatives of the order-p triangle basis from barycentric products."""
    bary = (1.0 - xi[0] - xi[1], xi[0], xi[1])
    tuples = tri_node_tuples(order)
    n_q = xi.shape[1]
    val = np.empty((len(tuples), n_q))
    d = [np.empty((len(tuples), n_q)) for _ in range(2)]
    for idx, counts in enumerate(tuples):
        vals, ders = zip(*(_lagrange_factor(order, c, lv) for lv, c in zip(bary, counts)))
        val[idx] = vals[0] * vals[1] * vals[2]
        dl = [ders[0] * vals[1] * vals[2], vals[0] * ders[1] * vals[2], vals[0] * vals[1] * ders[2]]
        for ax in range(2):
            d[ax][idx] = dl[ax + 1] - dl[0]
    return val, d[0], d[1]


def _reference_p4_tri_dxi2_quarter_nodes(xi: np.ndarray) -> np.ndarray:
    """The reference's tabulated d/dxi2 of the 2D P4 quarter-point nodes 8-11.

    ``src/slope_stability/fem/basis.py:100-123`` lists, for nodes 8-11, expressions that are not
    the xi2-derivatives of its own basis functions (lines 68-71): for example node 10's entry is the
    xi1-derivative of node 10's function, and the four rows do not sum with the others to zero.
    The strain, force and tangent of a 2D P4 element are sums over these tabulated values, so they
    are reproduced here value for value; the table's other 26 rows are the exact derivatives.
    Returns shape (4, n_q).
    """
    x1, x2 = xi
    x0 = 1.0 - x1 - x2
    k = 8.0 / 3.0
    return np.array([
        k * x1 * ((4 * x1 - 1) * (4 * x1 - 2) + 4 * x2 * (4 * x1 - 1)),
        k * x1 * ((4 * x1 - 1) * (4 * x2 - 1) + 4 * x2 * (4 * x2 - 1)),
        -k * x2 * (4 * x2 - 1) * (4 * x2 - 2),
        k * x2 * ((4 * x2 - 1) * (4 * x2 - 2) + 4 * x0 * (4 * x2 - 2) + 4 * x0 * (4 * x2 - 1)),
    ])


@lru_cache(maxsize=None)
def reference_values(dim: int, elem_type: str) -> np.ndarray:
    """Basis values at the quadrature points, shape (n_p, n_q) (basis.py:15-33, 134-157)."""
    xi, _ = quadrature(dim, elem_type)
    et = elem_type.upper()
    if dim == 3 and et in ("P1", "P2"):
        l1, l2, l3 = xi
        lam = [1.0 - l1 - l2 - l3, l1, l2, l3]
        if et == "P1":
            return np.array(lam)
        verts = [lv * (2.0 * lv - 1.0) for lv in lam]
        edges = [4.0 * lam[i] * lam[j] for i, j in ((0, 1), (1, 2), (0, 2), (1, 3), (2, 3), (0, 3))]
        return np.array(verts + edges)
    if dim == 2 and et in ("P1", "P2"):
        l1, l2 = xi
        lam = [1.0 - l1 - l2, l1, l2]
        if et == "P1":
            return np.array(lam)
        verts = [lv * (2.0 * lv - 1.0) for lv in lam]
        return np.array(verts + [4.0 * lam[1] * lam[2], 4.0 * lam[0] * lam[2], 4.0 * lam[0] * lam[1]])
    if dim == 2 and et == "P4":
        return _tri_lagrange(4, xi)[0]
    if dim == 3 and et == "P4":
        bary = (1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2])
        out = np.empty((N_NODES[(3, "P4")], xi.shape[1]))
        for idx, counts in enumerate(tet_node_tuples(4)):
            val = np.ones(xi.shape[1])
            for lv, c in zip(bary, counts):
                val = val * _lagrange_factor(4, c, lv)[0]
            out[idx] = val
        return out
    raise ValueError(f"no basis values for {dim}D {elem_type}")


@lru_cache(maxsize=None)
def reference_gradients(dim: int, elem_type: str) -> np.ndarray:
    """Basis gradients on the reference element at the quadrature points, shape (dim, n_p, n_q)."""
    xi, _ = quadrature(dim, elem_type)
    et = elem_type.upper()
    n_q = xi.shape[1]
    z = np.zeros(n_q)
    if dim == 2:
        x1, x2 = xi
        x0 = 1.0 - x1 - x2
        if et == "P1":
            g1 = np.repeat(np.array([-1.0, 1.0, 0.0])[:, None], n_q, axis=1)
            g2 = np.repeat(np.array([-1.0, 0.0, 1.0])[:, None], n_q, axis=1)
        elif et == "P2":
            g1 = np.array([1 - 4 * x0, 4 * x1 - 1, z, 4 * x2, -4 * x2, 4 * (x0 - x1)])
            g2 = np.array([1 - 4 * x0, z, 4 * x2 - 1, 4 * x1, 4 * (x0 - x2), -4 * x1])
        elif et == "P4":
            _, g1, g2 = _tri_lagrange(4, xi)
            g2[8:12] = _reference_p4_tri_dxi2_quarter_nodes(xi)
        else:
            raise ValueError(et)
        return np.stack((g1, g2))
    x1, x2, x3 = xi
    x0 = 1.0 - x1 - x2 - x3
    if et == "P1":
        base = np.array([[-1.0, 1.0, 0.0, 0.0], [-1.0, 0.0, 1.0, 0.0], [-1.0, 0.0, 0.0, 1.0]])
        return np.repeat(base[:, :, None], n_q, axis=2)
    if et == "P2":
        g1 = np.array([1 - 4 * x0, 4 * x1 - 1, z, z, 4 * (x0 - x1), 4 * x2, -4 * x2, 4 * x3, z, -4 * x3])
        g2 = np.array([1 - 4 * x0, z, 4 * x2 - 1, z, -4 * x1, 4 * x1, 4 * (x0 - x2), z, 4 * x3, -4 * x3])
        g3 = np.array([1 - 4 * x0, z, z, 4 * x3 - 1, -4 * x1, z, -4 * x2, 4 * x1, 4 * x2, 4 * (x0 - x3)])
        return np.stack((g1, g2, g3))
    if et == "P4":
        return np.stack(_tet_lagrange_grads(4, xi))
    raise ValueError(et)
