"""The moment form of the P2 plastic correction, as algebra (no GPU).

The kernels `correction_p2_moment_kernel` (FP64) and `correction_p2_moment_f32_kernel` (mixed form,
`csrc/assembly.cu`) regroup the reference's contraction K_e = sum_q B_q^T dD_q B_q
(`src/slope_stability/cython/assemble_tangent_values_3d.c:135-214`) for straight-sided P2
tetrahedra: with lambda_4 = 1 as a fifth barycentric coordinate every node's gradient has two
terms c lambda_m grad lambda_k, so

    K[(a,c),(b,d)] = sum_{x,y} c_ax c_by R_(m_ax m_by)[(k_ax,c),(k_by,d)],   R_mn = beta^T M_mn beta,
    M_mn = sum_q lambda_qm lambda_qn dD_q,   R_m4 = sum_n R_mn,   R_44 = sum_m R_m4.

This restates that construction in numpy (node order, term table and strain layout as the kernels
use them) and checks it against the direct contraction with the reference element's own P2
gradients (`fem.reference_gradients`, the reference's basis.py tables) mapped by J^-T; models the
mixed form's FP32 regrouping against the same contraction; and checks the Taylor polynomials the
return mapping uses for the sine and cosine of the Lode angle.
"""

from __future__ import annotations

import numpy as np
import pytest

EDGES = ((0, 1), (1, 2), (0, 2), (1, 3), (2, 3), (0, 3))  # mid-edge nodes 4..9


def node_terms(a):
    """(m, coefficient, k) of node a's gradient, m = 4 the constant coordinate."""
    if a < 4:
        return ((a, 4.0, a), (4, -1.0, a))
    i, j = EDGES[a - 4]
    return ((i, 4.0, j), (j, 4.0, i))


def strain_rows(c):
    """Strain rows of the gradient components x, y, z of displacement component c (xx, yy, zz, xy, yz, xz)."""
    return ((0, 3, 5), (3, 1, 4), (5, 4, 2))[c]


def b_matrix(grads):
    """6 x 30 strain-displacement matrix of one point from the ten physical gradients (10, 3)."""
    B = np.zeros((6, 30))
    for a in range(10):
        for c in range(3):
            for comp, row in enumerate(strain_rows(c)):
                B[row, 3 * a + c] = grads[a, comp]
    return B


def beta(v):
    """12 x 6: row (k, c) is the strain of grad lambda_k (x) e_c."""
    out = np.zeros((12, 6))
    for k in range(4):
        for c in range(3):
            for comp, row in enumerate(strain_rows(c)):
                out[3 * k + c, row] = v[k, comp]
    return out


def moment_form(jinv, lam, dD):
    """The kernels' regrouping: lam (n, 4) barycentric coordinates, dD (n, 6, 6) weighted."""
    v = np.vstack([-jinv.sum(axis=0), jinv])  # grad lambda_0..3 (rows of J^-1 for 1..3)
    lam5 = np.hstack([lam, np.ones((lam.shape[0], 1))])
    bt = beta(v)
    R = {}
    for m in range(4):
        for n in range(m, 4):
            M = np.einsum("q,qij->ij", lam5[:, m] * lam5[:, n], dD)
            R[(m, n)] = bt @ M @ bt.T
    for m in range(4):  # the coordinates sum to one
        R[(m, 4)] = sum(R[(min(m, n), max(m, n))] for n in range(4))
    R[(4, 4)] = sum(R[(m, 4)] for m in range(4))
    K = np.zeros((30, 30))
    for a in range(10):
        for b in range(10):
            for ma, ca, ka in node_terms(a):
                for mb, cb, kb in node_terms(b):
                    blk = R[(min(ma, mb), max(ma, mb))]
                    K[3 * a:3 * a + 3, 3 * b:3 * b + 3] += ca * cb * blk[3 * ka:3 * ka + 3, 3 * kb:3 * kb + 3]
    return K


@pytest.mark.parametrize("seed,n_plastic", [(0, 11), (1, 5), (2, 1)])
def test_moment_form_equals_the_point_contraction(seed, n_plastic):
    from slope_stability_petsc4py_gb300 import fem

    rng = np.random.default_rng(seed)
    ghat = fem.reference_gradients(3, "P2")  # (3, 10, 11): d phi_a / d xi at the points
    xi, _ = fem.quadrature(3, "P2")
    J = np.eye(3) + 0.4 * rng.standard_normal((3, 3))  # x = x0 + J xi, a straight-sided tetrahedron
    jinv = np.linalg.inv(J)
    pts = np.sort(rng.choice(xi.shape[1], size=n_plastic, replace=False))
    A = rng.standard_normal((n_plastic, 6, 6))
    dD = -(A @ A.transpose(0, 2, 1)) * rng.uniform(0.5, 2.0, (n_plastic, 1, 1))  # symmetric, weighted
    K_direct = np.zeros((30, 30))
    for k, q in enumerate(pts):
        grads = ghat[:, :, q].T @ jinv  # (10, 3): J^-T ghat_a
        B = b_matrix(grads)
        K_direct += B.T @ dD[k] @ B
    lam = np.column_stack([1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]])[pts]
    K_moment = moment_form(jinv, lam, dD)
    scale = np.abs(K_direct).max()
    assert np.abs(K_moment - K_direct).max() <= 1e-13 * scale
    assert np.allclose(K_moment, K_moment.T, rtol=0, atol=1e-14 * scale)


def test_two_term_gradients_match_the_reference_table():
    """Every P2 gradient is sum over its two terms of c lambda_m grad lambda_k (lambda_4 = 1)."""
    from slope_stability_petsc4py_gb300 import fem

    ghat = fem.reference_gradients(3, "P2")
    xi, _ = fem.quadrature(3, "P2")
    lam5 = np.column_stack([1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2], np.ones(xi.shape[1])])
    dlam = np.vstack([-np.ones(3), np.eye(3)])  # reference gradients of lambda_0..3
    for a in range(10):
        g = sum(c * lam5[:, m][:, None] * dlam[k][None, :] for m, c, k in node_terms(a))
        assert np.allclose(g, ghat[:, a, :].T, rtol=0, atol=1e-14)


def test_moment_form_in_fp32_stays_within_the_mixed_tolerance():
    """The mixed form's kernel runs the regrouping in FP32 after FP64 DS - D_el: modelled here by
    rounding the inputs to float32 and carrying out every stage in float32, the element
    correction stays within a few 1e-7 of its own scale (the mixed form's bound on the tangent,
    which also holds the elastic part, is 1e-6)."""
    from slope_stability_petsc4py_gb300 import fem

    rng = np.random.default_rng(5)
    ghat = fem.reference_gradients(3, "P2")
    xi, _ = fem.quadrature(3, "P2")
    lam_all = np.column_stack([1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]])
    worst = 0.0
    for trial in range(4):
        J = np.eye(3) + 0.4 * rng.standard_normal((3, 3))
        jinv = np.linalg.inv(J)
        A = rng.standard_normal((11, 6, 6))
        dD = -(A @ A.transpose(0, 2, 1)) * 1e7
        K_direct = sum(b_matrix(ghat[:, :, q].T @ jinv).T @ dD[q] @ b_matrix(ghat[:, :, q].T @ jinv)
                       for q in range(11))
        f32 = np.float32
        v = np.vstack([-jinv.sum(axis=0), jinv]).astype(f32)
        lam5 = np.hstack([lam_all, np.ones((11, 1))]).astype(f32)
        bt = beta(v.astype(np.float64)).astype(f32)
        R = {}
        for m in range(4):
            for n in range(m, 4):
                M = np.einsum("q,qij->ij", (lam5[:, m] * lam5[:, n]).astype(f32), dD.astype(f32)).astype(f32)
                R[(m, n)] = (bt @ M @ bt.T).astype(f32)
        for m in range(4):
            R[(m, 4)] = sum(R[(min(m, n), max(m, n))] for n in range(4)).astype(f32)
        R[(4, 4)] = sum(R[(m, 4)] for m in range(4)).astype(f32)
        K = np.zeros((30, 30), f32)
        for a in range(10):
            for b in range(10):
                for ma, ca, ka in node_terms(a):
                    for mb, cb, kb in node_terms(b):
                        blk = R[(min(ma, mb), max(ma, mb))]
                        K[3 * a:3 * a + 3, 3 * b:3 * b + 3] += f32(ca * cb) * blk[3 * ka:3 * ka + 3, 3 * kb:3 * kb + 3]
        worst = max(worst, np.abs(K.astype(np.float64) - K_direct).max() / np.abs(K_direct).max())
    assert 1e-9 < worst < 1e-6, worst


def test_lode_angle_sine_and_cosine_polynomials():
    """The Taylor polynomials the return mapping evaluates for sin and cos of the Lode angle
    (`sincos_lode`, csrc/constitutive.cu: through theta^17 and theta^18, Horner in theta^2) agree
    with the library functions to within one ulp on [0, pi/3]."""
    from math import factorial

    theta = np.linspace(0.0, np.pi / 3.0, 400_001)
    z = theta * theta
    ps = np.zeros_like(z)
    for k in range(8, 0, -1):  # 1/17! .. -1/3!
        ps = ps * z + (-1.0) ** k / factorial(2 * k + 1)
    s = theta * z * ps + theta
    pc = np.zeros_like(z)
    for k in range(9, 0, -1):  # -1/18! .. -1/2!
        pc = pc * z + (-1.0) ** k / factorial(2 * k)
    c = z * pc + 1.0
    ulp_s = np.abs(s - np.sin(theta))[1:] / np.spacing(np.sin(theta[1:]))
    ulp_c = np.abs(c - np.cos(theta)) / np.spacing(np.cos(theta))
    assert ulp_s.max() <= 1.0 and ulp_c.max() <= 1.0
