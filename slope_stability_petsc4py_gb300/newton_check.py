"""A minimal damped Newton solve on top of the GPU builder, for verifying tangent forms.

This is not the reference's Newton (``src/slope_stability/nonlinear/newton.py``, which stays on
PETSc): it is a small stand-in with SciPy direct solves, used to show what the mixed-precision
tangent changes in a Newton iteration.  For a fixed strength-reduction factor it solves
F_int(U) = F_gravity on the free dofs with the regularised tangent, a backtracking line search on
||residual||, and compares, at every iterate of the plain-FP64 solve, the Newton update computed
with the mixed tangent.
"""

from __future__ import annotations

import numpy as np
from scipy.sparse.linalg import spsolve

from .fem import quadrature, reference_values


def gravity_load(op, mesh, gamma: float) -> np.ndarray:
    """F_ext = int N^T (0, -gamma, 0) dV on all dofs (Fortran-flattened (dim, n_nodes))."""
    pat = op.owned_tangent_pattern
    _, wf = quadrature(mesh.dim, mesh.elem_type)
    phi = reference_values(mesh.dim, mesh.elem_type)  # (n_p, n_q)
    w = pat.overlap_assembly_weight.reshape(-1, pat.n_q)  # (n_el, n_q), |det J| * wf
    nodal = (w[:, None, :] * phi[None, :, :]).sum(axis=2)  # (n_el, n_p)
    F = np.zeros(mesh.dim * mesh.n_nodes)
    elem = mesh.elem[:, pat.overlap_elements]
    np.add.at(F, mesh.dim * elem.T.reshape(-1) + 1, -gamma * nodal.reshape(-1))
    return F


def _free_system(op, K_mat):
    pat = op.owned_tangent_pattern
    K = K_mat.to_scipy()
    free_rows = np.flatnonzero(pat.owned_free_mask)
    free_cols = np.flatnonzero(op.q_mask.reshape(-1, order="F"))
    return K[free_rows][:, free_cols].tocsc()


def newton_compare(op, mesh, *, lam: float, gamma: float = 20.0, r: float = 0.0, tol: float = 1e-9,
                   max_it: int = 30) -> dict:
    """Plain-FP64 Newton solve; at each iterate also the mixed form's force, tangent and update,
    compared with the FP64 ones (relative errors per Newton step)."""
    free = np.flatnonzero(op.q_mask.reshape(-1, order="F"))
    F_ext = gravity_load(op, mesh, gamma)[free]
    norm_ext = float(np.linalg.norm(F_ext))
    U = np.zeros(mesh.dim * mesh.n_nodes)

    def residual(Ufull):
        op.reduction(lam)
        F = op.build_F_reduced_free(Ufull.reshape(mesh.dim, -1, order="F"))
        return np.asarray(F) - F_ext

    history = []
    op.reduction(lam)
    for it in range(max_it):
        Ushape = U.reshape(mesh.dim, -1, order="F")
        op.tangent_form = "plain"
        F_free, K = op.build_F_K_regularized_all_free(lam, Ushape, r)
        R = np.asarray(F_free) - F_ext
        rel = float(np.linalg.norm(R)) / norm_ext
        if rel < tol:
            history.append({"it": it, "residual": rel})
            break
        Kp = _free_system(op, K)
        dU = spsolve(Kp, -R)
        # the mixed form (compensated strain and force, mixed tangent) at the same iterate
        op.tangent_form = "mixed"
        F_m, Km = op.build_F_K_regularized_all_free(lam, Ushape, r)
        f_err = float(np.linalg.norm(np.asarray(F_m) - np.asarray(F_free)) / max(np.linalg.norm(F_free), 1e-300))
        Kmx = _free_system(op, Km)
        dUm = spsolve(Kmx, -R)
        op.tangent_form = "plain"
        k_err = float(abs(Kmx - Kp).max() / abs(Kp).max())
        du_err = float(np.linalg.norm(dUm - dU) / max(np.linalg.norm(dU), 1e-300))
        alpha, r0 = 1.0, float(np.linalg.norm(R))
        while alpha > 1e-4:
            Utry = U.copy()
            Utry[free] += alpha * dU
            if float(np.linalg.norm(residual(Utry))) < r0:
                break
            alpha *= 0.5
        U[free] += alpha * dU
        history.append({"it": it, "residual": rel, "tangent_rel_err": k_err, "force_rel_err": f_err,
                        "update_rel_err": du_err, "alpha": alpha})
    return {"iterations": len(history) - 1, "converged": history[-1]["residual"] < tol, "history": history, "U": U}


def newton_iterations(op, mesh, *, form: str, lam: float, gamma: float = 20.0, r: float = 0.0, tol: float = 1e-9,
                      max_it: int = 30) -> tuple[int, float, np.ndarray]:
    """A full damped Newton solve with one tangent form; (iterations, final residual, U)."""
    free = np.flatnonzero(op.q_mask.reshape(-1, order="F"))
    F_ext = gravity_load(op, mesh, gamma)[free]
    norm_ext = float(np.linalg.norm(F_ext))
    U = np.zeros(mesh.dim * mesh.n_nodes)
    op.tangent_form = form
    rel = np.inf
    for it in range(max_it):
        F_free, K = op.build_F_K_regularized_all_free(lam, U.reshape(mesh.dim, -1, order="F"), r)
        R = np.asarray(F_free) - F_ext
        rel = float(np.linalg.norm(R)) / norm_ext
        if rel < tol:
            op.tangent_form = "plain"
            return it, rel, U
        dU = spsolve(_free_system(op, K), -R)
        alpha, r0 = 1.0, float(np.linalg.norm(R))
        while alpha > 1e-4:
            Utry = U.copy()
            Utry[free] += alpha * dU
            op.reduction(lam)
            Rt = np.asarray(op.build_F_reduced_free(Utry.reshape(mesh.dim, -1, order="F"))) - F_ext
            if float(np.linalg.norm(Rt)) < r0:
                break
            alpha *= 0.5
        U[free] += alpha * dU
    op.tangent_form = "plain"
    return max_it, rel, U
