"""The reference's Newton iteration on the host cores, through the oracle.

TEST INFRASTRUCTURE ONLY: the oracle the benchmark and the tests compare the GPU runs with, and
the CPU baseline of the benchmark.  The product package never imports it.

One step is what the reference's ``ConstitutiveOperator.build_F_K_regularized_all_free`` does per
Newton iteration on its owned rows (src/slope_stability/constitutive/problem.py:2114-2146):
reduction (constitutive/reduction.py:14-78), overlap strain (cython/assemble_tangent_values_3d.c:
216-273; 2D fem/assembly.py:96-123), return mapping (cython/constitutive_3D_kernel.h:68-351; 2D
constitutive/problem.py:143-475), owned force (assemble_tangent_values_3d.c:275-327; 2D
fem/distributed_tangent.py:845-852), tangent rows (assemble_tangent_values_3d.c:111-214; 2D the
scatter form, distributed_tangent.py:1437-1484), constrained diagonals (:1606-1607) and the
regularised blend (constitutive/problem.py:1595-1644).  The pattern, geometry and elastic values
are built once by the oracle's own restatements.
"""

from __future__ import annotations

import time

import numpy as np

from . import oracle_py as o


class OracleNewtonStep:
    """The reference's Newton iteration on the host cores, through the oracle's restatement of its
    kernels (oracle/oracle.c, oracle/oracle_py.py): its own pattern, geometry and elastic values for
    an owned node block, then per step the reduction, strain, return mapping, owned force, rows
    tangent, constrained diagonals and the regularised blend.  Loads only oracle/ libraries."""

    def __init__(self, mesh, specs, owned=None):
        from slope_stability_petsc4py_gb300 import fem
        from slope_stability_petsc4py_gb300.materials import heterogenous_materials

        o.build()
        self.o = o
        n0, n1 = owned if owned is not None else (0, mesh.n_nodes)
        self.owned = (int(n0), int(n1))
        t0 = time.perf_counter()
        p = o.owned_pattern_c(mesh.elem, mesh.q_mask, self.owned)
        self.pattern_s = time.perf_counter() - t0
        self.p = p
        self.dim, et = mesh.dim, mesh.elem_type
        _xi, wf = fem.quadrature(self.dim, et)
        self.n_q = len(wf)
        self.n_p = mesh.elem.shape[0]
        ov = p["overlap_elements"]
        elem_ov = mesh.elem[:, ov]
        t1 = time.perf_counter()
        dhat = fem.reference_gradients(self.dim, et)
        if self.dim == 3:
            self.d, self.w = o.geometry_3d_c(mesh.coord, elem_ov, dhat, wf)
        else:
            self.d, self.w = o.geometry(mesh.coord, elem_ov, 2, dhat, wf)
            self.scatter = o.scatter_from_slots(p, 2 * self.n_p)
        self.geometry_s = time.perf_counter() - t1
        self.n_int = int(ov.size) * self.n_q
        self.nnz = int(p["indices"].size)
        self.mat = dict(zip(("c0", "phi", "psi", "shear", "bulk", "lame"),
                            heterogenous_materials(np.asarray(mesh.material_id)[ov], np.ones(self.n_int, bool),
                                                   self.n_q, specs)[:6]))
        self.free = p["owned_free_mask"]
        t2 = time.perf_counter()
        self.elastic = self._tangent(o.elastic_ds(self.dim, self.mat["shear"], self.mat["bulk"], self.mat["lame"]))
        self.elastic[p["constrained_diag_positions"]] = 1.0
        self.elastic_s = time.perf_counter() - t2
        self.n_nodes = mesh.n_nodes

    def _tangent(self, DS, library=None):
        o, p, d = self.o, self.p, self.d
        if self.dim == 3:
            return o.tangent_rows_3d(d[0], d[1], d[2], DS, self.w, p["row_slot_ptr"], p["slot_elem"], p["slot_lrow"],
                                     p["slot_pos"], self.n_q, self.nnz, library=library)
        return o.tangent_scatter(2, d[0], d[1], None, DS, self.w, self.scatter, self.n_q, self.nnz)

    def constitutive(self, E, lam, davis="B", library=None):
        """S, DS (AoS) of the reference's return mapping on given strains E (n_int, n_s) at lam."""
        o, m = self.o, self.mat
        cb, sp = o.reduction(m["c0"], m["phi"], m["psi"], lam, davis)
        if self.dim == 3:
            return o.constitutive_3d(E, cb, sp, m["shear"], m["bulk"], m["lame"], library=library)
        S4, DS9 = o.constitutive_2d(np.asarray(E).T, cb, sp, m["shear"], m["bulk"], m["lame"])
        return np.ascontiguousarray(S4.T), np.ascontiguousarray(DS9.T)

    def step(self, U, lam, r, davis="B", library=None):
        """One Newton iteration at U (dim, n_nodes): dict of E, S, DS (AoS), F (owned rows) and K.
        library: the C restatement to run the 3D kernels with (default: oracle/_build/liboracle.so;
        oracle_py.nofma_lib() is the same code without fused multiply-adds)."""
        o, p, d, m = self.o, self.p, self.d, self.mat
        cb, sp = o.reduction(m["c0"], m["phi"], m["psi"], lam, davis)
        u_ov = np.ascontiguousarray(U.reshape(-1, order="F")[p["overlap_global_dofs"]])
        if self.dim == 3:
            E = o.strain_3d(d[0], d[1], d[2], u_ov, p["overlap_element_dof_lids"], self.n_q, library=library)
            S, DS = o.constitutive_3d(E, cb, sp, m["shear"], m["bulk"], m["lame"], library=library)
            F = o.force_rows_3d(d[0], d[1], d[2], S, self.w, p["row_slot_ptr"], p["slot_elem"], p["slot_lrow"],
                                self.n_q, library=library)
        else:
            E = o.strain_2d(d[0], d[1], u_ov, p["overlap_element_dof_lids"], self.n_q)
            S4, DS9 = o.constitutive_2d(E.T, cb, sp, m["shear"], m["bulk"], m["lame"])
            S, DS = np.ascontiguousarray(S4.T), np.ascontiguousarray(DS9.T)
            f_ov = o.overlap_force_2d(d[0], d[1], np.ascontiguousarray(S[:, :3]), self.w,
                                      p["overlap_element_dof_lids"], self.n_q, p["overlap_global_dofs"].size)
            F = f_ov[p["owned_local_overlap_dofs"]]
        F[~self.free] = 0.0
        K = self._tangent(DS, library)
        K[p["constrained_diag_positions"]] = 1.0
        K *= 1.0 - r
        K += r * self.elastic
        return {"E": E, "S": S, "DS": DS, "F": F, "K": K}

    def time_steps(self, states, steps, warmup, lam, r, budget_s=None):
        """Wall-clock seconds of each of `steps` steps cycling through `states` after `warmup`."""
        for k in range(warmup):
            self.step(states[k % len(states)], lam, r)
        times = []
        t_start = time.perf_counter()
        for k in range(steps):
            t0 = time.perf_counter()
            self.step(states[k % len(states)], lam, r)
            times.append(time.perf_counter() - t0)
            if budget_s is not None and time.perf_counter() - t_start > budget_s:
                break
        return times
