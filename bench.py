"""Benchmark of the Newton hot path: quadrature points per second of one builder pass.

One step = one Newton iteration of the reference's owned-row builder on a fixed synthetic slope:
strength reduction -> strain B u -> Mohr-Coulomb return mapping (S and DS) -> owned internal
force B^T (w S) -> tangent CSR values sum B^T (w DS) B -> constrained diagonals and the
regularised blend (1-r) K + r K_elast.  ``value`` is measured with inputs resident in HBM;
``e2e`` goes through the public ``ConstitutiveOperator`` API with pinned host inputs and host
outputs (U uploaded, F_free and every CSR value copied back each step, as the PETSc hand-off
needs).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config 3d_p2_homo] [--impl reference]

``--impl reference`` times the reference algorithm on the host cores instead (the oracle's C
restatement of the reference kernels, all threads), on the same workload.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "quad-pts/s constitutive+tangent; FP64 plain vs mixed+learned at ≤1e-6 err"
LAMBDA, R_REG = 1.1, 0.1

# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the step kernels, from one
# ncu capture of the full-size workload on a GB300 (one pass per launch, the second Newton step of
# `bench.py --steps 3 --warmup 3`); keyed by workload and C-ABI entry point.
NCU_TRAFFIC = {
    "3d_p2_homo": {
        "ssp_tangent_plastic_correction": 286.20e6 + 63.73e6,
        "ssp_tangent_plastic_correction_mixed": 298.00e6 + 72.01e6,
        "ssp_assemble_overlap_strain_3d_affine_mixed": 22.82e6 + 0.04e6,
        "ssp_assemble_force_element_affine_mixed": 84.88e6 + 1.49e6,
        "ssp_assemble_overlap_strain_3d_mixed": 281.74e6 + 35.76e6,
        "ssp_assemble_overlap_strain_3d": 284.63e6 + 36.25e6,
        "ssp_assemble_force_element": 343.75e6 + 2.57e6,
        "ssp_assemble_overlap_strain_3d_p2_affine": 22.85e6 + 1.40e6,
        "ssp_assemble_force_element_p2_affine": 84.94e6 + 0.30e6,
        "ssp_assemble_overlap_strain_3d_p2_affine_mixed": 23.48e6 + 2.04e6,
        "ssp_assemble_force_element_p2_affine_mixed": 84.95e6 + 0.02e6,
        "ssp_constitutive_3d_sds_binned": (90.67 + 304.28 + 22.35 + 1.76 + 34.33 + 1.12) * 1e6,
    },
    "3d_p4_hetero": {
        "ssp_tangent_plastic_correction_mixed": 1121.05e6 + 524.74e6,
        "ssp_assemble_overlap_strain_3d": 1784.86e6 + 50.96e6,
        "ssp_assemble_force_element": 1102.46e6 + 11.75e6,
        "ssp_constitutive_3d_sds_binned": (121.29 + 245.19 + 39.91 + 39.69 + 41.21 + 1.96) * 1e6,
    },
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="3d_p2_homo")
    ap.add_argument("--mesh", default=None, help="a gmsh .msh tet4 file as the workload (overrides --config)")
    ap.add_argument("--mesh-elem", default="P2", choices=["P1", "P2", "P4"], help="element order for --mesh")
    ap.add_argument("--form", default="plain", choices=["plain", "mixed"],
                    help="plain: FP64 tangent (the drop-in); mixed: FP32 plastic-point products")
    ap.add_argument("--return-mapping", default="binned", choices=["binned", "unsorted", "learned"],
                    help="binned: two-pass exact binning; unsorted: one divergent pass; learned: bins proposed "
                         "by the branch network (trained on the GPU before the timed region)")
    ap.add_argument("--no-forms", action="store_true", help="skip timing the mixed / learned / unsorted forms")
    ap.add_argument("--bddc", action="store_true", help="also time the BDDC subdomain tangent of half the mesh")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-clocks", action="store_true")
    return ap.parse_args()


# ----------------------------------------------------------------------------- workload


def workload(name: str):
    from slope_stability_petsc4py_gb300 import synthetic

    cfg = synthetic.CONFIGS[name]
    mesh = synthetic.build_config_mesh(name)
    mats = synthetic.MaterialSet.layered(4, seed=0) if cfg["n_layers"] > 1 else synthetic.MaterialSet.homogeneous()
    specs = [dict(c0=float(mats.c0[i]), phi=float(mats.phi[i]), psi=float(mats.psi[i]), young=float(mats.young[i]),
                  poisson=float(mats.poisson[i]), gamma_sat=float(mats.gamma[i]), gamma_unsat=float(mats.gamma[i]))
             for i in range(mats.c0.size)]
    U = synthetic.displacement_field(mesh, mats, amplitude=cfg["amplitude"], seed=3)
    return mesh, mats, specs, U


def describe(name, mesh, n_int, nnz):
    return (f"{name}: {mesh.n_elem:,} {mesh.dim}D {mesh.elem_type} elements, {n_int:,} quadrature points, "
            f"{mesh.n_nodes * mesh.dim:,} dofs, {nnz:,} CSR nnz")


# ----------------------------------------------------------------------------- clocks


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.idx = device_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------------------------- CPU reference path


class OracleRunner:
    """The reference algorithm (oracle restatement of its C kernels) on the host cores."""

    def __init__(self, mesh, specs, U, dphi=None, weight=None):
        from oracle import oracle_py as oracle
        from slope_stability_petsc4py_gb300 import fem
        from slope_stability_petsc4py_gb300.distributed_tangent import _PatternBuild
        from slope_stability_petsc4py_gb300.materials import heterogenous_materials

        self.o = oracle
        oracle.build()
        pb = _PatternBuild(mesh.elem, mesh.q_mask, (0, mesh.n_nodes))
        keys = ("overlap_nodes", "overlap_element_dof_lids", "row_slot_ptr", "slot_elem", "slot_lrow", "slot_pos",
                "constrained_diag_positions", "owned_free_mask", "overlap_elements")
        self.p = {k: pb.get(k) for k in keys}
        self.nnz = pb.sizes["nnz"]
        pb.close()
        xi, wf = fem.quadrature(mesh.dim, mesh.elem_type)
        self.n_q = xi.shape[1]
        if dphi is None:
            dphi, weight = oracle.geometry(mesh.coord, mesh.elem[:, self.p["overlap_elements"]], mesh.dim,
                                           fem.reference_gradients(mesh.dim, mesh.elem_type), wf)
        self.d, self.w = dphi, weight
        nodes = self.p["overlap_nodes"]
        dim = mesh.dim
        gd = dim * np.repeat(nodes, dim) + np.tile(np.arange(dim), nodes.size)
        self.u_ov = np.ascontiguousarray(U.reshape(-1, order="F")[gd])
        n_int = mesh.n_elem * self.n_q
        self.mat = dict(zip(("c0", "phi", "psi", "shear", "bulk", "lame"),
                            heterogenous_materials(mesh.material_id, np.ones(n_int, bool), self.n_q, specs)[:6]))
        self.n_int = n_int
        self.dim = dim
        self.elastic = None

    def step(self):
        o, p, d = self.o, self.p, self.d
        cb, sp = o.reduction(self.mat["c0"], self.mat["phi"], self.mat["psi"], LAMBDA, "B")
        E = o.strain_3d(d[0], d[1], d[2], self.u_ov, p["overlap_element_dof_lids"], self.n_q)
        S, DS = o.constitutive_3d(E, cb, sp, self.mat["shear"], self.mat["bulk"], self.mat["lame"])
        F = o.force_rows_3d(d[0], d[1], d[2], S, self.w, p["row_slot_ptr"], p["slot_elem"], p["slot_lrow"], self.n_q)
        F[~p["owned_free_mask"].astype(bool)] = 0.0
        K = o.tangent_rows_3d(d[0], d[1], d[2], DS, self.w, p["row_slot_ptr"], p["slot_elem"], p["slot_lrow"],
                              p["slot_pos"], self.n_q, self.nnz)
        K[p["constrained_diag_positions"]] = 1.0
        if self.elastic is not None:
            K *= 1.0 - R_REG
            K += R_REG * self.elastic
        return F, K

    def time_steps(self, steps, warmup, budget_s=60.0):
        for _ in range(warmup):
            self.step()
        times = []
        t_start = time.perf_counter()
        for _ in range(steps):
            t0 = time.perf_counter()
            self.step()
            times.append(time.perf_counter() - t0)
            if time.perf_counter() - t_start > budget_s:
                break
        return times


# ----------------------------------------------------------------------------- GPU arm


def fp64_peak(torch, lib):
    """Measured FP64 FMA rate of this device (TFLOP/s), from the ssp_probe_dfma kernel."""
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads, iters = sms * 8, 256, 8192
    out = torch.empty(blocks * threads, dtype=torch.float64, device="cuda")
    for _ in range(2):
        lib.call("ssp_probe_dfma", iters, blocks, threads, lib.ptr(out), lib.stream_handle())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    lib.call("ssp_probe_dfma", iters, blocks, threads, lib.ptr(out), lib.stream_handle())
    e1.record()
    torch.cuda.synchronize()
    flops = 16.0 * iters * threads * blocks
    return flops / (e0.elapsed_time(e1) * 1e-3) / 1e12


def peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def kernel_profile(torch, lib, step, op, reps=3):
    """Per-entry-point CUDA-event times, the launches serialised on one stream (the concurrent force
    and the staged values copy would otherwise share the GPU with the kernels inside the brackets)."""
    saved = (op.concurrent_force, op.stage_values)
    op.concurrent_force = False
    op.stage_values = False
    lib.TRACE = []
    for _ in range(reps):
        step()
    torch.cuda.synchronize()
    per = {}
    for name, a, b in lib.TRACE:
        per.setdefault(name, []).append(a.elapsed_time(b))
    lib.TRACE = None
    op.concurrent_force, op.stage_values = saved
    total = sum(sum(v) for v in per.values()) / reps
    return {k: {"ms_per_launch": float(np.mean(v)), "launches_per_step": len(v) / reps,
                "ms_per_step": float(np.sum(v)) / reps, "share": float(np.sum(v)) / reps / total}
            for k, v in sorted(per.items(), key=lambda kv: -sum(kv[1]))}


def workload_stats(op):
    pat = op.owned_tangent_pattern
    n_q = pat.n_q
    br = op._branch.view(-1, n_q)
    plastic = br != 0
    return {"n": pat.n_local_int, "n_el": int(pat.overlap_elements.size), "n_p": pat.n_p, "n_q": n_q, "dim": pat.dim,
            "ns": pat.n_strain, "nnz": pat.nnz, "n_rows": int(pat.local_matrix_pattern.shape[0]),
            "n_u": int(pat.overlap_global_dofs.size), "n_plastic": int(plastic.sum().item()),
            "n_plastic_el": int(plastic.any(dim=1).sum().item()),
            "working_set": sum(v.numel() * v.element_size() for v in pat.device.values())}


def algorithmic(name, st):
    """Algorithmic HBM bytes and FP64 flops of one launch (each datum read or written once)."""
    n, n_el, n_p, n_q, dim, ns = st["n"], st["n_el"], st["n_p"], st["n_q"], st["dim"], st["ns"]
    nld = dim * n_p
    s_out = 6 if dim == 3 else 4
    if name in ("ssp_constitutive_sds_branch", "ssp_constitutive_3d_sds_binned", "ssp_constitutive_3d_sds_learned",
                "ssp_constitutive_3d_sds_binned_mixed", "ssp_constitutive_3d_sds_learned_mixed"):
        return {"bytes": n * (8 * ns + 4 * 8 + 8 * s_out + 8 * ns * ns + 1), "flops": 0}
    if name in ("ssp_assemble_overlap_strain_3d", "ssp_assemble_overlap_strain_2d", "ssp_assemble_overlap_strain_3d_mixed"):
        fp64 = 0 if name.endswith("_mixed") else n * 2 * 9 * n_p  # the mixed kernel's products are FP32
        return {"bytes": n * (8 * dim * n_p + 8 * ns) + n_el * 4 * nld + 8 * st["n_u"], "flops": fp64}
    if name == "ssp_assemble_overlap_strain_3d_affine_mixed":  # J^{-1} per element instead of per-point gradients
        return {"bytes": n * 8 * ns + n_el * (4 * nld + 72) + 8 * st["n_u"], "flops": 0}
    if name == "ssp_assemble_force_element_affine_mixed":
        return {"bytes": n * (8 * ns + 8) + n_el * (4 * nld + 72) + 8 * st["n_rows"], "flops": 0}
    if name == "ssp_assemble_overlap_strain_3d_p2_affine":  # barycentric regrouping, FP64: ≈470 per element
        return {"bytes": n * 8 * ns + n_el * (4 * nld + 72) + 8 * st["n_u"], "flops": n_el * 2 * (204 + 24 * n_q)}
    if name == "ssp_assemble_force_element_p2_affine":  # moments of w σ, FP64: ≈530 per 11-point element
        return {"bytes": n * (8 * ns + 8) + n_el * (4 * nld + 72) + 8 * st["n_rows"], "flops": n_el * 2 * (200 + 30 * n_q)}
    if name == "ssp_assemble_overlap_strain_3d_p2_affine_mixed":  # double-float, barycentric form
        return {"bytes": n * 8 * ns + n_el * (4 * nld + 72) + 8 * st["n_u"], "flops": 0}
    if name == "ssp_assemble_force_element_p2_affine_mixed":
        return {"bytes": n * (8 * ns + 8) + n_el * (4 * nld + 72) + 8 * st["n_rows"], "flops": 0}
    if name in ("ssp_assemble_force_element", "ssp_assemble_force_element_mixed"):
        fp64 = 0 if name.endswith("_mixed") else n * nld * 8
        return {"bytes": n * (8 * dim * n_p + 8 * ns + 8) + n_el * 4 * nld + 8 * st["n_rows"], "flops": fp64}
    if name == "ssp_blend_values":
        return {"bytes": 3 * 8 * st["nnz"], "flops": 0}
    if name == "ssp_reduction":
        return {"bytes": 40 * n, "flops": 0}
    if name == "ssp_gather":
        return {"bytes": 20 * st["n_u"], "flops": 0}
    if name.startswith("ssp_tangent_plastic_correction"):
        npl, npe = st["n_plastic"], st["n_plastic_el"]
        fp64 = npl * 2.0 * nld * ns * dim  # H = B^T (w D): FP64 in both forms
        if not name.endswith("_mixed"):
            fp64 += npl * 2.0 * nld * (nld + 1) // 2 * dim  # the B^T H products
        return {"bytes": n + npl * (8 * ns * ns + 8 * dim * n_p + 24) + npe * (4 * nld * nld + 16 * nld * nld),
                "flops": fp64}
    return {"bytes": 0, "flops": 0}


def time_steps(torch, step, warmup, steps):
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def compare_forms(torch, lib, op, mesh, mats, args, step, ms_plain):
    """The same step in the other forms, on the same state and timed the same way: the mixed
    tangent, the mixed tangent with the learned branch proposal, and the unsorted single-pass
    return mapping (the method without binning).  Restores the plain form afterwards."""
    n_int = op.owned_tangent_pattern.n_local_int
    out = {"plain": {"value": n_int / (ms_plain * 1e-3), "ms_per_step": ms_plain}}
    w = max(args.warmup, 3)
    op.tangent_form = "plain"
    step()
    kp = op.build_K_regularized(R_REG).values.clone()
    for name, form, mapping in (("mixed", "mixed", "binned"), ("mixed+learned", "mixed", "learned"),
                                ("plain+unsorted", "plain", "unsorted"), ("plain+learned", "plain", "learned")):
        if mapping == "learned" and op.branch_model is None:
            out["learned_training"] = train_branch_model(torch, op, mesh, mats, args.config)
        op.tangent_form, op.return_mapping = form, mapping
        ms = time_steps(torch, step, w, args.steps)
        entry = {"value": n_int / (ms * 1e-3), "ms_per_step": ms, "speedup_vs_plain": ms_plain / ms}
        if form == "mixed":
            km = op.build_K_regularized(R_REG).values
            entry["tangent_error_vs_fp64"] = float((km - kp).abs().max() / kp.abs().max())
        out[name] = entry
    op.tangent_form, op.return_mapping = "plain", "binned"
    lib.raise_on_device_status()
    return out


def measure_bddc(torch, lib, op, mesh, specs, args, step):
    """BDDC subdomain tangent of the workload's state: the subdomain owning the elements of the
    lower half of the node range (prepare_bddc_subdomain_pattern), one regularised subdomain build
    per Newton iteration after the owned evaluation; timed with the elastic predictor + plastic
    corrections (FP64 and mixed), and with the full contraction of every subdomain point."""
    from slope_stability_petsc4py_gb300 import prepare_bddc_subdomain_pattern

    owners = np.sort(mesh.elem.min(axis=0))
    owned = (0, int(owners[owners.size // 2]))
    t0 = time.perf_counter()
    pat = prepare_bddc_subdomain_pattern(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs, owned,
                                         elem_type=mesh.elem_type,
                                         overlap_local_int_indices=op.owned_tangent_pattern.local_int_indices)
    prep_s = time.perf_counter() - t0
    op.set_bddc_subdomain_pattern(pat)
    w = max(args.warmup, 3)
    out = {"subdomain_elements": int(pat.local_elements.size), "subdomain_points": pat.n_local_int,
           "nnz": pat.nnz, "owned_node_range": list(owned), "prepare_s": prep_s}
    for name, form in (("plain", "plain"), ("mixed", "mixed")):
        op.tangent_form = form
        step()
        ms = time_steps(torch, lambda: op._build_bddc_regularized_matrix(R_REG), w, args.steps)
        out[name] = {"ms_per_build": ms, "subdomain_quad_pts_per_s": pat.n_local_int / (ms * 1e-3),
                     "assembled_nnz_per_s": pat.nnz / (ms * 1e-3)}
    op.tangent_form = "plain"
    step()
    kp = op._build_bddc_regularized_matrix(R_REG).values.clone()
    op._bddc["predictor_ok"] = False  # time the full contraction of every subdomain point
    ms = time_steps(torch, lambda: op._build_bddc_regularized_matrix(R_REG), w, args.steps)
    kf = op._build_bddc_regularized_matrix(R_REG).values
    out["full_contraction"] = {"ms_per_build": ms, "max_rel_diff_vs_predictor": float((kf - kp).abs().max() / kp.abs().max())}
    op.set_bddc_subdomain_pattern(None)
    lib.raise_on_device_status()
    return out


def measure_graph_replay(torch, lib, op, U_dev, args):
    """The same step as a CUDA graph (ConstitutiveOperator.capture_regularized_build), replayed on
    the displacement tensor: the kernels of build_F_K_regularized_all_free without the host work of
    the Python entry point, for the plain and the mixed form."""
    n_int = op.owned_tangent_pattern.n_local_int
    w = max(args.warmup, 3)
    out = {}
    for form in ("plain", "mixed"):
        op.tangent_form = form
        run = op.capture_regularized_build(LAMBDA, U_dev, R_REG)
        ms = time_steps(torch, run.replay, w, args.steps)
        out[form] = {"value": n_int / (ms * 1e-3), "ms_per_step": ms}
    op.tangent_form = "plain"
    lib.raise_on_device_status()
    return out


def train_branch_model(torch, op, mesh, mats, name):
    """Train the branch-proposal network on continuation states other than the timed one
    (strength-reduction factors 1.0..1.4, shear-band amplitudes 0.4..1.6 x the workload's)."""
    from slope_stability_petsc4py_gb300 import learned, synthetic

    amp0 = synthetic.CONFIGS[name]["amplitude"]
    t0 = time.perf_counter()
    states = [(float(lam), torch.as_tensor(synthetic.displacement_field(mesh, mats, amplitude=amp0 * f, seed=100 + k),
                                           device="cuda"))
              for k, (lam, f) in enumerate(zip(np.linspace(1.0, 1.4, 6), np.linspace(0.4, 1.6, 6)))]
    X, y = learned.collect_training_data(op, states)
    model = learned.BranchProposal(seed=0)
    hist = model.train(X, y, epochs=6, batch=8192, lr=3e-3)
    torch.cuda.synchronize()
    op.branch_model = model
    return {"training_samples": int(X.shape[0]), "samples": "points the elastic screen lists", "epochs": 6,
            "batch": 8192, "final_loss": hist[-1][0],
            "final_train_accuracy": hist[-1][1], "training_s": time.perf_counter() - t0,
            "training_states": "6 states, lambda 1.0..1.4, amplitude 0.4..1.6x (the timed state is held out)"}


def run_gpu(args):
    import torch

    from slope_stability_petsc4py_gb300 import ConstitutiveOperator, _lib

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    mesh, mats, specs, U = workload(args.config)
    op = ConstitutiveOperator.from_mesh(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, specs,
                                        elem_type=mesh.elem_type)
    pat = op.owned_tangent_pattern
    n_int, nnz = pat.n_local_int, pat.nnz
    U_dev = torch.as_tensor(U, device="cuda")
    op.host_outputs = False
    op.tangent_form = args.form
    learned_info = None
    if args.return_mapping == "learned":
        learned_info = train_branch_model(torch, op, mesh, mats, args.config)
    op.return_mapping = args.return_mapping

    def step():  # one Newton iteration through the operator's composite entry point
        op.build_F_K_regularized_all_free(LAMBDA, U_dev, R_REG)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    _lib.raise_on_device_status()

    clocks = ClockSampler(local) if not args.no_clocks else None
    launches0 = _lib.LAUNCHES["count"]
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
        time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    h0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    host_ms = (time.perf_counter() - h0) * 1e3 / args.steps  # the host's enqueue time per step
    e1.record()
    torch.cuda.synchronize()
    clock_info = clocks.stop() if clocks else None
    if dist is not None:
        dist.barrier()
    launches = _lib.LAUNCHES["count"] - launches0
    ms = e0.elapsed_time(e1) / args.steps
    _lib.raise_on_device_status()
    if dist is not None:
        t = torch.tensor([ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())

    # per-kernel durations from a separate traced pass (CUDA events on the launch stream)
    kernels = kernel_profile(torch, _lib, step, op, reps=3)
    stats = workload_stats(op)
    hbm_peak, hbm_src = peaks()
    fp64_tf = fp64_peak(torch, _lib)
    dominant = max(kernels, key=lambda k: kernels[k]["ms_per_step"])
    alg = algorithmic(dominant, stats)
    k_ms = kernels[dominant]["ms_per_launch"]
    achieved_gbs = alg["bytes"] / (k_ms * 1e-3) / 1e9
    corr = "ssp_tangent_plastic_correction" + ("_mixed" if args.form == "mixed" else "")
    tangent_err = None
    if args.form == "mixed":  # tangent error of this form against the FP64 form, same state
        op.tangent_form = "plain"
        step()
        kp = op.build_K_regularized(R_REG).values.clone()
        op.tangent_form = "mixed"
        step()
        km = op.build_K_regularized(R_REG).values
        tangent_err = {"max_norm_rel": float((km - kp).abs().max() / kp.abs().max()),
                       "frobenius_rel": float(torch.linalg.norm(km - kp) / torch.linalg.norm(kp))}
    fl = algorithmic(corr, stats)["flops"]
    corr_ms = kernels.get(corr, {}).get("ms_per_launch")
    line = {
        "metric": METRIC, "value": world * n_int / (ms * 1e-3), "unit": "quad-pts/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "tangent_error_vs_fp64": tangent_err,
        "config": {"workload": describe(args.config, mesh, n_int, nnz), "form": args.form,
                   "return_mapping": args.return_mapping,
                   "plastic_elements": stats["n_plastic_el"],
                   "step": "reduction + strain + return mapping (S, DS) + owned force + tangent CSR values + "
                           "constrained diagonals + regularised blend",
                   "plastic_fraction": stats["n_plastic"] / n_int,
                   "l2": f"inputs larger than L2 (per-step HBM working set {stats['working_set'] / 1e9:.2f} GB > 129 MB)",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "assembled_nnz_per_s": world * nnz / (ms * 1e-3),
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved_gbs / hbm_peak,
                     "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if hbm_src == "measured" else hbm_src,
                     "traffic": NCU_TRAFFIC.get(args.config, {}).get(dominant), "ms_per_launch": k_ms,
                     "algorithmic_bytes": alg["bytes"]},
        "roofline_fp64": ({"bound": "fp64", "kernel": corr, "achieved": fl / (corr_ms * 1e-3) / 1e12, "peak": fp64_tf,
                           "unit": "TFLOP/s", "frac": fl / (corr_ms * 1e-3) / 1e12 / fp64_tf,
                           "peak_source": "measured live (ssp_probe_dfma, FP64 FMA)", "algorithmic_flops": fl,
                           "ms_per_launch": corr_ms} if corr_ms else None),
        "kernels": kernels,
        "host_enqueue_ms_per_step": host_ms,
        "gpu_launches": launches,
        "clocks": clock_info,
    }
    if learned_info is not None:
        from slope_stability_petsc4py_gb300 import learned

        br = op._branch
        listed, bins = learned.proposal_bins(op._scratch, br.numel())
        n_listed = max(1, listed.numel())
        learned_info["listed_points"] = int(listed.numel())
        learned_info["bench_state_accuracy_listed"] = float(
            sum(int((br.index_select(0, bins[k]) == k).sum().item()) for k in range(5)) / n_listed)
        learned_info["distinct_branches_per_warp_listed"] = {
            "screen_order": learned.warp_branch_mix(br, listed),
            "learned_bins": learned.warp_branch_mix(br, torch.cat(bins))}
        line["learned"] = learned_info

    if args.form == "plain" and args.return_mapping == "binned" and pat.dim == 3 and not args.no_forms:
        line["forms"] = compare_forms(torch, _lib, op, mesh, mats, args, step, ms)
    if args.bddc:
        line["bddc"] = measure_bddc(torch, _lib, op, mesh, specs, args, step)
    if args.form == "plain" and args.return_mapping == "binned" and not args.no_forms:
        line["graph_replay"] = measure_graph_replay(torch, _lib, op, U_dev, args)

    if rank == 0 and not args.no_e2e:
        op.host_outputs = True
        U_pin = torch.as_tensor(U).pin_memory()
        for _ in range(3):
            F_free, K = op.build_F_K_regularized_all_free(LAMBDA, U_pin, R_REG)
            K.getValuesCSR()
        torch.cuda.synchronize()
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            F_free, K = op.build_F_K_regularized_all_free(LAMBDA, U_pin, R_REG)
            K.getValuesCSR()  # synchronises: the CSR values are on the host
            times.append(time.perf_counter() - t0)
        t_e2e = float(np.median(times))
        # the host mirror of K is refreshed where the values can have changed since the previous
        # build (rows of both builds' plastic elements); the rest already holds this r's values
        line["e2e"] = {"value": n_int / t_e2e, "unit": "quad-pts/s", "h2d_bytes_per_step": int(U.nbytes),
                       "d2h_bytes_per_step": int(F_free.nbytes + K.host_copy_bytes()), "ms_per_step": t_e2e * 1e3,
                       "d2h_csr_bytes_full": 8 * nnz,
                       "api": "ConstitutiveOperator.build_F_K_regularized_all_free(lam, U_host, r) + K.getValuesCSR()"}
        if args.form == "plain" and pat.dim == 3 and not args.no_forms:
            # the same end-to-end step in the mixed form
            op.tangent_form = "mixed"
            for _ in range(3):
                op.build_F_K_regularized_all_free(LAMBDA, U_pin, R_REG)[1].getValuesCSR()
            times = []
            for _ in range(args.steps):
                t0 = time.perf_counter()
                F_free, K = op.build_F_K_regularized_all_free(LAMBDA, U_pin, R_REG)
                K.getValuesCSR()
                times.append(time.perf_counter() - t0)
            op.tangent_form = "plain"
            t_mx = float(np.median(times))
            line["e2e"]["mixed"] = {"value": n_int / t_mx, "ms_per_step": t_mx * 1e3,
                                    "d2h_bytes_per_step": int(F_free.nbytes + K.host_copy_bytes())}

    if rank == 0 and not args.no_cpu_baseline:
        runner = OracleRunner(mesh, specs, U, dphi=(pat.dphi1, pat.dphi2, pat.dphi3), weight=pat.overlap_assembly_weight)
        runner.elastic = pat.elastic_values
        times = runner.time_steps(steps=5, warmup=1, budget_s=30.0)
        t_cpu = float(np.median(times))
        line["cpu_baseline"] = {"value": n_int / t_cpu, "unit": "quad-pts/s", "cores": runner.o.num_threads(),
                                "kind": "port",
                                "sample": f"full workload, {len(times)} passes after 1 warm-up, median; oracle C "
                                          f"restatement of the reference kernels (rows tangent), OpenMP"}
    if dist is not None:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    mesh, mats, specs, U = workload(args.config)
    runner = OracleRunner(mesh, specs, U)
    times = runner.time_steps(args.steps, args.warmup, budget_s=150.0)
    t = float(np.median(times))
    value = runner.n_int / t
    line = {"metric": METRIC, "value": value, "unit": "quad-pts/s", "n_gpus": world, "steps": len(times),
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": describe(args.config, mesh, runner.n_int, runner.nnz), "form": "plain",
                       "parallelism": "host cores (OpenMP)"},
            "cpu_baseline": {"value": value, "unit": "quad-pts/s", "cores": runner.o.num_threads(), "kind": "port",
                             "sample": f"full workload per step, median of {len(times)}; the reference's C kernels "
                                       f"restated (oracle), constrained diagonals without the elastic blend"},
            "e2e": {"value": value, "unit": "quad-pts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.mesh:
        from slope_stability_petsc4py_gb300 import synthetic

        args.config = synthetic.register_mesh_file(args.mesh, elem_type=args.mesh_elem)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
