"""Benchmark of the Newton hot path: quadrature points per second of one builder pass.

One step = one Newton iteration of the reference's owned-row builder on a synthetic slope:
strength reduction -> strain B u -> Mohr-Coulomb return mapping (S and DS) -> owned internal
force B^T (w S) -> tangent CSR values sum B^T (w DS) B -> constrained diagonals and the
regularised blend (1-r) K + r K_elast.  The timed steps cycle through four displacement states of
one continuation (a shear band growing at fixed lambda and r), pre-uploaded to HBM, so the plastic
set moves from step to step.

* ``value``: inputs resident in HBM, CUDA events over the timed steps.
* ``e2e``: the same steps through ``ConstitutiveOperator.build_F_K_regularized_all_free`` with
  pinned host U and host outputs (F_free and the CSR values the PETSc hand-off reads).
* ``parity``: the GPU outputs (plain and mixed forms) of one state against the oracle -- the CPU
  restatement of the reference's kernels -- on the whole workload, pattern included.
* ``cpu_baseline`` / ``--impl reference``: the oracle's restatement of the reference's kernels on
  the host cores, on a bounded sample of the workload (contiguous runs of elements spread over the
  mesh, built as a mesh of their own), the same states.
* ``roofline`` / ``roofline_fp64``: the dominant kernel's algorithmic bytes over its CUDA-event
  time against the measured HBM bandwidth, and its FP64 operations against the live FP64 probe;
  ``kernel_rooflines`` the same for every step kernel.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config 3d_p2_large] [--impl reference]
"""

from __future__ import annotations

import argparse
import json
import math
import os
import platform
import subprocess
import sys
import tempfile
import time
from pathlib import Path
from types import SimpleNamespace

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "quad-pts/s constitutive+tangent; FP64 plain vs mixed+learned at ≤1e-6 err"
LAMBDA, R_REG, DAVIS = 1.1, 0.1, "B"
DEFAULT_CONFIG = "3d_p2_large"
# the other benchmarked configurations, measured (and checked against the oracle) after the headline
OTHER_WORKLOADS = ("2d_p2_homo", "3d_p2_homo", "3d_p2_hetero", "3d_p4_hetero")
# shear-band amplitude of the four timed states, times the workload's amplitude (fixed lambda and r)
STATE_FACTORS = (0.9, 1.0, 1.1, 1.2)
# a strength-reduction sequence: 10 lambda steps of 6 Newton iterations; the load and the band grow
# over the steps so the plastic fraction rises from about 2 % to 35 % (3D heterogeneous slopes)
SSR_STEPS, SSR_ITERS = 10, 6
# points per step of the bounded CPU samples (all host threads, and one thread)
SAMPLE_POINTS, SAMPLE_POINTS_1T = 4_000_000, 250_000
# DRAM bytes (read + write) per launch of the step kernels, from one ncu capture each (the command in
# profiles/dram_traffic_3d_p2_large.md), keyed by workload and entry point; reported as roofline.traffic
# with that source when the bench's dominant kernel is one of them
NCU_TRAFFIC = {"3d_p2_large": {
    "ssp_tangent_plastic_correction_p2_moments": (2994.5e6 + 1058.4e6,
                                                  "ncu capture 2026-12-04, profiles/dram_traffic_3d_p2_large.md"),
    "ssp_tangent_plastic_correction_p2_moments_mixed": (4694.0e6 + 1440.7e6,
                                                        "ncu capture 2026-12-04, profiles/dram_traffic_3d_p2_large.md"),
}}
STEP_TEXT = ("reduction + strain + return mapping (S, DS) + owned force + tangent CSR values + constrained diagonals "
             "+ regularised blend")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default=DEFAULT_CONFIG)
    ap.add_argument("--mesh", default=None, help="a gmsh .msh tet4 file as the workload (overrides --config)")
    ap.add_argument("--mesh-elem", default="P2", choices=["P1", "P2", "P4"], help="element order for --mesh")
    ap.add_argument("--form", default="plain", choices=["plain", "mixed"],
                    help="plain: FP64 tangent (the drop-in); mixed: FP32 plastic-point products")
    ap.add_argument("--return-mapping", default="binned", choices=["binned", "unsorted", "learned", "previous"],
                    help="binned: exact screen/decide/finish binning; unsorted: one divergent pass; learned: bins "
                         "proposed by the branch network; previous: bins of the previous iteration's branches")
    ap.add_argument("--no-forms", action="store_true", help="skip timing the mixed / learned / unsorted forms")
    ap.add_argument("--no-ssr", action="store_true", help="skip the strength-reduction sequence")
    ap.add_argument("--no-others", action="store_true", help="skip the other benchmarked configurations")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle comparison")
    ap.add_argument("--bddc", action="store_true", help="also time the BDDC subdomain tangent of half the mesh")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-clocks", action="store_true")
    return ap.parse_args()


# ----------------------------------------------------------------------------- workload


def workload(name: str):
    """Mesh, materials and the displacement basis (G, V) of a named configuration: every state of
    the benchmark is g G + a V (load factor g, shear-band amplitude a)."""
    from slope_stability_petsc4py_gb300 import synthetic

    return synthetic.config_workload(name)


def timed_states(w):
    return [w.G + (f * w.amp) * w.V for f in STATE_FACTORS]


def ssr_target(w, k):
    """lambda and displacement at the end of strength-reduction step k (k = -1: the undeformed start)."""
    if k < 0:
        return 1.0, np.zeros_like(w.G)
    x = k / (SSR_STEPS - 1)
    g = 0.13 * (1.0 / 0.13) ** x
    a = 0.15 * (12.0 / 0.15) ** x
    return 1.0 + 0.05 * k, g * w.G + (a * w.amp) * w.V


def ssr_states(w):
    """(lambda, U) of every Newton iteration of the sequence: within step k the iterates move from
    the previous step's solution towards this step's by 1/2, 3/4, 7/8, ... of the increment."""
    prev = ssr_target(w, -1)[1]
    for k in range(SSR_STEPS):
        lam, tgt = ssr_target(w, k)
        for it in range(SSR_ITERS):
            s = 1.0 - 0.5 ** (it + 1)
            yield k, it, lam, prev + s * (tgt - prev)
        prev = tgt


def describe(name, mesh, n_int, nnz):
    return (f"{name}: {mesh.n_elem:,} {mesh.dim}D {mesh.elem_type} elements, {n_int:,} quadrature points, "
            f"{mesh.n_nodes * mesh.dim:,} dofs, {nnz:,} CSR nnz")


def bench_config(w, n_int, nnz):
    """The workload's description; both arms print this same dict."""
    return {"workload": describe(w.name, w.mesh, n_int, nnz), "step": STEP_TEXT,
            "states": f"{len(STATE_FACTORS)} displacement states cycled (gravity + tanh shear band, amplitude "
                      f"{', '.join(f'{f:g}' for f in STATE_FACTORS)} x {w.amp:g} m), lambda {LAMBDA}, r {R_REG}, "
                      f"Davis {DAVIS}",
            "l2": f"inputs larger than L2: >= 424 B per point of constitutive data alone "
                  f"({424 * n_int / 1e9:.2f} GB) against the 129 MB L2"}


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


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return f"{line.split(':', 1)[1].strip()} ({platform.machine()})"
    except Exception:
        pass
    return platform.processor() or platform.machine()


# ----------------------------------------------------------------------------- the reference on the CPU


def oracle_runner(w):
    from oracle.newton_step import OracleNewtonStep

    return OracleNewtonStep(w.mesh, w.specs)


def cpu_sample(w, n_points_goal, n_q):
    """A bounded sample of the workload for the CPU: about n_points_goal quadrature points worth of
    elements (sixteen contiguous runs spread over the element order) as a mesh of its own, and the
    timed states restricted to its nodes.  The reference does the same work per element on it."""
    from slope_stability_petsc4py_gb300 import synthetic

    sub, nodes = synthetic.element_sample(w.mesh, max(1, n_points_goal // n_q))
    return sub, [U[:, nodes] for U in timed_states(w)]


def cpu_reference_figures(w, *, steps, warmup, budget_s):
    """The oracle timed on bounded samples of the workload: every host thread on one sample, one
    thread on a smaller one.  Returns a dict for the line's cpu_baseline."""
    from oracle import oracle_py as o
    from oracle.newton_step import OracleNewtonStep
    from slope_stability_petsc4py_gb300 import fem

    n_q = len(fem.quadrature(w.mesh.dim, w.mesh.elem_type)[1])
    sub, states = cpu_sample(w, SAMPLE_POINTS, n_q)
    runner = OracleNewtonStep(sub, w.specs)
    times = runner.time_steps(states, steps, warmup, LAMBDA, R_REG, budget_s=budget_s)
    t = float(np.median(times))
    threads = o.num_threads()
    sub1, states1 = cpu_sample(w, SAMPLE_POINTS_1T, n_q)
    one = OracleNewtonStep(sub1, w.specs)
    o.set_num_threads(1)
    try:
        t1 = float(np.median(one.time_steps(states1, 2, 1, LAMBDA, R_REG)))
    finally:
        o.set_num_threads(threads)
    return {"value": runner.n_int / t, "unit": "quad-pts/s", "cores": threads, "kind": "port",
            "cpu_model": cpu_model(), "ms_per_step": t * 1e3, "steps": len(times),
            "sample": sample_text(w, sub, runner, len(times), warmup, threads),
            "one_thread": {"value": one.n_int / t1, "unit": "quad-pts/s", "cores": 1, "ms_per_step": t1 * 1e3,
                           "sample": f"{sub1.n_elem:,} of the {w.mesh.n_elem:,} elements ({one.n_int:,} points, "
                                     f"{one.nnz:,} nnz), median of 2 steps after 1 warm-up"}}


def sample_text(w, sub, runner, steps, warmup, threads):
    return (f"{sub.n_elem:,} of the {w.mesh.n_elem:,} elements per step (16 contiguous runs spread over the mesh, "
            f"as a mesh of their own: {runner.n_int:,} points, {runner.nnz:,} nnz), the same {len(STATE_FACTORS)} "
            f"states; median of {steps} steps after {warmup} warm-up; the reference's C kernels restated (oracle), "
            f"OpenMP on {threads} threads; pattern, geometry and elastic values built once outside the steps")


# ----------------------------------------------------------------------------- GPU arm helpers


def fp64_peak(torch):
    """Measured FP64 FMA rate of this device (TFLOP/s): the bench-only probe library's kernel, eight
    independent FMA chains per thread over 8 CTAs per SM."""
    import ctypes

    from slope_stability_petsc4py_gb300 import build

    lib = ctypes.CDLL(str(build.PROBE_LIB))
    lib.ssp_probe_dfma.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 2
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads, iters = sms * 8, 256, 8192
    out = torch.empty(blocks * threads, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        assert lib.ssp_probe_dfma(iters, blocks, threads, out.data_ptr(), st) == 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    assert lib.ssp_probe_dfma(iters, blocks, threads, out.data_ptr(), st) == 0
    e1.record()
    torch.cuda.synchronize()
    return 16.0 * iters * threads * blocks / (e0.elapsed_time(e1) * 1e-3) / 1e12


def peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    return 6800.0, "fallback (6.8 TB/s)"


def make_step(op, states_dev, lam=LAMBDA, r=R_REG):
    """One Newton iteration per call through the operator's composite entry point, cycling the
    pre-uploaded states."""
    k = [0]

    def step():
        op.build_F_K_regularized_all_free(lam, states_dev[k[0] % len(states_dev)], r)
        k[0] += 1

    return step


def kernel_profile(torch, lib, op, states_dev):
    """Per-entry-point CUDA-event times over one pass through the states, the launches serialised on
    one stream (the concurrent force and the staged values copy would otherwise share the GPU with
    the kernels inside the brackets); plastic counts per state."""
    saved = (op.concurrent_force, op.stage_values)
    op.concurrent_force = False
    op.stage_values = False
    step = make_step(op, states_dev)
    for _ in range(len(states_dev)):  # settle the incremental restore on this state order
        step()
    torch.cuda.synchronize()
    lib.TRACE = []
    plastic = []
    for _ in range(len(states_dev)):
        step()
        plastic.append(workload_plastic(op))
    torch.cuda.synchronize()
    per = {}
    for name, a, b in lib.TRACE:
        per.setdefault(name, []).append(a.elapsed_time(b))
    lib.TRACE = None
    op.concurrent_force, op.stage_values = saved
    reps = len(states_dev)
    total = sum(sum(v) for v in per.values()) / reps
    kernels = {k: {"ms_per_launch": float(np.mean(v)), "launches_per_step": len(v) / reps,
                   "ms_per_step": float(np.sum(v)) / reps, "share": float(np.sum(v)) / reps / total}
               for k, v in sorted(per.items(), key=lambda kv: -sum(kv[1]))}
    return kernels, plastic


def workload_plastic(op):
    """Plastic points and elements of the current state; with the moment form of the P2 correction,
    also the elements (and their plastic points) at or above its plastic-point split."""
    n_q = op.owned_tangent_pattern.n_q
    plastic = op._branch.view(-1, n_q) != 0
    per_el = plastic.sum(dim=1)
    split = op.moment_min_points_mixed if op.tangent_form == "mixed" else op.moment_min_points
    many = per_el >= max(int(split or 0), 1)
    return {"n_plastic": int(plastic.sum().item()), "n_plastic_el": int(plastic.any(dim=1).sum().item()),
            "n_many_el": int(many.sum().item()), "n_plastic_many": int(per_el[many].sum().item())}


def workload_stats(op, plastic):
    pat = op.owned_tangent_pattern
    return {"n": pat.n_local_int, "n_el": int(pat.overlap_elements.size), "n_p": pat.n_p, "n_q": pat.n_q,
            "dim": pat.dim, "ns": pat.n_strain, "nnz": pat.nnz, "n_rows": int(pat.local_matrix_pattern.shape[0]),
            "n_u": int(pat.overlap_global_dofs.size),
            "n_plastic": float(np.mean([p["n_plastic"] for p in plastic])),
            "n_plastic_el": float(np.mean([p["n_plastic_el"] for p in plastic])),
            "n_many_el": float(np.mean([p["n_many_el"] for p in plastic])),
            "n_plastic_many": float(np.mean([p["n_plastic_many"] for p in plastic])),
            "device_bytes": sum(v.numel() * v.element_size() for v in pat.device.values())}


def algorithmic(name, st):
    """Algorithmic bytes and FP64 flops of one launch, from the per-unit costs of the hot-path cost
    table (reference layouts, every datum moved once):
      return mapping S+DS  424 B/point (3D: E 48, five material arrays 40, S 48, DS 288; 2D: 168)
      S only               136 B/point
      strain               24 n_p + 48 B/point + 3 n_p (8 + 4) B/element (2D: 16 n_p + 24, 2 n_p * 12)
      force                48 + 24 n_p B/point + 8 B/row (2D: 32 + 16 n_p)
      tangent values       per element: 288 n_q + 24 n_p n_q + 8 n_q + 4 (3 n_p)^2 + 8 nnz/n_el;
                           2 n_q 3 n_p (18 + 9 n_p) flops ('rows' formulation);
                           the plastic correction counts the plastic elements it visits.
    'fp64' is the FP64 work this library's kernels execute (symmetric halves, plastic points only)."""
    n, n_el, n_p, n_q, dim, ns = st["n"], st["n_el"], st["n_p"], st["n_q"], st["dim"], st["ns"]
    nld = dim * n_p
    if name == "ssp_constitutive_3d_s":
        return {"bytes": 136 * n, "flops": 0, "fp64": 0}
    if name.startswith("ssp_constitutive"):
        per = 424 if dim == 3 else 24 + 40 + 32 + 72
        return {"bytes": per * n, "flops": 0, "fp64": 0}
    if name.startswith("ssp_assemble_overlap_strain"):
        per_pt = 24 * n_p + 48 if dim == 3 else 16 * n_p + 24
        fp64 = 0 if "mixed" in name else (n_el * 2 * (222 + 18 * n_q) if "p2_affine" in name else n * 2 * 9 * n_p)
        return {"bytes": n * per_pt + n_el * nld * 12, "flops": n * 2 * ns * dim * n_p, "fp64": fp64}
    if name.startswith("ssp_assemble_force"):
        per_pt = 48 + 24 * n_p if dim == 3 else 32 + 16 * n_p
        fp64 = 0 if "mixed" in name else (n_el * 2 * (200 + 30 * n_q) if "p2_affine" in name else n * nld * 8)
        return {"bytes": n * per_pt + 8 * st["n_rows"], "flops": n * 2 * ns * nld, "fp64": fp64}
    per_el = 288 * n_q + 24 * n_p * n_q + 8 * n_q + 4 * nld * nld + 8 * st["nnz"] / max(n_el, 1)
    fl_el = 2 * n_q * nld * (18 + 9 * n_p)
    if name == "ssp_tangent_plastic_correction_p2_moments_mixed":
        # FP64 only for DS - D_el (21 entries) and w s per plastic point; the rest FP32
        units = st["n_many_el"]
        return {"bytes": units * per_el, "flops": units * fl_el, "fp64": 2.0 * 22 * st["n_plastic_many"],
                "units": f"{units:.0f} plastic elements in moment form per launch"}
    if name == "ssp_tangent_plastic_correction_p2_moments":
        # elements at or above the split: 7,530 FP64 operations per element + 261 per plastic point
        # (DS - D_el, weighted coordinate products, moments, beta^T M, R, the R sums, K), FMA-equivalent
        units = st["n_many_el"]
        return {"bytes": units * per_el, "flops": units * fl_el,
                "fp64": 2.0 * (7530 * units + 261 * st["n_plastic_many"]),
                "units": f"{units:.0f} plastic elements at or above the moment-form split per launch"}
    if name.startswith("ssp_tangent_plastic_correction"):
        units, n_pl = st["n_plastic_el"], st["n_plastic"]
        if st.get("moments"):  # the elements below the split
            units, n_pl = units - st["n_many_el"], n_pl - st["n_plastic_many"]
        fp64 = n_pl * 2.0 * nld * ns * dim  # H = B^T (w dD): FP64 in both forms
        if not name.endswith("_mixed"):
            fp64 += n_pl * 2.0 * nld * (nld + 1) // 2 * dim  # the B^T H products, upper half
        return {"bytes": units * per_el, "flops": units * fl_el, "fp64": fp64,
                "units": f"{units:.0f} plastic elements per launch"}
    if name in ("ssp_tangent_element", "ssp_assemble_tangent_values_3d_rows", "ssp_assemble_tangent_values_3d_p2"):
        return {"bytes": n_el * per_el, "flops": n_el * fl_el, "fp64": n_el * fl_el}
    if name == "ssp_blend_values":
        return {"bytes": 24 * st["nnz"], "flops": 0, "fp64": 0}
    return {"bytes": 0, "flops": 0, "fp64": 0}


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


def train_branch_model(torch, op, w, *, total=5_000_000, max_per_state=500_000):
    """Train the branch-proposal network on the exact return mapping's (features, branch) pairs of a
    strength-reduction sequence: every Newton iterate of its ten lambda steps (plastic fraction about
    2 % to 40 %), at most max_per_state screen-listed points of each, then a seeded uniform sample of
    `total` of them.  The timed states are not among them."""
    from slope_stability_petsc4py_gb300 import learned

    t0 = time.perf_counter()
    Xs, ys = [], []
    for k, it, lam, U in ssr_states(w):
        X, y = learned.collect_training_data(op, [(lam, torch.as_tensor(U, device="cuda"))],
                                             max_per_state=max_per_state, seed=7 * k + it)
        Xs.append(X)
        ys.append(y)
    X, y = torch.cat(Xs), torch.cat(ys)
    del Xs, ys
    collected = int(X.shape[0])
    if collected > total:
        gen = torch.Generator(device="cuda")
        gen.manual_seed(11)
        pick = torch.randperm(collected, device="cuda", generator=gen)[:total]
        X, y = X.index_select(0, pick).contiguous(), y.index_select(0, pick).contiguous()
    model = learned.BranchProposal(seed=0)
    epochs = 4
    hist = model.train(X, y, epochs=epochs, batch=16384, lr=3e-3)
    torch.cuda.synchronize()
    op.branch_model = model
    counts = torch.bincount(y.long(), minlength=5).cpu().numpy()
    op.reduction(LAMBDA)
    return {"training_samples": int(X.shape[0]), "collected": collected, "samples": "points the elastic screen lists",
            "label_counts": {b: int(c) for b, c in zip(learned.BRANCHES, counts)}, "epochs": epochs, "batch": 16384,
            "final_loss": hist[-1][0], "final_train_accuracy": hist[-1][1], "training_s": time.perf_counter() - t0,
            "training_states": f"every Newton iterate ({SSR_STEPS} lambda steps x {SSR_ITERS}) of the strength-reduction "
                               f"sequence (lambda 1.0..1.45), at most {max_per_state:,} listed points each, then "
                               f"{total:,} drawn uniformly"}


def compare_forms(torch, lib, op, w, states_dev, args, ms_plain):
    """The same steps in the other forms, on the same moving states, timed the same way: the mixed
    tangent; the exact binning replaced by the network's proposal (learned) or by the previous
    iteration's branches (previous, the trivial predictor); the single-pass unsorted return mapping
    (the method without binning).  Restores the plain binned form afterwards."""
    n_int = op.owned_tangent_pattern.n_local_int
    out = {"plain": {"value": n_int / (ms_plain * 1e-3), "ms_per_step": ms_plain}}
    wu = max(args.warmup, 3)
    step = make_step(op, states_dev)
    op.tangent_form, op.return_mapping = "plain", "binned"
    for _ in range(len(states_dev)):
        step()
    ref_K = []
    for U in states_dev:
        op.build_F_K_regularized_all_free(LAMBDA, U, R_REG)
        ref_K.append(op.build_K_regularized(R_REG).values.clone())
    for name, form, mapping in (("mixed", "mixed", "binned"), ("mixed+learned", "mixed", "learned"),
                                ("mixed+previous", "mixed", "previous"), ("plain+unsorted", "plain", "unsorted"),
                                ("plain+learned", "plain", "learned"), ("plain+previous", "plain", "previous")):
        if mapping == "learned" and op.branch_model is None:
            out["learned_training"] = train_branch_model(torch, op, w)
        op.tangent_form, op.return_mapping = form, mapping
        ms = time_steps(torch, step, wu, args.steps)
        entry = {"value": n_int / (ms * 1e-3), "ms_per_step": ms, "speedup_vs_plain": ms_plain / ms}
        if form == "mixed":
            errs = []
            for U, kp in zip(states_dev, ref_K):
                op.build_F_K_regularized_all_free(LAMBDA, U, R_REG)
                km = op.build_K_regularized(R_REG).values
                errs.append(float((km - kp).abs().max() / kp.abs().max()))
            entry["tangent_error_vs_fp64"] = max(errs)
        out[name] = entry
    op.tangent_form, op.return_mapping = "plain", "binned"
    lib.raise_on_device_status()
    return out


def measure_new_lambda_r(torch, lib, op, states_dev, reps=6):
    """Steps that start a new continuation step: every one at a new (lambda, r), so the reduction
    and the regularised elastic base are recomputed inside it (CUDA events around each step)."""
    out = {}
    for form in ("plain", "mixed"):
        op.tangent_form = form
        times = []
        for k in range(reps):
            lam, r = LAMBDA + 0.013 * (k + 1), R_REG + 0.007 * (k + 1)
            U = states_dev[k % len(states_dev)]
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            op.build_F_K_regularized_all_free(lam, U, r)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        out[form] = {"ms_per_step": float(np.median(times[1:])), "steps": reps - 1,
                     "value": op.owned_tangent_pattern.n_local_int / (np.median(times[1:]) * 1e-3)}
    op.tangent_form = "plain"
    op.build_F_K_regularized_all_free(LAMBDA, states_dev[0], R_REG)  # back to the timed lambda and r
    torch.cuda.synchronize()
    lib.raise_on_device_status()
    return out


def measure_ssr(torch, lib, op, w, forms=(("plain", "plain", "binned"), ("mixed", "mixed", "binned"),
                                        ("mixed+learned", "mixed", "learned"))):
    """The strength-reduction sequence (10 lambda steps x 6 Newton iterations, load and shear band
    growing, r fixed) with every state pre-uploaded: each iteration one composite build; per-lambda-step
    plastic fractions and the time of the whole sequence per form."""
    seq = [(k, it, lam, torch.as_tensor(U, device="cuda")) for k, it, lam, U in ssr_states(w)]
    n_int = op.owned_tangent_pattern.n_local_int
    out = {"lambda_steps": SSR_STEPS, "newton_iterations_per_step": SSR_ITERS, "r": R_REG}
    fractions = []
    for name, form, mapping in forms:
        if mapping == "learned" and op.branch_model is None:
            continue
        op.tangent_form, op.return_mapping = form, mapping
        for k, it, lam, U in seq[:3]:  # warm-up
            op.build_F_K_regularized_all_free(lam, U, R_REG)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for k, it, lam, U in seq:
            op.build_F_K_regularized_all_free(lam, U, R_REG)
            if name == "plain" and it == SSR_ITERS - 1:
                fractions.append((k, lam, (op._branch != 0).float().mean()))
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / len(seq)
        out[name] = {"ms_per_iteration": ms, "value": n_int / (ms * 1e-3)}
    out["plastic_fraction_per_step"] = [{"step": k, "lambda": round(lam, 3), "plastic_fraction": float(f.item())}
                                        for k, lam, f in fractions]
    op.tangent_form, op.return_mapping = "plain", "binned"
    del seq
    lib.raise_on_device_status()
    return out


def measure_graph_replay(torch, lib, op, states_dev, args):
    """The same steps as a CUDA graph (ConstitutiveOperator.capture_regularized_build), replayed
    after each state is copied into the captured displacement buffer (the copy is timed too)."""
    n_int = op.owned_tangent_pattern.n_local_int
    wu = max(args.warmup, 3)
    out = {}
    U_buf = states_dev[0].clone()
    for form in ("plain", "mixed"):
        op.tangent_form = form
        run = op.capture_regularized_build(LAMBDA, U_buf, R_REG)
        k = [0]

        def replay():
            U_buf.copy_(states_dev[k[0] % len(states_dev)])
            k[0] += 1
            run.replay()

        ms = time_steps(torch, replay, wu, args.steps)
        out[form] = {"value": n_int / (ms * 1e-3), "ms_per_step": ms}
    op.tangent_form = "plain"
    lib.raise_on_device_status()
    return out


def measure_bddc(torch, lib, op, w, states_dev, args):
    """BDDC subdomain tangent (prepare_bddc_subdomain_pattern on the lower half of the node range),
    one regularised subdomain build per Newton iteration after the owned evaluation: elastic
    predictor + plastic corrections (FP64 and mixed), and the full contraction of every point."""
    from slope_stability_petsc4py_gb300 import prepare_bddc_subdomain_pattern

    mesh = w.mesh
    owners = np.sort(mesh.elem.min(axis=0))
    owned = (0, int(owners[owners.size // 2]))
    t0 = time.perf_counter()
    pat = prepare_bddc_subdomain_pattern(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, w.specs, owned,
                                         elem_type=mesh.elem_type,
                                         overlap_local_int_indices=op.owned_tangent_pattern.local_int_indices)
    prep_s = time.perf_counter() - t0
    op.set_bddc_subdomain_pattern(pat)
    wu = max(args.warmup, 3)
    out = {"subdomain_elements": int(pat.local_elements.size), "subdomain_points": pat.n_local_int,
           "nnz": pat.nnz, "owned_node_range": list(owned), "prepare_s": prep_s}
    op.build_F_K_regularized_all_free(LAMBDA, states_dev[1], R_REG)
    for form in ("plain", "mixed"):
        op.tangent_form = form
        op.build_F_K_regularized_all_free(LAMBDA, states_dev[1], R_REG)
        ms = time_steps(torch, lambda: op.build_bddc_regularized_matrix(R_REG), wu, args.steps)
        out[form] = {"ms_per_build": ms, "subdomain_quad_pts_per_s": pat.n_local_int / (ms * 1e-3),
                     "assembled_nnz_per_s": pat.nnz / (ms * 1e-3)}
    op.tangent_form = "plain"
    op.build_F_K_regularized_all_free(LAMBDA, states_dev[1], R_REG)
    kp = op.build_bddc_regularized_matrix(R_REG).values.clone()
    op._bddc["predictor_ok"] = False  # time the full contraction of every subdomain point
    ms = time_steps(torch, lambda: op.build_bddc_regularized_matrix(R_REG), wu, args.steps)
    kf = op.build_bddc_regularized_matrix(R_REG).values
    out["full_contraction"] = {"ms_per_build": ms, "max_rel_diff_vs_predictor": float((kf - kp).abs().max() /
                                                                                       kp.abs().max())}
    op.set_bddc_subdomain_pattern(None)
    lib.raise_on_device_status()
    return out


def measure_e2e(torch, op, states_host, args, form):
    """The timed steps through the public API with host buffers: pinned host U in, F_free and the
    CSR values (K.getValuesCSR(), the PETSc hand-off's input) out, wall clock per step."""
    op.host_outputs = True
    op.tangent_form = form
    pinned = [torch.as_tensor(U).pin_memory() for U in states_host]
    nst = len(pinned)
    for k in range(max(3, nst)):
        op.build_F_K_regularized_all_free(LAMBDA, pinned[k % nst], R_REG)[1].getValuesCSR()
    torch.cuda.synchronize()
    times, d2h = [], []
    for k in range(args.steps):
        t0 = time.perf_counter()
        F_free, K = op.build_F_K_regularized_all_free(LAMBDA, pinned[k % nst], R_REG)
        K.getValuesCSR()  # synchronises: the CSR values are on the host
        times.append(time.perf_counter() - t0)
        d2h.append(int(F_free.nbytes + K.host_copy_bytes()))
    op.host_outputs = False
    op.tangent_form = "plain"
    t = float(np.median(times))
    n_int = op.owned_tangent_pattern.n_local_int
    return {"value": n_int / t, "unit": "quad-pts/s", "h2d_bytes_per_step": int(states_host[0].nbytes),
            "d2h_bytes_per_step": int(np.mean(d2h)), "ms_per_step": t * 1e3, "d2h_csr_bytes_full": 8 * op.owned_tangent_pattern.nnz,
            "api": "ConstitutiveOperator.build_F_K_regularized_all_free(lam, U_host, r) + K.getValuesCSR()"}


def parity_check(torch, op, runner, U_host, U_dev):
    """Plain and mixed GPU outputs of one state against the oracle's on the same inputs (max-norm
    relative errors; comparisons on the device), the CSR pattern and the element -> CSR map bit for
    bit.  The oracle builds its own pattern, geometry and elastic values.

    Stage by stage as well: the strain against the oracle's strain, and the return mapping against
    the oracle's return mapping on the GPU's own strain.  And the oracle's own spread: the same
    restatement compiled without fused multiply-adds, whose outputs move by as much as a change of
    rounding in the strain moves them (the consistent tangent of a point whose principal strains
    nearly coincide amplifies last-bit differences of the strain, itself a sum with cancellation)."""
    from oracle import oracle_py as o
    from slope_stability_petsc4py_gb300.distributed_tangent import overlap_strain_device

    pat = op.owned_tangent_pattern
    t0 = time.perf_counter()
    ref = runner.step(U_host, LAMBDA, R_REG, DAVIS)
    oracle_s = time.perf_counter() - t0
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")  # noqa: E731

    def rel(a, b):
        scale = b.abs().max().clamp_min(1e-300)
        return float(((a - b).abs().max() / scale).item())

    K_o, F_o = dev(ref["K"]), dev(ref["F"][runner.free])
    S_o, DS_o = dev(ref["S"]), dev(ref["DS"])
    out = {"state": f"amplitude {STATE_FACTORS[1]:g} x, lambda {LAMBDA}, r {R_REG}", "oracle_step_s": oracle_s,
           "oracle_pattern_s": runner.pattern_s, "points": runner.n_int, "nnz": runner.nnz}
    out["indices_bit_exact"] = bool(np.array_equal(pat.local_matrix_pattern.indptr, runner.p["indptr"]) and
                                    np.array_equal(pat.local_matrix_pattern.indices, runner.p["indices"]))
    sm = pat.device["scatter_map"]
    p = runner.p
    nld = pat.dim * pat.n_p
    se = torch.as_tensor(p["slot_elem"].astype(np.int64), device="cuda")
    sl = torch.as_tensor(p["slot_lrow"].astype(np.int64), device="cuda")
    cols = sl[:, None] * nld + torch.arange(nld, device="cuda")[None, :]
    out["element_map_bit_exact"] = bool(torch.equal(sm[se[:, None], cols], dev(p["slot_pos"])))
    out["constrained_diagonals_bit_exact"] = bool(np.array_equal(pat.constrained_diag_positions,
                                                                 p["constrained_diag_positions"]))
    del se, sl, cols
    for form in ("plain", "mixed"):
        op.tangent_form = form
        F, K = op.build_F_K_regularized_all_free(LAMBDA, U_dev, R_REG)
        torch.cuda.synchronize()
        out[form] = {"S": rel(op._S_aos, S_o), "DS": rel(op._owned_local_DS.aos, DS_o), "F_free": rel(F, F_o),
                     "K": rel(K.values, K_o)}
        if form == "plain":
            E_g = overlap_strain_device(pat, U_dev)
            S_gE, DS_gE = runner.constitutive(E_g.cpu().numpy(), LAMBDA, DAVIS)
            out["stages"] = {"strain": rel(E_g, dev(ref["E"])),
                             "S_on_gpu_strain": rel(op._S_aos, dev(S_gE)),
                             "DS_on_gpu_strain": rel(op._owned_local_DS.aos, dev(DS_gE))}
            del E_g, S_gE, DS_gE
    op.tangent_form = "plain"
    if runner.dim == 3:
        nf = runner.step(U_host, LAMBDA, R_REG, DAVIS, library=o.nofma_lib())
        out["oracle_without_fma"] = {k: rel(dev(nf[k2]), v) for k, k2, v in (
            ("strain", "E", dev(ref["E"])), ("S", "S", S_o), ("DS", "DS", DS_o), ("K", "K", K_o))}
        del nf
    spread = out.get("oracle_without_fma", {}).get("DS", 0.0)
    out["tolerance"] = {"plain": "1e-12 max-norm relative: strain, S, F_free, K, and DS on the same strain; "
                                 "DS end to end within max(1e-12, the oracle's own spread without FMA)",
                        "mixed": "1e-6 tangent (K), 1e-11 force (F_free)"}
    out["pass"] = bool(out["indices_bit_exact"] and out["element_map_bit_exact"] and
                       out["constrained_diagonals_bit_exact"] and
                       all(out["plain"][k] <= 1e-12 for k in ("S", "F_free", "K")) and
                       out["plain"]["DS"] <= max(1e-12, spread) and
                       all(v <= 1e-12 for v in out["stages"].values()) and
                       out["mixed"]["K"] <= 1e-6 and out["mixed"]["F_free"] <= 1e-11)
    del K_o, F_o, S_o, DS_o
    return out


def measure_workload(torch, lib, w, args, *, headline):
    """Build the operator of workload w and measure it.  headline: the full set of figures of the
    bench line; otherwise the summary of an other configuration (plain, mixed, the proposal forms on
    3D P4, and parity against the oracle)."""
    from slope_stability_petsc4py_gb300 import ConstitutiveOperator

    mesh = w.mesh
    t0 = time.perf_counter()
    op = ConstitutiveOperator.from_mesh(mesh.coord, mesh.elem, mesh.q_mask, mesh.material_id, w.specs,
                                        elem_type=mesh.elem_type)
    setup_s = time.perf_counter() - t0
    pat = op.owned_tangent_pattern
    states_host = timed_states(w)
    states_dev = [torch.as_tensor(U, device="cuda") for U in states_host]
    op.host_outputs = False
    res = SimpleNamespace(op=op, states_host=states_host, states_dev=states_dev, setup_s=setup_s)
    if headline:
        return res
    wu = max(args.warmup, 3)
    step = make_step(op, states_dev)
    out = {"workload": describe(w.name, mesh, pat.n_local_int, pat.nnz), "setup_s": setup_s}
    for name, form, mapping in (("plain", "plain", "binned"), ("mixed", "mixed", "binned")):
        if mesh.dim == 2 and form == "mixed":
            continue
        op.tangent_form, op.return_mapping = form, mapping
        ms = time_steps(torch, step, wu, args.steps)
        out[name] = {"value": pat.n_local_int / (ms * 1e-3), "ms_per_step": ms}
    if mesh.dim == 3 and mesh.elem_type == "P4":  # the learned form's configuration
        out["learned_training"] = train_branch_model(torch, op, w)
        for name, form, mapping in (("mixed+learned", "mixed", "learned"), ("mixed+previous", "mixed", "previous"),
                                    ("plain+unsorted", "plain", "unsorted"), ("plain+learned", "plain", "learned"),
                                    ("plain+previous", "plain", "previous")):
            op.tangent_form, op.return_mapping = form, mapping
            ms = time_steps(torch, step, wu, args.steps)
            out[name] = {"value": pat.n_local_int / (ms * 1e-3), "ms_per_step": ms,
                         "speedup_vs_plain": out["plain"]["ms_per_step"] / ms}
    op.tangent_form, op.return_mapping = "plain", "binned"
    if "mixed" in out:
        out["mixed"]["speedup_vs_plain"] = out["plain"]["ms_per_step"] / out["mixed"]["ms_per_step"]
    if not args.no_parity:
        runner = oracle_runner(w)
        out["parity"] = parity_check(torch, op, runner, states_host[1], states_dev[1])
        del runner
    lib.raise_on_device_status()
    return out


def run_gpu(args):
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    w = workload(args.config)
    res = measure_workload(torch, _lib, w, args, headline=True)
    op, states_dev, states_host = res.op, res.states_dev, res.states_host
    pat = op.owned_tangent_pattern
    n_int, nnz = pat.n_local_int, pat.nnz
    op.tangent_form = args.form
    learned_info = None
    if args.return_mapping == "learned":
        learned_info = train_branch_model(torch, op, w)
    op.return_mapping = args.return_mapping
    step = make_step(op, states_dev)
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

    kernels, plastic = kernel_profile(torch, _lib, op, states_dev)
    stats = workload_stats(op, plastic)
    stats["moments"] = any(k.startswith("ssp_tangent_plastic_correction_p2_moments") for k in kernels)
    hbm_peak, hbm_src = peaks()
    fp64_tf = fp64_peak(torch)
    dominant = max(kernels, key=lambda k: kernels[k]["ms_per_step"])
    alg = algorithmic(dominant, stats)
    k_ms = kernels[dominant]["ms_per_launch"]
    achieved_gbs = alg["bytes"] / (k_ms * 1e-3) / 1e9
    rooflines = {}
    for name, kv in kernels.items():
        a = algorithmic(name, stats)
        if a["bytes"]:
            t_s = kv["ms_per_launch"] * 1e-3
            rooflines[name] = {"achieved_gbs": a["bytes"] / t_s / 1e9, "frac_hbm": a["bytes"] / t_s / 1e9 / hbm_peak,
                               "fp64_tflops": a["fp64"] / t_s / 1e12, "frac_fp64": a["fp64"] / t_s / 1e12 / fp64_tf}
    line = {
        "metric": METRIC, "value": world * n_int / (ms * 1e-3), "unit": "quad-pts/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.form == "plain" else "f64 (FP32 tangent products)",
        "data": "synthetic",
        "config": bench_config(w, n_int, nnz),
        "gpu_form": {"form": args.form, "return_mapping": args.return_mapping,
                     "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                     "plastic_points_per_state": [p["n_plastic"] for p in plastic],
                     "plastic_elements_per_state": [p["n_plastic_el"] for p in plastic],
                     "plastic_fraction": stats["n_plastic"] / n_int,
                     "device_pattern_bytes": stats["device_bytes"], "setup_s": res.setup_s},
        "assembled_nnz_per_s": world * nnz / (ms * 1e-3),
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved_gbs / hbm_peak, "peak_source": hbm_src,
                     "traffic": NCU_TRAFFIC.get(args.config, {}).get(dominant, (None, None))[0],
                     "traffic_source": NCU_TRAFFIC.get(args.config, {}).get(dominant, (None, "not captured"))[1],
                     "ms_per_launch": k_ms, "algorithmic_bytes": alg["bytes"],
                     "units": alg.get("units")},
        "roofline_fp64": {"bound": "fp64", "kernel": dominant, "achieved": alg["fp64"] / (k_ms * 1e-3) / 1e12,
                          "peak": fp64_tf, "unit": "TFLOP/s", "frac": alg["fp64"] / (k_ms * 1e-3) / 1e12 / fp64_tf,
                          "peak_source": "measured live (bench-only FP64 FMA probe)",
                          "executed_fp64_flops": alg["fp64"], "algorithmic_flops": alg["flops"]},
        "kernel_rooflines": rooflines,
        "kernels": kernels,
        "host_enqueue_ms_per_step": host_ms,
        "gpu_launches": launches,
        "clocks": clock_info,
    }
    if learned_info is not None:
        line["learned"] = learned_info

    rich = args.form == "plain" and args.return_mapping == "binned"
    if rich and pat.dim == 3 and not args.no_forms:
        line["forms"] = compare_forms(torch, _lib, op, w, states_dev, args, ms)
        line["new_lambda_r"] = measure_new_lambda_r(torch, _lib, op, states_dev)
    if rich and pat.dim == 3 and not args.no_ssr:
        line["ssr_sequence"] = measure_ssr(torch, _lib, op, w)
    if args.bddc:
        line["bddc"] = measure_bddc(torch, _lib, op, w, states_dev, args)
    if rich and not args.no_forms:
        line["graph_replay"] = measure_graph_replay(torch, _lib, op, states_dev, args)
    if rank == 0 and not args.no_e2e:
        line["e2e"] = measure_e2e(torch, op, states_host, args, args.form)
        if rich and pat.dim == 3 and not args.no_forms:
            line["e2e"]["mixed"] = measure_e2e(torch, op, states_host, args, "mixed")
    if rank == 0 and not args.no_parity:
        runner = oracle_runner(w)
        line["parity"] = parity_check(torch, op, runner, states_host[1], states_dev[1])
        del runner
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_reference_figures(w, steps=5, warmup=1, budget_s=30.0)
    del op, res, states_dev
    torch.cuda.empty_cache()
    if rank == 0 and not args.no_others and args.config == DEFAULT_CONFIG and args.form == "plain":
        line["other_workloads"] = {}
        for name in OTHER_WORKLOADS:
            ow = workload(name)
            line["other_workloads"][name] = measure_workload(torch, _lib, ow, args, headline=False)
            torch.cuda.empty_cache()
    if dist is not None:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


def run_reference(args):
    """The reference arm: the oracle's restatement of the reference's kernels on the host cores,
    every host thread, one bounded sample of the workload per step (same states)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle_py as o
    from oracle.newton_step import OracleNewtonStep
    from slope_stability_petsc4py_gb300 import fem

    w = workload(args.config)
    n_q = len(fem.quadrature(w.mesh.dim, w.mesh.elem_type)[1])
    sub, states = cpu_sample(w, SAMPLE_POINTS, n_q)
    runner = OracleNewtonStep(sub, w.specs)
    times = runner.time_steps(states, args.steps, args.warmup, LAMBDA, R_REG)
    t = float(np.median(times))
    value = runner.n_int / t
    n_int = w.mesh.n_elem * n_q
    full = runner if sub is w.mesh else None
    nnz_full = full.nnz if full is not None else \
        int(o.owned_pattern_c(w.mesh.elem, w.mesh.q_mask, (0, w.mesh.n_nodes))["indices"].size)
    threads = o.num_threads()
    line = {"metric": METRIC, "value": value, "unit": "quad-pts/s", "n_gpus": world, "steps": len(times),
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": bench_config(w, n_int, nnz_full),
            "cpu_baseline": {"value": value, "unit": "quad-pts/s", "cores": threads, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": sample_text(w, sub, runner, len(times), args.warmup, threads)},
            "e2e": {"value": value, "unit": "quad-pts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "setup_s": {"pattern": runner.pattern_s, "geometry": runner.geometry_s, "elastic_values": runner.elastic_s}}
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
