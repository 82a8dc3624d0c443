"""The reference arm of bench.py on the host (no GPU): the oracle's restatement of the reference's
kernels timed on a small workload, printing the result line the GPU arm prints, with the same
metric and the same config (the two arms build it with the same function), plus its own
cpu_baseline and an e2e block with no host-device copies.  Under torchrun only rank 0 prints."""

from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]


def _run(extra_env=None):
    env = dict(os.environ)
    env.update(extra_env or {})
    cmd = [sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--config", "2d_p2_homo",
           "--steps", "2", "--warmup", "1"]
    return subprocess.run(cmd, cwd=REPO, env=env, capture_output=True, text=True, timeout=600)


@pytest.fixture(scope="module")
def oracle_built():
    from oracle import oracle_py

    oracle_py.build()


def test_reference_arm_prints_the_result_line(oracle_built):
    out = _run()
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [line for line in out.stdout.splitlines() if line.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    sys.path.insert(0, str(REPO))
    import bench
    from slope_stability_petsc4py_gb300 import fem

    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "quad-pts/s"
    assert d["higher_is_better"] is True and d["n_gpus"] == 1 and d["steps"] == 2 and d["warmup"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "quad-pts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the same config dict as the GPU arm's line
    w = bench.workload("2d_p2_homo")
    n_int = w.mesh.n_elem * len(fem.quadrature(w.mesh.dim, w.mesh.elem_type)[1])
    from oracle import oracle_py as o

    nnz = int(o.owned_pattern_c(w.mesh.elem, w.mesh.q_mask, (0, w.mesh.n_nodes))["indices"].size)
    assert d["config"] == bench.bench_config(w, n_int, nnz)


def test_reference_arm_other_ranks_print_nothing(oracle_built):
    out = _run({"RANK": "1", "WORLD_SIZE": "2"})
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip() == ""


def test_correction_accounting_splits_the_plastic_elements():
    """bench.algorithmic charges the FP64 moment kernel with the elements at or above the split and
    the point-by-point kernel with the others: units add up to the plastic elements, FP64 work to
    7,530 per element + 261 per plastic point on one side and 1,935 per plastic point on the other."""
    sys.path.insert(0, str(REPO))
    import bench

    st = {"n": 22_360_800, "n_el": 2_032_800, "n_p": 10, "n_q": 11, "dim": 3, "ns": 6, "nnz": 690_405_587,
          "n_rows": 8_000_000, "n_plastic": 2_600_000.0, "n_plastic_el": 300_000.0,
          "n_many_el": 240_000.0, "n_plastic_many": 2_300_000.0, "moments": True}
    mom = bench.algorithmic("ssp_tangent_plastic_correction_p2_moments", st)
    pt = bench.algorithmic("ssp_tangent_plastic_correction", st)
    per_el = mom["bytes"] / st["n_many_el"]
    assert abs(pt["bytes"] - per_el * (st["n_plastic_el"] - st["n_many_el"])) < 1e-3 * pt["bytes"]
    assert mom["fp64"] == 2.0 * (7530 * 240_000 + 261 * 2_300_000)
    assert pt["fp64"] == 2.0 * 1935 * (2_600_000 - 2_300_000)
    mixed = bench.algorithmic("ssp_tangent_plastic_correction_p2_moments_mixed", st)
    assert mixed["fp64"] == 2.0 * 22 * 2_300_000
    without = bench.algorithmic("ssp_tangent_plastic_correction", dict(st, moments=False))
    assert without["fp64"] == 2.0 * 1935 * 2_600_000
