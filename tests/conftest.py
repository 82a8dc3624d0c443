"""Shared test helpers.  GPU tests are marked ``gpu``; everything else runs on the CPU."""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
GOLDEN = REPO / "tests" / "golden"
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

# Parity tolerance of the plain FP64 path: max-norm relative error against the oracle /
# reference output on the same inputs.
PLAIN_RTOL = 1.0e-12


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on a GB300)")


def golden(name: str) -> dict:
    with np.load(GOLDEN / name, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def golden_files(prefix: str) -> list[str]:
    return sorted(p.name for p in GOLDEN.glob(f"{prefix}*.npz"))


def rel_err(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    if a.size == 0:
        return 0.0
    scale = max(float(np.max(np.abs(b))), 1.0e-300)
    return float(np.max(np.abs(a - b))) / scale


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle_py

    oracle_py.build()
    return oracle_py


@pytest.fixture(scope="session")
def cuda_device():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
