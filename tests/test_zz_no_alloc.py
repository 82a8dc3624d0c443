"""The no-allocation return-mapping entry point gives the allocating entry point's results.

``ssp_constitutive_3d_sds_binned_noalloc`` is for callers that cannot allocate device memory
(a constitutive hook inside another solver's assembly loop that only receives device pointers to
its inputs and outputs).  It keeps its point lists in a fixed array inside the library instead of
caller-provided scratch.  This file is collected last on purpose: a failure here comes after
every other test has run.  It passes alone in a fresh process as well as after the other tests.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import PLAIN_RTOL, golden, rel_err

pytestmark = pytest.mark.gpu


def _inputs(seed, n_random):
    rng = np.random.default_rng(seed)
    scales = np.repeat(np.array([1e-4, 1e-3, 3e-3]), n_random // 3)
    E = rng.standard_normal((scales.size, 6)) * scales[:, None]
    E = np.vstack([E, golden("constitutive_3d.npz")["E"]])
    n = E.shape[0]
    young, nu = rng.uniform(1.5e4, 3e4), rng.uniform(0.3, 0.49)
    shear = np.full(n, young / (2 * (1 + nu)))
    lame = np.full(n, young / (3 * (1 - 2 * nu))) - 2 * shear / 3
    phi = np.deg2rad(rng.uniform(25.0, 45.0))
    c_bar = np.full(n, 2.0 * 6.0 * np.cos(phi))
    sin_phi = np.full(n, np.sin(phi))
    return E, c_bar, sin_phi, shear, lame


def _run(entry, arrays, with_scratch):
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    lib = _lib.load()
    dev = [torch.as_tensor(np.ascontiguousarray(a), device="cuda") for a in arrays]
    n = dev[0].shape[0]
    S = torch.empty((n, 6), dtype=torch.float64, device="cuda")
    DS = torch.empty((n, 36), dtype=torch.float64, device="cuda")
    br = torch.empty(n, dtype=torch.int8, device="cuda")
    args = [t.data_ptr() for t in dev] + [n, S.data_ptr(), DS.data_ptr(), br.data_ptr()]
    if with_scratch:
        scratch = torch.empty(3 * n + 4, dtype=torch.int32, device="cuda")
        args.append(scratch.data_ptr())
    status = getattr(lib, entry)(*args, torch.cuda.current_stream().cuda_stream)
    assert status == 0, status
    torch.cuda.synchronize()
    return S.cpu().numpy(), DS.cpu().numpy(), br.cpu().numpy()


def test_noalloc_entry_point_matches_allocating_entry_point(cuda_device):
    # two calls in a row with different inputs: the shared fixed scratch keeps the first call's
    # lists, and the second call must not see them
    for seed, n_random in ((5, 90_000), (6, 30_000)):
        arrays = _inputs(seed, n_random)
        S_ref, DS_ref, b_ref = _run("ssp_constitutive_3d_sds_binned", arrays, with_scratch=True)
        S, DS, b = _run("ssp_constitutive_3d_sds_binned_noalloc", arrays, with_scratch=False)
        assert np.array_equal(b, b_ref)
        assert set(np.unique(b).tolist()) & {1, 2, 3}
        # the same kernels on the same grid, each point independent of the lists' order: bit for
        # bit, so a stale list entry left in the shared array by the previous call would show
        assert np.array_equal(S, S_ref) and np.array_equal(DS, DS_ref)


def test_noalloc_entry_point_matches_reference_outputs(cuda_device):
    """Directly against the reference's own C kernel outputs (golden fixture), twice in a row."""
    g = golden("constitutive_3d.npz")
    for tag in ("test_l1.3", "bench_l1.0"):
        arrays = (g["E"], g[f"{tag}_c_bar"], g[f"{tag}_sin_phi"], g[f"{tag}_shear"], g[f"{tag}_lame"])
        S, DS, _b = _run("ssp_constitutive_3d_sds_binned_noalloc", arrays, with_scratch=False)
        assert rel_err(S, g[f"{tag}_S_c"]) <= PLAIN_RTOL
        assert rel_err(DS, g[f"{tag}_DS_c"]) <= PLAIN_RTOL


def test_noalloc_entry_point_rejects_sizes_beyond_its_scratch(cuda_device):
    import torch

    from slope_stability_petsc4py_gb300 import _lib

    lib = _lib.load()
    max_points = 2097152  # SSP_NOALLOC_MAX_POINTS in include/ssp_gb300.h
    tiny = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = tiny.data_ptr()
    status = lib.ssp_constitutive_3d_sds_binned_noalloc(p, p, p, p, p, max_points + 1, p, p, p, None)
    assert status == 6  # SSP_ERR_TOO_LARGE, returned before any work
    assert lib.ssp_constitutive_3d_sds_binned_noalloc(p, p, p, p, p, -1, p, p, p, None) == 1
