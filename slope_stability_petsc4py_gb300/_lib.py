"""ctypes binding of ``_build/libssp_gb300.so`` (the C ABI of ``include/ssp_gb300.h``).

There is no CPU fallback: if the library is missing or fails to load, every entry point of this
package raises.  Device buffers are torch CUDA tensors; only their raw pointers and the raw
``cudaStream_t`` of torch's current stream cross the boundary.
"""

from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

from . import build as _build

_LIB = None
# SSP_POTENTIAL_PARTIALS of the header: the block partials ssp_potential_energy needs as scratch
POTENTIAL_PARTIALS = 1024
_c_int, _c_ll, _c_dbl, _vp = ctypes.c_int, ctypes.c_longlong, ctypes.c_double, ctypes.c_void_p

# ssp_constitutive_3d_sds_screened: binning sources and option bits (include/ssp_gb300.h)
BINS_EXACT, BINS_LEARNED, BINS_GIVEN = 0, 1, 2
RM_COMPENSATED_DS, RM_PLASTIC_DS_ONLY = 1, 2

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "unsupported element", 4: "int32 overflow",
          5: "pattern is missing a structural entry", 6: "more points than the fixed scratch holds"}

_SIGS = {
    "ssp_constitutive_3d_s": [_vp] * 6 + [_c_int, _vp, _vp],
    "ssp_constitutive_3d_sds": [_vp] * 6 + [_c_int, _vp, _vp, _vp],
    "ssp_constitutive_3d_branch": [_vp] * 5 + [_c_int, _vp, _vp, _vp],
    "ssp_constitutive_2d": [_vp] * 6 + [_c_int, _vp, _vp, _vp],
    "ssp_potential_energy": [_c_int] + [_vp] * 7 + [_c_int] + [_vp] * 5,
    "ssp_assemble_overlap_strain_3d_p2_affine": [_vp] * 3 + [_c_int, _vp, _c_int, _c_int, _c_int, _vp, _vp],
    "ssp_assemble_overlap_strain_3d_affine": [_vp] * 3 + [_c_int, _vp, _c_int, _c_int, _c_int, _c_int, _vp, _vp],
    "ssp_assemble_force_element_affine": [_vp] * 5 + [_c_int] * 4 + [_vp, _vp],
    "ssp_assemble_force_element_p2_affine": [_vp] * 5 + [_c_int, _c_int, _c_int, _vp, _vp],
    "ssp_assemble_overlap_strain_3d_p2_affine_mixed": [_vp] * 3 + [_c_int, _vp, _c_int, _c_int, _c_int, _vp, _vp],
    "ssp_assemble_force_element_p2_affine_mixed": [_vp] * 5 + [_c_int, _c_int, _c_int, _vp, _vp],
    "ssp_host_writable": [_vp],
    "ssp_copy_out": [_vp, _c_ll, _vp, _vp],
    "ssp_copy_device": [_vp, _c_ll, _vp, _vp],
    "ssp_copy_rows_device": [_vp, _vp, _vp, _c_int, _c_ll, _vp, _vp],
    "ssp_copy_rows_device_share": [_vp, _vp, _vp, _c_int, _c_ll, _vp, _c_int, _vp],
    "ssp_mark_element_rows": [_vp, _c_int, _c_int, _vp, _vp, _c_int, _vp, _vp],
    "ssp_copy_rows_out": [_vp, _vp, _vp, _c_int, _c_ll, _vp, _vp],
    "ssp_copy_rows_out_share": [_vp, _vp, _vp, _c_int, _c_ll, _vp, _c_int, _vp],
    "ssp_tc_tf32_probe": [_vp, _vp, _c_int, _c_int, _vp, _vp],
    "ssp_tc_wait_probe": [_c_ll, _vp, _vp],
    "ssp_constitutive_sds_branch": [_c_int] + [_vp] * 5 + [_c_int, _vp, _vp, _vp, _vp],
    "ssp_constitutive_3d_sds_binned": [_vp] * 5 + [_c_int, _vp, _vp, _vp, _vp, _vp],
    "ssp_constitutive_3d_sds_binned_mixed": [_vp] * 5 + [_c_int, _vp, _vp, _vp, _vp, _vp],
    "ssp_constitutive_3d_sds_binned_noalloc": [_vp] * 5 + [_c_int, _vp, _vp, _vp, _vp],
    "ssp_tangent_plastic_correction": [_c_int] + [_vp] * 8 + [_vp, _c_int, _c_int, _c_int, _c_ll, _c_dbl, _vp, _vp, _vp,
                                       _vp],
    "ssp_plastic_elements": [_vp, _c_int, _c_int, _vp, _vp, _vp],
    "ssp_plastic_elements_split": [_vp, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp],
    "ssp_tangent_plastic_correction_p2_moments": [_vp] * 8 + [_c_int, _c_int, _c_ll, _c_dbl, _vp, _vp, _vp, _vp],
    "ssp_tangent_plastic_correction_p2_moments_mixed": [_vp] * 8 + [_c_int, _c_int, _c_ll, _c_dbl, _vp, _vp, _vp,
                                                                    _vp],
    "ssp_tangent_plastic_correction_mixed": [_c_int] + [_vp] * 8 + [_vp, _c_int, _c_int, _c_int, _c_ll, _c_dbl, _vp,
                                             _vp, _vp, _vp],
    "ssp_elastic_tangent_blocks": [_c_int, _vp, _vp, _c_int, _vp, _vp],
    "ssp_blend_values": [_vp, _vp, _vp, _c_dbl, _c_ll, _vp],
    "ssp_reduction": [_vp, _vp, _vp, _c_int, _c_dbl, ctypes.c_char, _vp, _vp, _vp],
    "ssp_geometry": [_c_int, _vp, _vp, _vp, _vp, _c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp],
    "ssp_assemble_overlap_strain_3d": [_vp, _vp, _vp, _vp, _c_int, _vp, _c_int, _c_int, _c_int, _c_int, _vp, _vp],
    "ssp_assemble_overlap_strain_2d": [_vp, _vp, _vp, _c_int, _vp, _c_int, _c_int, _c_int, _c_int, _vp, _vp],
    "ssp_assemble_force_3d_rows": [_vp] * 8 + [_c_int] * 6 + [_vp, _vp],
    "ssp_assemble_force_element": [_c_int] + [_vp] * 6 + [_c_int] * 4 + [_vp, _vp],
    "ssp_assemble_overlap_strain_3d_mixed": [_vp, _vp, _vp, _vp, _c_int, _vp, _c_int, _c_int, _c_int, _c_int, _vp, _vp],
    "ssp_assemble_force_element_mixed": [_vp] * 5 + [_c_int] * 4 + [_vp, _vp],
    "ssp_constitutive_2d_sds_binned": [_vp] * 5 + [_c_int] + [_vp] * 5,
    "ssp_assemble_overlap_strain_3d_affine_mixed": [_vp, _vp, _vp, _c_int, _vp, _c_int, _c_int, _c_int, _c_int, _vp, _vp],
    "ssp_assemble_force_element_affine_mixed": [_vp] * 5 + [_c_int] * 4 + [_vp, _vp],
    "ssp_split_f64": [_vp, _vp, _c_ll, _c_int, _vp, _vp],
    "ssp_assemble_tangent_values_3d_rows": [_vp] * 9 + [_c_int] * 6 + [_vp, _vp],
    "ssp_assemble_tangent_values_3d_p2": [_vp] * 6 + [_c_int] * 5 + [_vp, _vp],
    "ssp_tangent_element": [_c_int, _c_int] + [_vp] * 6 + [_c_int, _c_int, _c_int, _c_ll, _vp, _c_int, _vp],
    "ssp_finish_values": [_vp, _c_ll, _vp, _c_int, _vp, _c_dbl, _vp],
    "ssp_gather": [_vp, _vp, _c_int, _vp, _vp],
    "ssp_device_status": [ctypes.POINTER(_c_int), _c_int],
    "ssp_branch_features": [_vp] * 5 + [_c_int, _vp, _vp],
    "ssp_mlp_predict": [_vp, _vp, _c_int, _c_int, _vp, _vp],
    "ssp_mlp_loss_grad": [_vp, _vp, _vp, _c_int, _vp, _vp, _vp, _vp],
    "ssp_mlp_adam": [_vp, _vp, _vp, _vp, _c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                     ctypes.c_float, _vp],
    "ssp_constitutive_3d_sds_learned": [_vp] * 6 + [_c_int, _vp, _vp, _vp, _vp, _vp],
    "ssp_constitutive_3d_sds_learned_mixed": [_vp] * 6 + [_c_int, _vp, _vp, _vp, _vp, _vp],
    "ssp_constitutive_3d_sds_proposed": [_vp] * 6 + [_c_int, _vp, _vp, _vp, _vp, _vp],
    "ssp_constitutive_3d_sds_screened": [_vp] * 5 + [_c_int, _vp, _vp, _vp, _vp, _c_int, _vp, _c_int, _vp],
    "ssp_fill_elastic_ds": [_c_int, _vp, _vp, _vp, _c_int, _vp, _vp],
    "ssp_constitutive_3d_sds_proposed_mixed": [_vp] * 6 + [_c_int, _vp, _vp, _vp, _vp, _vp],
    "ssp_pattern_build": [_c_int, _c_int, _c_int, _c_int, _vp, _vp, _c_int, _c_int, ctypes.POINTER(_vp)],
    "ssp_pattern_sizes": [_vp, _vp],
    "ssp_pattern_copy": [_vp, ctypes.c_char_p, _vp],
    "ssp_pattern_free": [_vp],
}


class SSPError(RuntimeError):
    """A C-ABI call returned a non-zero ssp_status or a kernel flagged a bad index."""


def library_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed and possible) the sm_103a library; raise if impossible."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not path.exists() or os.environ.get("SSP_FORCE_REBUILD"):
        if not build_if_missing:
            raise ImportError(f"CUDA library {path} is not built; run __graft_entry__.build()")
        _build.build()
    lib = ctypes.CDLL(str(path))
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = None if name == "ssp_pattern_free" else _c_int
    _LIB = lib
    return lib


def exported_symbols() -> list[str]:
    return sorted(_SIGS)


def check(status: int, what: str) -> None:
    if status != 0:
        raise SSPError(f"{what} failed: {STATUS.get(int(status), status)}")


# kernels each entry point launches per call (for launch accounting); callables take the args
_KERNELS_PER_CALL = {
    "ssp_constitutive_3d_s": 1, "ssp_constitutive_3d_sds": 1, "ssp_constitutive_3d_branch": 1,
    "ssp_constitutive_2d": 1, "ssp_reduction": 1, "ssp_geometry": 1, "ssp_assemble_overlap_strain_3d": 1,
    "ssp_assemble_overlap_strain_2d": 1, "ssp_assemble_force_3d_rows": 1, "ssp_assemble_force_element": 1,
    "ssp_assemble_tangent_values_3d_rows": 1, "ssp_assemble_tangent_values_3d_p2": 1, "ssp_tangent_element": 1,
    "ssp_gather": 1, "ssp_tc_tf32_probe": 1, "ssp_tc_wait_probe": 1, "ssp_constitutive_sds_branch": 1,
    "ssp_copy_out": 1, "ssp_copy_device": 1, "ssp_copy_rows_device": 1, "ssp_copy_rows_device_share": 1, "ssp_host_writable": 0, "ssp_plastic_elements": 1, "ssp_mark_element_rows": 1,
    "ssp_copy_rows_out": 1, "ssp_copy_rows_out_share": 1,
    "ssp_assemble_overlap_strain_3d_mixed": 1, "ssp_assemble_force_element_mixed": 1, "ssp_split_f64": 1,
    "ssp_assemble_overlap_strain_3d_affine_mixed": 1, "ssp_assemble_force_element_affine_mixed": 1,
    "ssp_assemble_overlap_strain_3d_p2_affine": 1, "ssp_assemble_force_element_p2_affine": 1,
    "ssp_assemble_overlap_strain_3d_affine": 1, "ssp_assemble_force_element_affine": 1,
    "ssp_assemble_overlap_strain_3d_p2_affine_mixed": 1, "ssp_assemble_force_element_p2_affine_mixed": 1,
    "ssp_constitutive_2d_sds_binned": 2,
    "ssp_tangent_plastic_correction": 1, "ssp_plastic_elements_split": 1,
    "ssp_tangent_plastic_correction_p2_moments": 1, "ssp_tangent_plastic_correction_p2_moments_mixed": 1,
    "ssp_constitutive_3d_sds_binned": 3, "ssp_constitutive_3d_sds_binned_noalloc": 3,
    "ssp_constitutive_3d_sds_binned_mixed": 3, "ssp_constitutive_3d_sds_learned_mixed": 4,
    "ssp_tangent_plastic_correction_mixed": 1, "ssp_branch_features": 1, "ssp_mlp_predict": 1,
    "ssp_mlp_loss_grad": 1, "ssp_mlp_adam": 1, "ssp_constitutive_3d_sds_learned": 4,
    "ssp_constitutive_3d_sds_proposed": 4, "ssp_constitutive_3d_sds_proposed_mixed": 4,
    "ssp_constitutive_3d_sds_screened": lambda a: 3 if a[10] == 0 else 4, "ssp_fill_elastic_ds": 1,
    "ssp_elastic_tangent_blocks": 1, "ssp_blend_values": 1,
    "ssp_finish_values": lambda a: int(bool(a[3])) + int(a[4] is not None),
    "ssp_potential_energy": lambda a: int(a[8] > 0) + int(a[12] is not None),
}
LAUNCHES = {"count": 0}
# When set to a list, every kernel-launching call appends (name, start_event, end_event), recorded
# on torch's current stream (the stream the kernels run on).  Used by the benchmark's per-kernel
# timing; None (the default) adds no work.
TRACE = None


def call(name: str, *args) -> None:
    k = _KERNELS_PER_CALL.get(name, 0)
    n_k = k(args) if callable(k) else k
    if TRACE is not None and n_k:
        t = torch()
        e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
        e0.record()
        check(getattr(load(), name)(*args), name)
        e1.record()
        TRACE.append((name, e0, e1))
    else:
        check(getattr(load(), name)(*args), name)
    LAUNCHES["count"] += n_k


def host_writable(ptr_value) -> bool:
    """True if kernels can store to this host address directly (pinned, device-mapped memory)."""
    return bool(load().ssp_host_writable(ptr_value))


def device_status(clear: bool = True) -> int:
    v = _c_int(0)
    check(load().ssp_device_status(ctypes.byref(v), 1 if clear else 0), "ssp_device_status")
    return int(v.value)


def raise_on_device_status() -> None:
    st = device_status(clear=True)
    if st:
        raise SSPError(f"a kernel flagged invalid input (device status {st:#x})")


# ----------------------------------------------------------------------------- torch helpers


def torch():
    import torch as _t

    return _t


def ptr(t) -> int | None:
    """Raw device pointer of a contiguous CUDA tensor (None passes NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise SSPError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise SSPError("expected a contiguous tensor")
    return t.data_ptr()


def stream_handle() -> int:
    return torch().cuda.current_stream().cuda_stream


def require_cuda():
    t = torch()
    if not t.cuda.is_available():
        raise SSPError("no CUDA device: the GB300 hot path has no CPU fallback")
    load()
    return t


def to_device(a, dtype=None):
    """numpy / torch -> contiguous CUDA tensor (no copy if already there with that dtype)."""
    t = torch()
    if isinstance(a, t.Tensor):
        out = a
        if dtype is not None and out.dtype != dtype:
            out = out.to(dtype)
        if not out.is_cuda:
            out = out.cuda()
        return out.contiguous()
    arr = np.ascontiguousarray(a)
    out = t.from_numpy(arr)
    if dtype is not None:
        out = out.to(dtype)
    return out.cuda(non_blocking=False).contiguous()
