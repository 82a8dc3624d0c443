"""Davis-type strength reduction on the GPU.

Same signature, semantics and errors as ``reduction`` in
``src/slope_stability/constitutive/reduction.py:14-78``: returns ``(c_bar, sin_phi)`` with
``c_bar = 2 c_lambda cos(phi_lambda)``.  NumPy inputs give NumPy outputs; CUDA tensors stay on
the device.
"""

from __future__ import annotations

import numpy as np

from . import _lib


def reduction(c0, phi, psi, lam: float, Davis_type: str = "A"):
    t = _lib.require_cuda()
    as_torch = isinstance(c0, t.Tensor)
    shapes = {tuple(np.shape(a)) for a in (c0, phi, psi)}
    if len(shapes) != 1:
        raise ValueError("c0, phi and psi must have the same shape")
    if lam <= 0:
        raise ValueError("Reduction parameter lambda must be positive")
    typ = str(Davis_type).upper()
    if typ not in ("A", "B", "C"):
        raise ValueError("Incorrect choice of the Davis approach")
    shape = shapes.pop()
    c, f, p = (_lib.to_device(a if as_torch else np.asarray(a, dtype=np.float64).reshape(-1), t.float64).reshape(-1)
               for a in (c0, phi, psi))
    n = int(c.numel())
    cb = t.empty(n, dtype=t.float64, device="cuda")
    sp = t.empty(n, dtype=t.float64, device="cuda")
    _lib.call("ssp_reduction", _lib.ptr(c), _lib.ptr(f), _lib.ptr(p), n, float(lam), typ.encode(), _lib.ptr(cb),
              _lib.ptr(sp), _lib.stream_handle())
    if as_torch:
        return cb.reshape(shape), sp.reshape(shape)
    return cb.cpu().numpy().reshape(shape), sp.cpu().numpy().reshape(shape)
