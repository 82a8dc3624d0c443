"""Device-resident arrays that still behave like the reference's NumPy outputs when asked.

The reference returns per-point fields as NumPy views of its C arrays, e.g. ``S`` as the
(6, n_int) transpose of a C-contiguous (n_int, 6) buffer (constitutive/problem.py:829-839).
Here the buffer stays in HBM; ``DeviceArray`` exposes the same shape and converts to NumPy only
when a caller asks (``np.asarray(x)``), so callers that never look at the values (Newton reads
only F and K) pay no device-to-host copy.
"""

from __future__ import annotations

import numpy as np


class DeviceArray:
    """A read-mostly view ``tensor.T`` of an AoS CUDA tensor of shape (n, k), shown as (k, n)."""

    __array_priority__ = 100

    def __init__(self, aos_tensor):
        self._t = aos_tensor  # (n, k) contiguous CUDA tensor

    @property
    def aos(self):
        """The underlying (n, k) CUDA tensor (the reference's C layout)."""
        return self._t

    @property
    def tensor(self):
        """(k, n) CUDA view, the reference's Python orientation."""
        return self._t.T

    @property
    def shape(self):
        n, k = self._t.shape
        return (k, n)

    @property
    def ndim(self):
        return 2

    @property
    def dtype(self):
        return np.float64

    @property
    def size(self):
        return int(self._t.numel())

    def numpy(self) -> np.ndarray:
        return self._t.detach().cpu().numpy().T

    def __array__(self, dtype=None, copy=None):
        a = self.numpy()
        return a.astype(dtype) if dtype is not None else a

    def __getitem__(self, idx):
        return self.numpy()[idx]

    def __len__(self):
        return self.shape[0]

    def __repr__(self):
        return f"DeviceArray(shape={self.shape}, device={self._t.device})"
