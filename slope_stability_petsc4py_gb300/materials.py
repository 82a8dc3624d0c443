"""Material specification and per-integration-point expansion.

Mirrors ``MaterialSpec`` and ``heterogenous_materials`` of
``src/slope_stability/mesh/materials.py:10-101`` (same field names, same derived moduli, same
errors), so material inputs written for the reference load unchanged.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class MaterialSpec:
    c0: float
    phi: float  # degrees
    psi: float  # degrees
    young: float
    poisson: float
    gamma_sat: float
    gamma_unsat: float

    @property
    def shear(self) -> float:
        return self.young / (2.0 * (1.0 + self.poisson))

    @property
    def bulk(self) -> float:
        return self.young / (3.0 * (1.0 - 2.0 * self.poisson))

    @property
    def lame(self) -> float:
        return self.bulk - 2.0 * self.shear / 3.0


def _as_specs(materials) -> list[MaterialSpec]:
    if isinstance(materials, (dict, MaterialSpec)):
        materials = [materials]
    return [m if isinstance(m, MaterialSpec) else MaterialSpec(**m) for m in materials]


def heterogenous_materials(mat_identifier, saturation, n_q: int, materials):
    """Per-point (c0, phi[rad], psi[rad], shear, bulk, lame, gamma), each of length n_e * n_q."""
    specs = _as_specs(materials)
    mid = np.asarray(mat_identifier, dtype=np.int64).ravel()
    n_e = mid.size
    max_mid = int(mid.max()) if mid.size else -1
    if len(specs) == 1 and max_mid > 0:
        specs = specs * (max_mid + 1)
    if max_mid >= len(specs):
        raise IndexError(f"Material identifier {max_mid} requires at least {max_mid + 1} material rows, got {len(specs)}.")
    table = np.array([[s.c0, np.deg2rad(s.phi), np.deg2rad(s.psi), s.shear, s.bulk, s.lame, s.gamma_sat, s.gamma_unsat]
                      for s in specs], dtype=np.float64).reshape(-1, 8)
    per_elem = table[mid] if n_e else np.zeros((0, 8))
    per_pt = np.repeat(per_elem, n_q, axis=0)
    sat = np.asarray(saturation, dtype=bool).ravel()
    if sat.size != n_e * n_q:
        raise ValueError("saturation must have size n_e * n_q")
    gamma = np.where(sat, per_pt[:, 6], per_pt[:, 7])
    return tuple(np.ascontiguousarray(per_pt[:, k]) for k in range(6)) + (gamma,)
