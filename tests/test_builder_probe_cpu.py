"""The builder surface the reference's Newton loop probes (no GPU).

Newton asks the constitutive builder for the matrix its preconditioner is built from by looking
the public BDDC builders up with ``getattr`` (``src/slope_stability/nonlinear/newton.py:188-206``)
and raises ``RuntimeError`` when none is found; the builders themselves raise
``RuntimeError("BDDC subdomain pattern not configured")`` without a subdomain pattern
(``src/slope_stability/constitutive/problem.py:2099-2112``).  The subdomain matrices are built by
the private builders (GPU; ``tests/test_gpu_bddc.py``); here they are replaced by stand-ins that
record the call, the way the reference's own tests inject dummy builders
(``tests/test_newton_cleanup.py:10-46``).
"""

from __future__ import annotations

import importlib
import os
import sys
from pathlib import Path
from unittest import mock

import numpy as np
import pytest


def _operator():
    from slope_stability_petsc4py_gb300 import ConstitutiveOperator

    z = np.zeros(4)
    return ConstitutiveOperator(B=None, c0=z, phi=z, psi=z, Davis_type="B", shear=z, bulk=z, lame=z, WEIGHT=z,
                                n_strain=6, n_int=4, dim=3)


def _with_recording_builders(op):
    calls = []
    op._build_bddc_tangent_matrix = lambda *, local_mat_type="aij": calls.append(("tangent", local_mat_type)) or "K_t"
    op._build_bddc_elastic_matrix = lambda *, local_mat_type="aij": calls.append(("elastic", local_mat_type)) or "K_e"
    op._build_bddc_regularized_matrix = (
        lambda r, *, local_mat_type="aij": calls.append(("regularized", r, local_mat_type)) or "K_r")
    return calls


def test_public_bddc_builders_raise_without_a_subdomain_pattern():
    op = _operator()
    for name, args in (("build_bddc_tangent_matrix", ()), ("build_bddc_regularized_matrix", (0.1,)),
                       ("build_bddc_elastic_matrix", ())):
        fn = getattr(op, name, None)
        assert callable(fn), name
        with pytest.raises(RuntimeError, match="BDDC subdomain pattern not configured"):
            fn(*args)


def test_public_bddc_builders_delegate_to_the_subdomain_builders():
    op = _operator()
    op.set_bddc_subdomain_pattern(object())
    calls = _with_recording_builders(op)
    assert op.build_bddc_tangent_matrix() == "K_t"
    assert op.build_bddc_regularized_matrix(0.25, local_mat_type="is") == "K_r"
    assert op.build_bddc_elastic_matrix(local_mat_type="aij") == "K_e"
    assert calls == [("tangent", "aij"), ("regularized", 0.25, "is"), ("elastic", "aij")]


def _reference_newton():
    root = os.environ.get("SSP_REFERENCE_ROOT")
    if not root or not (Path(root) / "src" / "slope_stability" / "nonlinear" / "newton.py").is_file():
        pytest.skip("SSP_REFERENCE_ROOT does not point at a reference checkout")
    sys.dont_write_bytecode = True
    for name in ("petsc4py", "petsc4py.PETSc", "mpi4py", "mpi4py.MPI", "h5py", "meshio", "matplotlib",
                 "matplotlib.pyplot", "pyvista"):
        sys.modules.setdefault(name, mock.MagicMock())
    src = str(Path(root) / "src")
    if src not in sys.path:
        sys.path.insert(0, src)
    return importlib.import_module("slope_stability.nonlinear.newton")


class _Solver:
    def __init__(self, source):
        self.source = source

    def get_preconditioner_matrix_source(self):
        return self.source


def test_reference_newton_finds_the_subdomain_matrices():
    """The reference's own _explicit_preconditioning_matrix, run against this package's operator."""
    newton = _reference_newton()
    op = _operator()
    op.set_bddc_subdomain_pattern(object())
    calls = _with_recording_builders(op)
    pick = newton._explicit_preconditioning_matrix
    assert pick(op, _Solver("elastic"), regularization_r=0.1) == "K_e"
    assert pick(op, _Solver("regularized"), regularization_r=0.1) == "K_r"
    assert pick(op, _Solver("tangent"), regularization_r=None) == "K_t"
    assert calls == [("elastic", "aij"), ("regularized", 0.1, "aij"), ("tangent", "aij")]
    # no subdomain pattern: the builder's RuntimeError reaches Newton, as with the reference's builder
    bare = _operator()
    with pytest.raises(RuntimeError, match="BDDC subdomain pattern not configured"):
        pick(bare, _Solver("tangent"), regularization_r=None)
