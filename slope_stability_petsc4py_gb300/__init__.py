"""GB300-native (sm_103a) Newton hot path of the slope-stability solver.

Drop-in replacements for the reference's constitutive builder and owned-row assembly:
``ConstitutiveOperator`` (constitutive/problem.py), ``prepare_owned_tangent_pattern`` and the
``assemble_*`` functions (fem/distributed_tangent.py), ``reduction`` (constitutive/reduction.py).
The arithmetic runs in hand-written CUDA kernels behind the C ABI of ``include/ssp_gb300.h``.
"""

from .bddc import (  # noqa: F401
    BDDCSubdomainPattern,
    assemble_bddc_subdomain_tangent_values,
    prepare_bddc_subdomain_pattern,
)
from .distributed_tangent import (  # noqa: F401
    DEFAULT_TANGENT_KERNEL,
    OwnedTangentPattern,
    assemble_overlap_strain,
    assemble_owned_force_from_local_stress,
    assemble_owned_regularized_matrix,
    assemble_owned_tangent_matrix,
    assemble_owned_tangent_values,
    prepare_owned_tangent_pattern,
)
from .materials import MaterialSpec, heterogenous_materials  # noqa: F401
from .problem import CapturedBuild, ConstitutiveOperator, OwnedCSRMatrix, SubdomainCSRMatrix  # noqa: F401
from .reduction import reduction  # noqa: F401

__version__ = "0.1.0"
