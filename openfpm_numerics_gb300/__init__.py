"""GB300-native DC-PSE hot path of openfpm_numerics.

Kernel assembly (per-particle moment systems solved in FP64 on the device)
and operator application (batched gather-weighted sums over CSR neighbour
lists) as hand-written sm_103a CUDA behind a C-ABI
(include/openfpm_dcpse/dcpse_capi.h).  This package is the Python host side:
``plan.DcpsePlan`` mirrors the C-ABI, ``operators`` mirrors the reference's
DCPSE_op.hpp operator objects.
"""
from . import _capi  # noqa: F401
from .plan import DcpsePlan  # noqa: F401
from .operators import (  # noqa: F401
    Derivative_G, Derivative_x, Derivative_xx, Derivative_xxx, Derivative_xxxx, Derivative_xxy,
    Derivative_xxyy, Derivative_xy, Derivative_xz, Derivative_y, Derivative_yy, Derivative_yyx,
    Derivative_yyy, Derivative_yyyy, Derivative_yz, Derivative_z, Derivative_zz, Gradient, Laplacian,
    OperatorSet, ParticleSet, VerletList, support_options,
)


def load():
    """Build (if needed) and load the CUDA extension; raises if unavailable."""
    return _capi.load()
