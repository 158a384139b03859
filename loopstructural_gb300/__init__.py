"""GB300-native (sm_103a) discrete implicit interpolation for LoopStructural.

Drop-in replacements for the reference's FiniteDifferenceInterpolator and
P1Interpolator (= PiecewiseLinearInterpolator) whose constraint assembly,
normal-equations CG solve and field evaluation run as hand-written CUDA
kernels behind the C ABI in include/ls_gb300.h.
"""
from . import constraints
from ._lib import ExtensionUnavailable, LsError
from .constraints import ValidationError
from .fold import FDFoldInterpolator
from .interpolators import FiniteDifferenceInterpolator
from .p1 import P1Interpolator, PiecewiseLinearInterpolator
from .regularisation import DirectionalRegularisation, RegularisationConfig
from .supports import StructuredGrid, TetMesh

__all__ = [
    "FiniteDifferenceInterpolator",
    "FDFoldInterpolator",
    "P1Interpolator",
    "PiecewiseLinearInterpolator",
    "StructuredGrid",
    "DirectionalRegularisation",
    "RegularisationConfig",
    "TetMesh",
    "ValidationError",
    "ExtensionUnavailable",
    "LsError",
    "constraints",
]


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile the sm_103a library in-tree; returns its path."""
    from . import _build

    return _build.build(verbose=verbose, force=force)
