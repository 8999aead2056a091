"""massivemds_gb300: a GB300-native (sm_103a) engine for the MassiveMDS
likelihood/gradient sweep.

The compute path is libmdsx.so (hand-written CUDA behind the C ABI in
include/mdsx.h); this package is its Python face, mirroring the reference's
engine interface and R API. There is no CPU fallback.
"""
from . import flags  # noqa: F401
from ._lib import MdsxError, load  # noqa: F401
from .engine import (  # noqa: F401
    Engine,
    MdsEngine,
    createEngine,
    factory,
    getGradient,
    getLogLikelihood,
    setPairwiseData,
    setPrecision,
    updateLocations,
)

__all__ = [
    "Engine", "MdsEngine", "MdsxError", "createEngine", "factory", "flags", "getGradient",
    "getLogLikelihood", "load", "setPairwiseData", "setPrecision", "updateLocations",
]
