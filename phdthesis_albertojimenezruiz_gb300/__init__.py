"""GB300-native sparse LU hot path of the PV-plant power-flow Newton iteration.

The product is the native library libpvglu.so (C ABI in include/pvglu.h):
host symbolic analysis plus sm_103a kernels for the Jacobian value scatter,
the GLU refactorization and the triangular solves.  This package is its
Python view; importing it loads the library and fails if it is missing.
"""
from . import _native
from ._native import (FP32, FP64, SCHED_LEVELS, SCHED_PERSISTENT, SCHED_THREAD_CHAIN,
                      PvgluError)
from .glu import Blocks, Numeric, Symbolic
from .newton import GMIN_STAGES, Newton, plant_power
from .plant import Plant

_native.lib()  # fail loudly at import when the native library is absent

__all__ = ["Blocks", "FP32", "FP64", "GMIN_STAGES", "SCHED_LEVELS", "SCHED_PERSISTENT",
           "SCHED_THREAD_CHAIN", "Newton", "Numeric", "PvgluError", "Plant", "Symbolic",
           "plant_power"]
