"""GB300-native coupled SPH + wave-heightfield simulation step.

The product is libcwa.so (include/cwa.h): hand-written sm_103a CUDA kernels
behind a C ABI.  This package holds its in-tree build and a thin ctypes
mirror of the reference's step interface for Python callers.
"""
from ._abi import (CWA_OK, PARTICLE_DTYPE, PASSES, PREC_COMPENSATED, PREC_FP32, PREC_FP64,
                   PRESET_MULLER, PRESET_REFERENCE_3D, TOTALS, CwaError, SceneDesc, load)
from .sim import Sim, WaveModule

__all__ = [
    "CWA_OK", "PARTICLE_DTYPE", "PASSES", "PREC_COMPENSATED", "PREC_FP32", "PREC_FP64",
    "PRESET_MULLER", "PRESET_REFERENCE_3D", "TOTALS", "CwaError", "SceneDesc", "Sim", "WaveModule",
    "load",
]
