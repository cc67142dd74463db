"""emsolvers_gb300 — GB300-native time-domain Maxwell engine.

The compute path is libems.so (C++ host code and hand-written sm_103a CUDA
kernels behind the C ABI in include/ems.h).  This package is a thin ctypes
front end that mirrors the reference's solver classes.
"""
from ._lib import (ABM, FP32, FP64, LEAPFROG, SYMP2, SYMP4, WAVE_REFERENCE, WAVE_RICKER, EmsError,  # noqa: F401
                   declared_functions, lib)
from .solvers import (MISFIT_L2, MISFIT_TF_ENVELOPE, MISFIT_TF_PHASE, FdtdSimulation, FemStabSimulation,  # noqa: F401
                      HexFemSimulation, TetFemBatch, TetFemSimulation, tet_element_matrices, trace_misfit)

__all__ = ["FdtdSimulation", "HexFemSimulation", "FemStabSimulation", "TetFemSimulation", "TetFemBatch", "EmsError", "lib", "declared_functions",
           "FP32", "FP64", "LEAPFROG", "SYMP2", "SYMP4", "ABM", "WAVE_REFERENCE", "WAVE_RICKER", "trace_misfit",
           "MISFIT_L2", "MISFIT_TF_ENVELOPE", "MISFIT_TF_PHASE", "tet_element_matrices"]
