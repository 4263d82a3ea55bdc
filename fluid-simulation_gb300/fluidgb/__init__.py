"""fluidgb — GB300-native FLIP/PIC substep of fluid-lab behind a C ABI.

The compute path is libfluidgb.so (hand-written sm_103a CUDA, include/fluidgb.h);
this package is the ctypes binding plus seeded scene generators.
"""
from ._abi import (FL_CELL_AIR, FL_CELL_LIQUID, FL_CELL_SOLID, FL_CG_F32, FL_CG_F64, FL_CG_F64_IEEE, FL_INVALID_ARG, FL_OK,
                   FL_RELAX_JACOBI, FL_RELAX_RBGS, FL_SOLVER_CG, FL_SOLVER_FOLLOW, FL_SOLVER_MGPCG, FL_TIMEOUT,
                   FlGridView, FlParams, FlStats, Fluid, FluidError, LIB_PATH, SIGNATURES,
                   Timestep, default_params, face_counts, load_library, solve_pressure)
from . import scenes

__all__ = [
    "FL_CELL_AIR", "FL_CELL_LIQUID", "FL_CELL_SOLID", "FL_CG_F32", "FL_CG_F64", "FL_CG_F64_IEEE", "FL_INVALID_ARG", "FL_OK",
    "FL_RELAX_JACOBI", "FL_RELAX_RBGS", "FL_SOLVER_CG", "FL_SOLVER_FOLLOW", "FL_SOLVER_MGPCG", "FL_TIMEOUT",
    "FlGridView", "FlParams", "FlStats", "Fluid", "FluidError", "LIB_PATH", "SIGNATURES",
    "Timestep", "default_params", "face_counts", "load_library", "solve_pressure", "scenes",
]
