"""GB300-native multishift Sternheimer solver (SternheimerGW's select_solver path).

The compute path is libsgw_gb300.so (hand-written sm_103a CUDA behind the C ABI
in include/sgw_capi.h).  Importing this package does not load it; the first
solver call does, and raises if it is missing.
"""
from .solver import (BICGSTAB_MULTI, BICGSTAB_NO_MULTI, SGW_LINEAR_SOLVER, BicgstabConfig, DenseOperator,
                     LinearSolverConfig, PlaneWaveOperator, SelectSolverConfig, bicgstab, host_array,
                     linear_solver, select_solver, solve_batch)
from ._capi import SgwError
from . import linter, solver

__all__ = ["BICGSTAB_MULTI", "BICGSTAB_NO_MULTI", "SGW_LINEAR_SOLVER", "BicgstabConfig", "DenseOperator",
           "LinearSolverConfig", "PlaneWaveOperator", "SelectSolverConfig", "bicgstab", "linear_solver",
           "select_solver", "solve_batch", "host_array", "SgwError", "solver", "linter"]
