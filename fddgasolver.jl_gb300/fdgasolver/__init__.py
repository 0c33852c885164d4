"""fdgasolver: GB300 implementation of fdDGAsolver.jl's parquet-iteration hot path.

The numerics run in libfdga (C ABI, include/fdga.h; hand-written sm_103a kernels).  This package
is the host-side mirror of the reference's Julia API; it has no CPU compute path.
"""
from ._lib import FdgaError, lib_path, load
from .models import compute_occupation, hubbard_bare_Green, siam_bare_Green
from .solver import (NL_ParquetSolver, ParquetSolver, RefVertex, Vertex, fixed_point, fixed_point_preconditioned,
                     flatten, init_sym_grp, iterate_solver, mfRGLinearMap, parquet_solver_hubbard_parquet_approximation,
                     parquet_solver_siam_parquet_approximation, solve, solve_using_mfRG_without_mixing, unflatten)

__all__ = [
    "FdgaError", "lib_path", "load", "compute_occupation", "hubbard_bare_Green", "siam_bare_Green",
    "NL_ParquetSolver", "ParquetSolver", "RefVertex", "Vertex", "fixed_point", "flatten", "init_sym_grp", "iterate_solver",
    "parquet_solver_hubbard_parquet_approximation", "parquet_solver_siam_parquet_approximation", "solve", "unflatten",
    "mfRGLinearMap", "fixed_point_preconditioned", "solve_using_mfRG_without_mixing",
]
