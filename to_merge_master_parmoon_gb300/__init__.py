"""GB300 (sm_103a) saddle-point multigrid for ParMooN's Q2/P1disc Oseen systems.

The solver itself is native (include/pmgpu.h, built into _build/libpmgpu.so);
this package holds its CUDA/C++ sources (csrc/), the in-tree build recipe and
thin Python handles used by the tests and the benchmark.
"""
from .problem import OseenProblem  # noqa: F401
from .solver import (PmError, PmFusedSolver, PmSolver, device_count, solve_batch,  # noqa: F401
                     solve_fused_groups)

__all__ = ["OseenProblem", "PmSolver", "PmFusedSolver", "PmError", "device_count",
           "solve_batch", "solve_fused_groups"]
