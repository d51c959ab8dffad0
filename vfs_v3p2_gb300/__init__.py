"""GB300-native pressure-projection step of VFS (trunglendsu/VFS_v3p2).

CUDA kernels for sm_103a behind a C ABI (include/vfs_gpu.h); capi binds it,
projection mirrors the reference's function names, synth builds the seeded
workloads.
"""
from . import capi, synth  # noqa: F401
from .projection import (UserCtx, PoissonLHSNew, PoissonRHS, PoissonSolver_MG, UpdatePressure,  # noqa: F401
                         Projection, Divergence, VolumeFlux, Flow_Solver_pressure)

__all__ = ["capi", "synth", "UserCtx", "PoissonLHSNew", "PoissonRHS", "PoissonSolver_MG", "UpdatePressure",
           "Projection", "Divergence", "VolumeFlux", "Flow_Solver_pressure"]
