"""Reference-shaped interface of the GB300 pressure-projection step.

The reference drives its pressure path through a UserCtx and free functions
(variables.h:745-785, called from Flow_Solver, solvers.c:871-931):

    PoissonLHSNew(user, Ap)        poisson.c:976
    PoissonRHS(user, B)            poisson_hypre.c:272 / poisson.c:1789
    PoissonSolver_MG(usermg, ...)  mhv_poisson.c:2121
    UpdatePressure(user)           poisson.c:2473
    Projection(user)               poisson.c:2122
    Divergence(user)               main.c:1244

UserCtx here holds a grid handle of the C ABI (include/vfs_gpu.h); its
fields (Ucont, P, Phi, Nvert) live in HBM and are read or written with the
accessors below.  The functions take the same arguments and keep the
reference's order and side effects, so a caller can swap them in one for one.
"""
from __future__ import annotations

import numpy as np

from . import capi


class UserCtx:
    """A grid of the pressure path with its resident device state."""

    def __init__(self, coor, nvert, mg_levels=3, immersed=0, periodic=(1, 0, 1), semi=(0, 0, 0), dt=0.04, st=1.0,
                 ctx: capi.Context | None = None):
        self.ctx = ctx or capi.Context()
        self.grid = self.ctx.grid_create(coor, nvert, mg_levels, immersed, periodic, semi)
        mz, my, mx = np.asarray(nvert).shape
        self.shape = (mz, my, mx)
        self.dt = dt
        self.st = st
        self.immersed = immersed
        self.mglevels = mg_levels

    # fields ---------------------------------------------------------------
    @property
    def Ucont(self) -> np.ndarray:
        return self.ctx.get_field(self.grid, capi.FIELD_UCONT, self.shape + (3,))

    @Ucont.setter
    def Ucont(self, u):
        self.ctx.set_field(self.grid, capi.FIELD_UCONT, u)

    @property
    def P(self) -> np.ndarray:
        return self.ctx.get_field(self.grid, capi.FIELD_P, self.shape)

    @P.setter
    def P(self, p):
        self.ctx.set_field(self.grid, capi.FIELD_P, p)

    @property
    def Phi(self) -> np.ndarray:
        return self.ctx.get_field(self.grid, capi.FIELD_PHI, self.shape)

    @property
    def B(self) -> np.ndarray:
        return self.ctx.get_field(self.grid, capi.FIELD_RHS, self.shape)

    @property
    def Ucat(self) -> np.ndarray:
        return self.ctx.get_field(self.grid, capi.FIELD_UCAT, self.shape + (3,))

    def close(self):
        if self.grid is not None:
            self.ctx.grid_destroy(self.grid)
            self.grid = None


def time_coeff(rans: int = 0, ti: int = 0, tistart: int = 0) -> float:
    """poisson.c:22-30: 1, or 1.5 with RANS after the first step."""
    if rans and ti != tistart:
        return 1.5
    return 1.0


def PoissonLHSNew(user: UserCtx) -> int:
    user.ctx.poisson_lhs(user.grid)
    return 0


def VolumeFlux(user: UserCtx):
    """IB flux balance before the RHS (poisson_hypre.c:662-667)."""
    return user.ctx.volume_flux(user.grid)


def PoissonRHS(user: UserCtx, meanfix: bool = True, coeff: float | None = None) -> float:
    """Right-hand side from the resident Ucont; returns the sum before the fix."""
    return user.ctx.poisson_rhs(user.grid, user.dt, user.st, time_coeff() if coeff is None else coeff, meanfix)


def PoissonSolver_MG(user: UserCtx, params: capi.SolveParams | None = None, **kw) -> dict:
    """Multigrid-preconditioned FGMRES, mean removal and phi finish."""
    p = params or capi.default_params(**kw)
    return user.ctx.poisson_solve(user.grid, p)


def UpdatePressure(user: UserCtx) -> int:
    user.ctx.update_pressure(user.grid)
    return 0


def Projection(user: UserCtx, coeff: float | None = None) -> int:
    user.ctx.projection(user.grid, user.dt, user.st, time_coeff() if coeff is None else coeff)
    return 0


def Divergence(user: UserCtx) -> float:
    return user.ctx.divergence_max(user.grid)


def Flow_Solver_pressure(user: UserCtx, params: capi.SolveParams | None = None, **kw):
    """The pressure section of Flow_Solver (solvers.c:871-931) in one call on
    the resident fields: VolumeFlux, PoissonRHS, PoissonSolver_MG,
    UpdatePressure, Projection, Divergence."""
    VolumeFlux(user)
    PoissonRHS(user)
    info = PoissonSolver_MG(user, params, **kw)
    UpdatePressure(user)
    Projection(user)
    return info, Divergence(user)
