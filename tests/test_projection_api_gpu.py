"""The reference-shaped Python interface (vfs_v3p2_gb300.projection: UserCtx
and the functions Flow_Solver calls, solvers.c:871-931) driven the way the
reference drives its pressure section, against the oracle's whole step on
the same inputs: phi to relative L2 <= 1e-8 after removing the fluid mean,
p and U within 1e-8, max |div u| < 1e-8.  Also each function on its own:
PoissonRHS returns the sum before the compatibility fix, Projection applies
the reference's operation order bit for bit to the solved phi."""
import math

import numpy as np
import pytest

import oracle as O
from vfs_v3p2_gb300 import capi, synth
from vfs_v3p2_gb300 import projection as P

pytestmark = pytest.mark.gpu


def _fluid(nv):
    fl = nv < 0.1
    fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = False, False, False, False, False, False
    return fl


def test_flow_solver_pressure_section_matches_oracle(gpu_ctx):
    case = synth.channel_case(32, 16, 16, seed=51, spheres=[(math.pi, 0.0, math.pi / 2, 0.6)], sigma=0.5, levels=3)
    g = case.grid
    user = P.UserCtx(g.coor, g.nvert, mg_levels=case.levels, immersed=case.immersed, ctx=gpu_ctx)
    try:
        assert P.PoissonLHSNew(user) == 0
        user.Ucont = case.ucont
        user.P = np.zeros(g.nvert.shape)
        info, divmax = P.Flow_Solver_pressure(user, precision="mixed", rtol=1e-12, div_tol=1e-8)
        ref = O.projection_step(g, case.ucont, levels=case.levels, immersed=case.immersed, rtol=1e-13, maxit=400)
        fl = _fluid(g.nvert)
        phi = user.Phi
        a, r = phi[fl] - phi[fl].mean(), ref["phi"][fl] - ref["phi"][fl].mean()
        assert info["converged"]
        assert np.linalg.norm(a - r) <= 1e-8 * np.linalg.norm(r)
        assert np.abs(user.P[fl] - ref["p"][fl]).max() <= 1e-8 * np.abs(ref["p"][fl]).max()
        assert np.abs(user.Ucont - ref["ucont"]).max() <= 1e-8 * np.abs(ref["ucont"]).max()
        assert divmax < 1e-8 and divmax == P.Divergence(user)
    finally:
        user.close()


def test_functions_one_by_one(gpu_ctx):
    case = synth.channel_case(16, 12, 16, seed=52, levels=3)
    g = case.grid
    d = O.dims_of(g)
    M = O.form_metrics(d, g.coor)
    user = P.UserCtx(g.coor, g.nvert, mg_levels=case.levels, ctx=gpu_ctx, dt=0.02, st=0.5)
    try:
        P.PoissonLHSNew(user)
        user.Ucont = case.ucont
        s = P.PoissonRHS(user)
        b, s_ref = O.rhs(d, case.ucont.copy(), g.nvert, 0.02, 0.5, 1.0)
        assert abs(s - s_ref) <= 1e-12 * np.abs(b).sum()
        assert np.abs(user.B - b).max() <= 1e-13 * np.abs(b).max()
        P.PoissonSolver_MG(user, precision="fp64", rtol=1e-12)
        phi = user.Phi
        u_ref = case.ucont.copy()
        O.projection(d, M, g.nvert, phi, u_ref, dt=0.02, st=0.5, coeff=P.time_coeff())
        assert P.Projection(user) == 0
        assert np.array_equal(user.Ucont, u_ref)
        assert P.time_coeff(rans=1, ti=3, tistart=0) == 1.5 and P.time_coeff(rans=1, ti=0, tistart=0) == 1.0
    finally:
        user.close()
