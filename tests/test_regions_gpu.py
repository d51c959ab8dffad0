"""Grids cut into separate fluid regions (CUDA path against the oracle).

Solid walls spanning whole k-planes split a channel; each region has its own
constant null vector, so the compatibility fix of the right-hand side and the
mean removal of phi act per region, and the coarsest dense solve regularises
each region (thick walls survive the coarsening, thin ones do not).  The
step then converges to the oracle's phi, pressure and fluxes and reaches
max |div u| < 1e-8, like a single-region grid."""
import os
import sys

import numpy as np
import pytest

from vfs_v3p2_gb300 import capi, synth

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
import oracle as O  # noqa: E402
from regions_cases import walled_channel  # noqa: E402

pytestmark = pytest.mark.gpu

# (walls, k periodic, regions on the finest level, on the coarsest level)
CASES = [(((9, 9), (25, 25)), 1, 2, 1), (((9, 12), (25, 28)), 1, 2, 2), (((16, 16),), 0, 2, 1),
         (((16, 16),), 1, 1, 1)]


def _create(ctx, case):
    g = case.grid
    return ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed,
                           periodic=(g.i_periodic, g.j_periodic, g.k_periodic))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("which", range(len(CASES)))
def test_split_grid_step_matches_oracle(gpu_ctx, which, precision):
    walls, kp, kf, kc = CASES[which]
    case = walled_channel(walls, kp=kp)
    g = case.grid
    gid = _create(gpu_ctx, case)
    try:
        gpu_ctx.poisson_lhs(gid)
        assert gpu_ctx.grid_components(gid) == (kf, kc)
        ref = O.projection_step(g, case.ucont, levels=case.levels, immersed=case.immersed, rtol=1e-13, maxit=400)
        params = capi.default_params(precision=precision, rtol=1e-12, maxit=300, div_tol=1e-8)
        u = np.ascontiguousarray(case.ucont.copy())
        p = np.zeros(g.nvert.shape)
        info, divmax = gpu_ctx.projection_step(gid, params, u, p)
        assert info["converged"] and info["relres"] < 1e-11 and divmax < 1e-8, (info, divmax)
        phi = gpu_ctx.get_field(gid, capi.FIELD_PHI, p.shape)
        d = O.dims_of(g)
        _, lab = O.fluid_regions(d, g.nvert)
        for q in range(kf):
            m = lab == q
            assert abs(phi[m].mean()) <= 1e-12 * np.abs(phi).max()
            assert np.linalg.norm(phi[m] - ref["phi"][m]) <= 1e-8 * np.linalg.norm(ref["phi"][m])
        fl = lab >= 0
        assert np.abs(p[fl] - ref["p"][fl]).max() <= 1e-8 * np.abs(ref["p"][fl]).max()
        assert np.abs(u - ref["ucont"]).max() <= 1e-8 * np.abs(ref["ucont"]).max()
    finally:
        gpu_ctx.grid_destroy(gid)


def test_single_region_grids_report_one(gpu_ctx):
    case = synth.c2_sphere(scale=4)
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    try:
        gpu_ctx.poisson_lhs(gid)
        assert gpu_ctx.grid_components(gid) == (1, 1)
    finally:
        gpu_ctx.grid_destroy(gid)
