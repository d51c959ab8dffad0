"""Moving bodies and deforming grids: after vfs_grid_update_nvert /
vfs_grid_update_coords and vfs_poisson_lhs, a grid's metrics, coarse masks
and operator coefficients equal those of a grid created from the new arrays,
bit for bit, and a projection step on it gives the same result."""
import math

import numpy as np
import pytest

from vfs_v3p2_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _case(center_x, skew=0.05, seed=51):
    return synth.channel_case(32, 16, 16, seed=seed, skew=skew, spheres=[(center_x, 0.0, math.pi / 2, 0.6)], sigma=0.5,
                              levels=3)


def _compare(ctx, ga, gb, levels, shape):
    for l in range(levels):
        assert np.array_equal(ctx.metrics(ga, l), ctx.metrics(gb, l))
        assert np.array_equal(ctx.level_nvert(ga, l), ctx.level_nvert(gb, l))
        for which in (0, 1, 2):
            assert np.array_equal(ctx.coef(ga, l, which), ctx.coef(gb, l, which))
    params = capi.default_params(rtol=1e-10, div_tol=1e-8)
    out = []
    for g in (ga, gb):
        ctx.set_field(g, capi.FIELD_P, np.zeros(shape))
        out.append(ctx.projection_step(g, params))
    assert out[0][0]["iterations"] == out[1][0]["iterations"] and out[0][1] == out[1][1]


def test_update_nvert_equals_fresh_grid(gpu_ctx):
    a, b = _case(math.pi - 0.8), _case(math.pi + 0.8)
    ga = gpu_ctx.grid_create(a.grid.coor, a.grid.nvert, a.levels, 1)
    gb = gpu_ctx.grid_create(b.grid.coor, b.grid.nvert, b.levels, 1)
    try:
        gpu_ctx.poisson_lhs(ga)
        gpu_ctx.update_nvert(ga, b.grid.nvert)          # the body moved
        with pytest.raises(capi.VfsError):              # the operator must be rebuilt first
            gpu_ctx.projection_step(ga, capi.default_params())
        gpu_ctx.poisson_lhs(ga)
        gpu_ctx.poisson_lhs(gb)
        for g in (ga, gb):
            gpu_ctx.set_field(g, capi.FIELD_USTAR, b.ucont)
        _compare(gpu_ctx, ga, gb, b.levels, b.grid.nvert.shape)
    finally:
        gpu_ctx.grid_destroy(ga)
        gpu_ctx.grid_destroy(gb)


def test_update_coords_equals_fresh_grid(gpu_ctx):
    a, b = _case(math.pi, skew=0.0), _case(math.pi, skew=0.08)
    ga = gpu_ctx.grid_create(a.grid.coor, b.grid.nvert, a.levels, 1)
    gb = gpu_ctx.grid_create(b.grid.coor, b.grid.nvert, b.levels, 1)
    try:
        gpu_ctx.poisson_lhs(ga)
        gpu_ctx.update_coords(ga, b.grid.coor)          # the grid deformed
        gpu_ctx.poisson_lhs(ga)
        gpu_ctx.poisson_lhs(gb)
        for g in (ga, gb):
            gpu_ctx.set_field(g, capi.FIELD_USTAR, b.ucont)
        _compare(gpu_ctx, ga, gb, b.levels, b.grid.nvert.shape)
    finally:
        gpu_ctx.grid_destroy(ga)
        gpu_ctx.grid_destroy(gb)
