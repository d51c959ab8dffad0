"""The finest-level face-form sweep that stages its operands in shared
memory by tensor-memory copies (mg_stage = 1) against the register-staged
sweep (mg_stage = 0): the same per-cell arithmetic, so one preconditioner
application and a whole projection step agree bit for bit.  Grids cover both alignments of the
tensor copies' odd rows (mx mod 4 = 2 and 0), partial tiles and bands, and
periodic seams in i, j and k (whose seam cells read their stencil from
global memory)."""
import math

import numpy as np
import pytest

from vfs_v3p2_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _cases():
    return {
        # mx = 258 (mx mod 4 = 2), 128 rows = 8 full 16-row bands
        "sphere_256x128x128": (synth.c2_sphere(), (1, 0, 1)),
        # mx = 256 (mx mod 4 = 0), a partial last tile (254 = 7 x 32 + 30), partial bands (66 = 4 x 16 + 2 = 4 x 14 + 10)
        "channel_254x66x64": (synth.channel_case(254, 66, 64, seed=71, levels=2), (1, 0, 1)),
        # every axis periodic: seam cells in i, j and k
        "periodic_128x64x128": (synth.channel_case(128, 64, 128, seed=72,
                                                   spheres=[(math.pi, 0.0, math.pi / 2, 0.5)], levels=3),
                                (1, 1, 1)),
    }


CASES = _cases()


def _fluid(nv):
    fl = nv < 0.1
    fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = False, False, False, False, False, False
    return fl


@pytest.mark.parametrize("name", sorted(CASES))
def test_staged_sweep_precond_bitexact(gpu_ctx, name):
    case, per = CASES[name]
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed, periodic=per)
    try:
        gpu_ctx.poisson_lhs(gid)
        rng = np.random.default_rng(73)
        v = rng.normal(size=g.nvert.shape)
        v[~_fluid(g.nvert)] = 0.0
        z = {t: gpu_ctx.apply_precond(gid, capi.VFS_MIXED, capi.default_params(precision="mixed", mg_stage=t), v)
             for t in (0, 1)}
        assert np.isfinite(z[0]).all() and np.abs(z[0]).max() > 0
        assert np.array_equal(z[1], z[0]), np.abs(z[1] - z[0]).max()
    finally:
        gpu_ctx.grid_destroy(gid)


@pytest.mark.parametrize("name", ["sphere_256x128x128", "periodic_128x64x128"])
def test_staged_sweep_step_bitexact(gpu_ctx, name):
    case, per = CASES[name]
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed, periodic=per)
    try:
        gpu_ctx.poisson_lhs(gid)
        out = []
        for t in (0, 1):
            u = np.ascontiguousarray(case.ucont.copy())
            p = np.zeros(g.nvert.shape)
            info, dm = gpu_ctx.projection_step(gid, capi.default_params(precision="mixed", rtol=1e-9, div_tol=1e-8,
                                                                        mg_stage=t), u, p)
            out.append((info["iterations"], dm, u, p, gpu_ctx.get_field(gid, capi.FIELD_PHI, p.shape)))
        i0, d0, u0, p0, f0 = out[0]
        for t, (i1, d1, u1, p1, f1) in enumerate(out[1:], 1):
            assert i0 == i1 and d0 == d1, t
            assert np.array_equal(f0, f1) and np.array_equal(u0, u1) and np.array_equal(p0, p1), t
        assert d0 < 1e-8
    finally:
        gpu_ctx.grid_destroy(gid)


def test_stage_value_checked(gpu_ctx):
    case = synth.channel_case(16, 8, 8, seed=75, levels=2)
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    try:
        gpu_ctx.poisson_lhs(gid)
        with pytest.raises(capi.VfsError):
            gpu_ctx.apply_precond(gid, capi.VFS_MIXED, capi.default_params(precision="mixed", mg_stage=2),
                                  np.zeros(g.nvert.shape))
    finally:
        gpu_ctx.grid_destroy(gid)


@pytest.mark.parametrize("name", sorted(CASES))
def test_warp_row_sweep_bitexact(gpu_ctx, name):
    """Automatic tiles (smooth_cols = 0) run the face form's full-width
    sweeps on 30-column warp-row tiles with shuffled i neighbours; explicit
    32-column tiles (smooth_cols = 32) run the one-cell-per-thread gathers.
    Same inputs and arithmetic per cell: bit-identical results."""
    case, per = CASES[name]
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed, periodic=per)
    try:
        gpu_ctx.poisson_lhs(gid)
        rng = np.random.default_rng(76)
        v = rng.normal(size=g.nvert.shape)
        v[~_fluid(g.nvert)] = 0.0
        z = {c: gpu_ctx.apply_precond(gid, capi.VFS_MIXED, capi.default_params(precision="mixed", smooth_cols=c), v)
             for c in (0, 32)}
        assert np.isfinite(z[0]).all() and np.abs(z[0]).max() > 0
        assert np.array_equal(z[0], z[32]), np.abs(z[0] - z[32]).max()
    finally:
        gpu_ctx.grid_destroy(gid)


def test_tma_bounded_wait_reports_and_recovers(gpu_ctx):
    """A tensor-copy sweep whose copies never all arrive (the test hook
    leaves out one band's 1/m copies in every block) ends its bounded wait
    after about 0.2 s: the call fails with VFS_ERR_CUDA and the reason, and
    the context stays usable -- the next call gives the register sweep's
    result bit for bit."""
    case = synth.channel_case(128, 64, 128, seed=77, levels=3)
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    lib = capi.load()
    try:
        gpu_ctx.poisson_lhs(gid)
        rng = np.random.default_rng(78)
        v = rng.normal(size=g.nvert.shape)
        v[~_fluid(g.nvert)] = 0.0
        p1 = capi.default_params(precision="mixed", mg_stage=1)
        assert lib.vfs_debug_tma_drop(0) == 0
        try:
            with pytest.raises(capi.VfsError) as e:
                gpu_ctx.apply_precond(gid, capi.VFS_MIXED, p1, v)
        finally:
            lib.vfs_debug_tma_drop(-1)
        assert e.value.code == 2 and "bounded wait" in str(e.value)
        z1 = gpu_ctx.apply_precond(gid, capi.VFS_MIXED, p1, v)
        z0 = gpu_ctx.apply_precond(gid, capi.VFS_MIXED, capi.default_params(precision="mixed"), v)
        assert np.isfinite(z0).all() and np.array_equal(z1, z0)
    finally:
        gpu_ctx.grid_destroy(gid)
