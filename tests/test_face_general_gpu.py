"""The general FP32 face form of the multigrid operator: on levels with i-j
or j-k cross terms (terrain-following grids) every face flux carries its
normal term and both cross terms (poisson.c:1173-1558), with the cross
weights' one-sided regimes in their low mantissa bits.  Checked against the
assembled operator on every level -- over the hill with walls in j and
periodic i and k, with immersed bodies on the terrain (one-sided regimes of
every cross term next to solid cells), and with every axis periodic -- and
through a whole mixed-precision projection step against the FP64 one."""
import math

import numpy as np
import pytest

from vfs_v3p2_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _terrain(ni, nj, nk, spheres=(), levels=3, per=(1, 0, 1)):
    coor = synth.terrain_coords(ni, nj, nk, 2.5)
    nv = synth.sphere_nvert(coor, spheres, *per) if spheres else np.zeros((nk + 2, nj + 2, ni + 2))
    rng = np.random.default_rng(81)
    u = synth.profile_ucont(coor, ni, nj, nk, rng, synth.loglaw, 0.05, *per)
    g = synth.Grid(ni, nj, nk, coor, nv)
    return synth.Case(f"terrain_{ni}x{nj}x{nk}", g, u, 1 if spheres else 0, levels), per


CASES = {
    "hill_64x32x32": lambda: _terrain(64, 32, 32),
    "hill_spheres_64x32x32": lambda: _terrain(64, 32, 32, spheres=[(math.pi, 0.45, math.pi / 2, 0.25),
                                                                  (1.0, 0.8, 0.5, 0.2)]),
    "hill_periodic_32x32x32": lambda: _terrain(32, 32, 32, spheres=[(math.pi, 0.5, math.pi / 2, 0.3)],
                                               per=(1, 1, 1)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_general_face_form_is_the_assembled_operator(gpu_ctx, name):
    (case, per) = CASES[name]()
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed, periodic=per)
    try:
        gpu_ctx.poisson_lhs(gid)
        rng = np.random.default_rng(82)
        general = 0
        for l in range(case.levels):
            coef = gpu_ctx.coef(gid, l, 1)
            if coef.reshape(19, -1)[7:15].any():  # i-j or j-k cross terms: the general form
                general += 1
            mz, my, mx = coef.shape[1:]
            x = rng.normal(size=(mz, my, mx))
            ref = gpu_ctx.apply_op(gid, l, 1, x.astype(np.float32).astype(np.float64))
            got = gpu_ctx.apply_op(gid, l, 4, x)
            assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max(), (l, np.abs(got - ref).max() / np.abs(ref).max())
        assert general >= 1
    finally:
        gpu_ctx.grid_destroy(gid)


@pytest.mark.parametrize("name", ["hill_64x32x32", "hill_spheres_64x32x32"])
def test_general_face_form_step(gpu_ctx, name):
    """A mixed step on the general face form reaches the FP64 step's phi and
    divergence bar (the multigrid only preconditions the FP64 FGMRES)."""
    (case, per) = CASES[name]()
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed, periodic=per)
    try:
        gpu_ctx.poisson_lhs(gid)
        out = {}
        for prec in ("fp64", "mixed"):
            u = np.ascontiguousarray(case.ucont.copy())
            p = np.zeros(g.nvert.shape)
            info, dm = gpu_ctx.projection_step(gid, capi.default_params(precision=prec, rtol=1e-11, div_tol=1e-8), u, p)
            out[prec] = (info, dm, gpu_ctx.get_field(gid, capi.FIELD_PHI, p.shape))
        fl = g.nvert < 0.1
        fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = (False,) * 6
        a, r = out["mixed"][2][fl], out["fp64"][2][fl]
        a, r = a - a.mean(), r - r.mean()
        assert out["mixed"][0]["converged"] and out["mixed"][1] < 1e-8
        assert np.linalg.norm(a - r) <= 1e-8 * np.linalg.norm(r)
    finally:
        gpu_ctx.grid_destroy(gid)
