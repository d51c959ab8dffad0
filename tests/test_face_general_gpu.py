"""The general FP32 face form of the multigrid operator: on levels with i-j
or j-k cross terms (terrain-following grids) every face flux carries its
normal term and both cross terms (poisson.c:1173-1558), with the cross
weights' one-sided regimes in their low mantissa bits.  Checked against the
assembled operator on every level -- over the hill with walls in j and
periodic i and k, with immersed bodies on the terrain (one-sided regimes of
every cross term next to solid cells), and with every axis periodic --
through a whole mixed-precision projection step against the FP64 one (also
with semi-coarsening), and in a grouped batch."""
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


def test_general_face_form_semi_coarsened(gpu_ctx):
    """Semi-coarsening in j (the face form's sweeps; the restriction falls
    back to the assembled coefficients): the mixed step reaches the FP64
    step's phi and divergence bar."""
    (case, per) = _terrain(64, 32, 32, spheres=[(math.pi, 0.45, math.pi / 2, 0.25)])
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, 3, case.immersed, periodic=per, semi=(0, 1, 0))
    try:
        gpu_ctx.poisson_lhs(gid)
        phi = {}
        for prec in ("fp64", "mixed"):
            u = np.ascontiguousarray(case.ucont.copy())
            p = np.zeros(g.nvert.shape)
            info, dm = gpu_ctx.projection_step(gid, capi.default_params(precision=prec, rtol=1e-11, div_tol=1e-8), u, p)
            assert info["converged"] and dm < 1e-8, (prec, info, dm)
            phi[prec] = gpu_ctx.get_field(gid, capi.FIELD_PHI, p.shape)
        fl = g.nvert < 0.1
        fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = (False,) * 6
        a, r = phi["mixed"][fl], phi["fp64"][fl]
        a, r = a - a.mean(), r - r.mean()
        assert np.linalg.norm(a - r) <= 1e-8 * np.linalg.norm(r)
    finally:
        gpu_ctx.grid_destroy(gid)


def test_grouped_batch_with_a_terrain_grid(gpu_ctx):
    """A batch holding a grid on the general face form runs it ungrouped
    under mg_grouped = 1 (the grouped kernels take the 11-slot form): the
    batch's results are those of mg_grouped = 0 bit for bit."""
    cases = [_terrain(32, 32, 32)[0]] + list(synth.c4_batch(count=3, seed=79, lo=(16, 16, 16), hi=(32, 32, 32)))
    ids = []
    try:
        for c in cases:
            gg = c.grid
            gid = gpu_ctx.grid_create(gg.coor, gg.nvert, c.levels, c.immersed)
            gpu_ctx.poisson_lhs(gid)
            ids.append(gid)
        out = {}
        for grouped in (0, 1):
            for gid, c in zip(ids, cases):
                gpu_ctx.set_field(gid, capi.FIELD_USTAR, c.ucont)
                gpu_ctx.set_field(gid, capi.FIELD_P, np.zeros(c.grid.nvert.shape))
            plist = [capi.default_params(precision="mixed", rtol=1e-9, div_tol=1e-8, mg_grouped=grouped)] * len(cases)
            infos, dm = gpu_ctx.projection_step_batch(ids, plist)
            assert all(i["converged"] for i in infos) and (dm < 1e-8).all()
            out[grouped] = ([i["iterations"] for i in infos], dm.copy(),
                            [gpu_ctx.get_field(gid, capi.FIELD_PHI, c.grid.nvert.shape) for gid, c in zip(ids, cases)])
        assert out[0][0] == out[1][0] and np.array_equal(out[0][1], out[1][1])
        for a, b in zip(out[0][2], out[1][2]):
            assert np.array_equal(a, b)
    finally:
        for gid in ids:
            gpu_ctx.grid_destroy(gid)
