"""The FP16 diagonal-normalised multigrid operator (mg_half) of the FP32
multigrid.

Per fluid row with diagonal D of the aj-scaled FP64 operator, the device
stores h_m = fp16(a_m / D) in the off-diagonal slots and fp16(delta) in the
centre slot, delta = sum_m (a_m / D - h_m) accumulated in FP64 in slot
order; the y-line pivots of the normalised tridiagonal in FP32 (0 on
non-fluid rows); and restriction weights fp32(max(0, 1 - nvert_f) D_f / D_c).
Those arrays are rebuilt here with numpy from the FP64 operator and
compared: the FP16 slots and the weights bit for bit, the pivots to FP32
rounding (their FP64 recurrence may contract to FMA on the device).  The
solves with the FP16 operator reach the same residual and divergence as with
the FP32 one: the operator storage only changes the preconditioner."""
import math

import numpy as np
import pytest

from vfs_v3p2_gb300 import capi, synth

pytestmark = pytest.mark.gpu

SP, NP = 4, 3


def _cases():
    return [
        synth.channel_case(32, 16, 16, seed=21, spheres=[(math.pi, 0.0, math.pi / 2, 0.6)], sigma=0.5, levels=3),
        synth.channel_case(24, 16, 8, seed=22, beta=2.5, skew=0.1, levels=2),
    ]


def _expected(mc):
    """numpy construction of the FP16 slots and the pivots from the FP64
    aj-scaled operator mc [19, mz, my, mx]."""
    D = mc[0]
    fl = D != 0
    h = np.zeros_like(mc)
    delta = np.zeros_like(D)
    for m in range(1, 19):
        a = np.where(fl, mc[m] / np.where(fl, D, 1.0), 0.0)
        hm = a.astype(np.float16).astype(np.float64)
        delta = delta + (a - hm)
        h[m] = hm
    h[0] = delta.astype(np.float16).astype(np.float64)
    mz, my, mx = D.shape
    lf = np.zeros_like(D)
    cprev = np.zeros((mz, mx))
    for j in range(1, my - 1):
        a = h[SP][:, j, :] if j > 1 else np.zeros((mz, mx))
        bb = 1.0 + h[0][:, j, :]
        cc = h[NP][:, j, :] if j < my - 2 else np.zeros((mz, mx))
        inv = 1.0 / (bb - a * cprev)
        f = fl[:, j, :]
        lf[:, j, :] = np.where(f, inv, 0.0)
        cprev = np.where(f, cc * inv, 0.0)
    lf[:, :, 0] = lf[:, :, -1] = 0.0
    lf[0] = lf[-1] = 0.0
    return h, lf.astype(np.float32).astype(np.float64)


def test_half_operator_matches_numpy(gpu_ctx):
    for case in _cases():
        g = case.grid
        gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
        try:
            gpu_ctx.poisson_lhs(gid)
            for l in range(case.levels):
                mc = gpu_ctx.coef(gid, l, 1)
                h, lf, rw = gpu_ctx.mg_half(gid, l)
                eh, elf = _expected(mc)
                assert np.array_equal(h, eh), (l, np.abs(h - eh).max())
                inner = (slice(1, -1), slice(1, -1), slice(1, -1))
                assert np.allclose(lf[inner], elf[inner], rtol=2e-7, atol=0), (l, np.abs(lf - elf).max())
                if l == 0:
                    assert not rw.any()
                    continue
                # restriction weights: fine cell (i, j, k) -> coarse ((i + 1) // 2, ...)
                nvf = gpu_ctx.level_nvert(gid, l)
                Dc = gpu_ctx.coef(gid, l - 1, 1)[0]
                mz, my, mx = nvf.shape
                k, j, i = np.meshgrid(np.arange(1, mz - 1), np.arange(1, my - 1), np.arange(1, mx - 1), indexing="ij")
                dc = Dc[(k + 1) // 2, (j + 1) // 2, (i + 1) // 2]
                df = mc[0][1:-1, 1:-1, 1:-1]
                ok = (df != 0) & (dc != 0)
                w = np.where(ok, np.maximum(0.0, 1.0 - nvf[1:-1, 1:-1, 1:-1]) * df / np.where(ok, dc, 1.0), 0.0)
                assert np.array_equal(rw[1:-1, 1:-1, 1:-1], w.astype(np.float32).astype(np.float64)), l
        finally:
            gpu_ctx.grid_destroy(gid)


def test_row_sums_kept(gpu_ctx):
    """1 + delta + sum_m h_m equals the normalised FP64 row sum to one FP16
    rounding of delta (|delta| <= 18 * 2^-12, so the error is <= 2^-22)."""
    case = _cases()[0]
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    try:
        gpu_ctx.poisson_lhs(gid)
        for l in range(case.levels):
            mc = gpu_ctx.coef(gid, l, 1)
            h, _, _ = gpu_ctx.mg_half(gid, l)
            fl = mc[0] != 0
            exact = mc.sum(axis=0)[fl] / mc[0][fl]
            got = 1.0 + h.sum(axis=0)[fl]
            assert np.abs(got - exact).max() <= 2.0 ** -22, l
    finally:
        gpu_ctx.grid_destroy(gid)


@pytest.mark.parametrize("orth", ["cgs", "cgs2"])
def test_half_solve_matches_fp32_storage(gpu_ctx, orth):
    case = synth.c2_sphere(scale=4)
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    try:
        gpu_ctx.poisson_lhs(gid)
        out = {}
        for half in (0, 1, 2):  # FP32 face form, FP16 normalised, FP32 assembled coefficients
            params = capi.default_params(precision="mixed", rtol=1e-12, maxit=300, orth=orth, div_tol=1e-8,
                                         mg_half=half)
            u = np.ascontiguousarray(case.ucont.copy())
            gpu_ctx.set_field(gid, capi.FIELD_P, np.zeros(g.nvert.shape))
            info, divmax = gpu_ctx.projection_step(gid, params, u, None)
            assert info["converged"] and info["relres"] < 1e-11 and divmax < 1e-8, (half, info, divmax)
            assert info["mg_half_used"] == (half == 1)
            out[half] = (info, gpu_ctx.get_field(gid, capi.FIELD_PHI, g.nvert.shape), u)
        i0, phi0, u0 = out[0]
        fl = (g.nvert < 0.1)
        fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = False, False, False, False, False, False
        for half in (1, 2):
            i1, phi1, u1 = out[half]
            assert abs(i1["iterations"] - i0["iterations"]) <= 1, (i0, i1)
            a, r = phi1[fl] - phi1[fl].mean(), phi0[fl] - phi0[fl].mean()
            assert np.linalg.norm(a - r) / np.linalg.norm(r) <= 1e-9
            assert np.abs(u1 - u0).max() <= 1e-9 * np.abs(u0).max()
    finally:
        gpu_ctx.grid_destroy(gid)


def test_mg_half_rejected_values(gpu_ctx):
    case = _cases()[1]
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    try:
        gpu_ctx.poisson_lhs(gid)
        for bad in (-1, 3):
            with pytest.raises(capi.VfsError):
                gpu_ctx.projection_step(gid, capi.default_params(mg_half=bad), np.ascontiguousarray(case.ucont.copy()),
                                        None)
    finally:
        gpu_ctx.grid_destroy(gid)


def test_face_form_vcycle_matches_assembled(gpu_ctx):
    """One FP32 V-cycle with the face form of the 11-slot levels (mg_half 0)
    against the same V-cycle on the assembled FP32 coefficients (mg_half 2):
    the same operator up to FP32 rounding, so the outputs agree closely."""
    case = synth.c2_sphere(scale=4)
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    try:
        gpu_ctx.poisson_lhs(gid)
        rng = np.random.default_rng(3)
        v = rng.normal(size=g.nvert.shape)
        fl = (g.nvert < 0.1)
        fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = False, False, False, False, False, False
        v[~fl] = 0.0
        z = {h: gpu_ctx.apply_precond(gid, capi.VFS_MIXED, capi.default_params(precision="mixed", mg_half=h), v)
             for h in (0, 2)}
        assert np.isfinite(z[0]).all()
        assert np.abs(z[0] - z[2]).max() <= 1e-4 * np.abs(z[2]).max()
    finally:
        gpu_ctx.grid_destroy(gid)
