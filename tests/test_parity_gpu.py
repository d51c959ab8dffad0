"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Setup kernels and the per-step FP64 kernels follow the reference's
arithmetic order without FMA contraction, so metrics, g tensor, operator
coefficients and the projection of a given phi are compared bit for bit.
Kernels with FMA or tree reductions are compared with the tolerance written
at each assert.  The solution criterion is the one the pressure path is
judged by: relative L2 of phi <= 1e-8 after removing the fluid mean
against a tightly converged oracle solve, and max |div u| at or below the
divergence the reference's own solver settings leave (poisson_tol = 5e-9,
poisson_it = 10 iterations, main.c:87,126)."""
import math

import numpy as np
import pytest

import oracle as O
from vfs_v3p2_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def small_cases():
    return [
        ("channel", synth.channel_case(16, 12, 16, seed=11, levels=3)),
        ("sphere", synth.channel_case(32, 16, 16, seed=12, spheres=[(math.pi, 0.0, math.pi / 2, 0.6)], sigma=0.5,
                                      levels=3)),
        ("uniform", synth.channel_case(12, 8, 8, seed=13, beta=0.0, skew=0.0, levels=2)),
        ("ragged", synth.channel_case(20, 6, 12, seed=14, levels=2)),
    ]


CASES = small_cases()


@pytest.fixture(scope="module", params=[c[0] for c in CASES])
def loaded(request, gpu_ctx):
    name, case = [c for c in CASES if c[0] == request.param][0]
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    gpu_ctx.poisson_lhs(gid)
    d = O.dims_of(g)
    mg = O.MG(d, g.coor, g.nvert, case.levels)
    yield case, gid, d, mg
    mg.close()
    gpu_ctx.grid_destroy(gid)


def test_metrics_bitexact_all_levels(gpu_ctx, loaded):
    case, gid, d, mg = loaded
    for l in range(case.levels):
        ref = mg.level_array(l, "M")
        got = gpu_ctx.metrics(gid, l)
        assert np.array_equal(got, ref), f"level {l}: max diff {np.abs(got - ref).max()}"


def test_nvert_coarsening_exact(gpu_ctx, loaded):
    case, gid, d, mg = loaded
    for l in range(case.levels - 1):
        ref = mg.level_array(l, "nvert")
        got = gpu_ctx.level_nvert(gid, l).ravel()
        assert np.array_equal(got, ref)


def test_lhs_coefficients_bitexact(gpu_ctx, loaded):
    case, gid, d, mg = loaded
    for l in range(case.levels):
        ref = mg.level_array(l, "coef")
        got = gpu_ctx.coef(gid, l, 0).ravel()
        assert np.array_equal(got, ref), f"level {l}: {np.abs(got - ref).max()}"
        refm = mg.level_array(l, "mcoef")
        assert np.array_equal(gpu_ctx.coef(gid, l, 1).ravel(), refm)
        assert np.array_equal(gpu_ctx.coef(gid, l, 2).ravel(), refm.astype(np.float32).astype(np.float64))


def test_operator_apply(gpu_ctx, loaded):
    case, gid, d, mg = loaded
    rng = np.random.default_rng(5)
    for l in range(case.levels):
        ld = mg.level_dims(l)
        x = rng.normal(size=(ld.mz, ld.my, ld.mx))
        coef = mg.level_array(l, "coef").reshape((19, ld.mz, ld.my, ld.mx))
        ref = O.matvec(ld, coef, x)
        got = gpu_ctx.apply_op(gid, l, 0, x)
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()  # FMA vs separate rounding
        refm = mg.matvec(l, x)
        gotm = gpu_ctx.apply_op(gid, l, 1, x)
        assert np.abs(gotm - refm).max() <= 1e-13 * np.abs(refm).max()
        got32 = gpu_ctx.apply_op(gid, l, 2, x)
        assert np.abs(got32 - refm).max() <= 1e-5 * np.abs(refm).max()  # FP32 coefficients and arithmetic


def test_face_form_operator(gpu_ctx, loaded):
    """The FP32 face form of an 11-slot level (the multigrid operator as aj
    times the divergence of face fluxes) is the assembled operator: equal to
    FP32 rounding against the FP64 coefficients and the FP32 ones."""
    case, gid, d, mg = loaded
    rng = np.random.default_rng(9)
    checked = 0
    for l in range(case.levels):
        if gpu_ctx.coef(gid, l, 1).reshape(19, -1)[7:15].any():  # i-j or j-k cross terms: not an 11-slot level
            continue
        ld = mg.level_dims(l)
        x = rng.normal(size=(ld.mz, ld.my, ld.mx))
        ref = gpu_ctx.apply_op(gid, l, 1, x.astype(np.float32).astype(np.float64))
        got = gpu_ctx.apply_op(gid, l, 4, x)
        assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max(), l  # FP32 arithmetic and storage
        got32 = gpu_ctx.apply_op(gid, l, 2, x)
        assert np.abs(got - got32).max() <= 1e-5 * np.abs(ref).max(), l
        checked += 1
    assert checked == case.levels


def test_krylov_product_fp32_operand_exact(gpu_ctx, loaded):
    """The mixed solver's FP64 product on FP32 directions widens each operand
    on the integer pipe; it must equal the FP64 product of the same rounded
    values bit for bit, across zeros, signed zeros, FP32 subnormals and the
    exponent range."""
    case, gid, d, mg = loaded
    L = case.levels - 1
    shp = (d.mz, d.my, d.mx)
    rng = np.random.default_rng(7)
    x = rng.standard_normal(shp) * np.exp2(rng.integers(-100, 100, size=shp))
    flat = x.reshape(-1)
    flat[::7] = 0.0
    flat[3::11] = -0.0
    flat[5::13] = 3e-41   # FP32 subnormal
    flat[6::17] = -1e-44
    x32 = x.astype(np.float32).astype(np.float64)
    y3 = gpu_ctx.apply_op(gid, L, 3, x)
    y1 = gpu_ctx.apply_op(gid, L, 1, x32)
    assert np.array_equal(y3, y1)


def test_transfer_and_smoother(gpu_ctx, loaded):
    case, gid, d, mg = loaded
    rng = np.random.default_rng(6)
    for l in range(1, case.levels):
        fd, cd = mg.level_dims(l), mg.level_dims(l - 1)
        xf = rng.normal(size=(fd.mz, fd.my, fd.mx))
        ref = mg.restrict(l, xf)
        got = gpu_ctx.mg_restrict(gid, l, xf)
        assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max()
        xc = rng.normal(size=(cd.mz, cd.my, cd.mx))
        ref = mg.prolong(l, xc)
        got = gpu_ctx.mg_prolong(gid, l, xc)
        assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max()
    for l in range(case.levels):
        ld = mg.level_dims(l)
        b = rng.normal(size=(ld.mz, ld.my, ld.mx))
        x = rng.normal(size=(ld.mz, ld.my, ld.mx))
        nv = mg.level_array(l, "nvert").reshape(b.shape)
        for a in (b, x):
            a[nv > 0.1] = 0.0
            a[0], a[-1], a[:, 0], a[:, -1], a[:, :, 0], a[:, :, -1] = 0, 0, 0, 0, 0, 0
        ref = x.copy()
        mg.smooth(l, b, ref, 1, 0.8)
        got = gpu_ctx.mg_smooth(gid, l, b, x, 0.8)
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_rhs_flux_projection_divergence(gpu_ctx, loaded):
    case, gid, d, mg = loaded
    g = case.grid
    M = O.form_metrics(d, g.coor)
    u = case.ucont.copy()
    fa = O.volume_flux(d, case.immersed, u, g.nvert, M)
    gpu_ctx.set_field(gid, capi.FIELD_UCONT, case.ucont)
    fa_g = gpu_ctx.volume_flux(gid)
    assert np.allclose(fa_g, fa, rtol=1e-12, atol=1e-13 * abs(fa[0]))  # flux after the balance is rounding residue
    assert np.abs(gpu_ctx.get_field(gid, capi.FIELD_UCONT, u.shape) - u).max() <= 1e-14 * np.abs(u).max()
    gpu_ctx.set_field(gid, capi.FIELD_UCONT, u)
    b, s = O.rhs(d, u, g.nvert)
    s_g = gpu_ctx.poisson_rhs(gid)
    bg = gpu_ctx.get_field(gid, capi.FIELD_RHS, b.shape)
    assert np.abs(bg - b).max() <= 1e-13 * np.abs(b).max()  # mean fix sums in tree order
    assert abs(s_g - s) <= 1e-12 * np.abs(b).sum()
    # projection of the same phi is bit-exact
    rng = np.random.default_rng(8)
    phi = rng.normal(size=b.shape)
    O.phi_finish(d, g.nvert, phi)
    u_ref = u.copy()
    O.projection(d, M, g.nvert, phi, u_ref)
    gpu_ctx.set_field(gid, capi.FIELD_UCONT, u)
    gpu_ctx.L.vfs_set_field(gpu_ctx.h, gid, capi.FIELD_PHI, capi.dptr(phi))
    gpu_ctx.projection(gid)
    u_got = gpu_ctx.get_field(gid, capi.FIELD_UCONT, u.shape)
    assert np.array_equal(u_got, u_ref)
    ucat_ref = O.contra2cart(d, M, g.nvert, u_ref)
    ucat = gpu_ctx.get_field(gid, capi.FIELD_UCAT, u.shape)
    fl = (g.nvert < 0.1)
    fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = False, False, False, False, False, False
    # precomputed inverse metric vs per-cell Cramer's rule: rounding only
    assert np.abs(ucat[fl] - ucat_ref[fl]).max() <= 1e-13 * np.abs(ucat_ref[fl]).max()
    dv = O.divergence(d, u_ref, O.metric(M, d, "aj"), g.nvert)
    assert gpu_ctx.divergence_max(gid) == dv


def test_projection_fractional_nvert_bitexact(gpu_ctx):
    """Non-integer nvert values take the FP64 nvert tests of the projection,
    the IB flux balance and the divergence check (integer ones the byte
    path); both must reproduce the reference's branch choices, so the
    corrected fluxes and the divergence maximum are bit-exact either way."""
    case = synth.channel_case(32, 16, 16, seed=15, spheres=[(math.pi, 0.0, math.pi / 2, 0.6)], sigma=0.5, levels=3)
    g = case.grid
    nv = g.nvert * 0.35  # 0, 0.35 (IB band) and 1.4 (solid)
    gid = gpu_ctx.grid_create(g.coor, nv, case.levels, 1)
    gpu_ctx.poisson_lhs(gid)
    d = O.dims_of(g)
    M = O.form_metrics(d, g.coor)
    rng = np.random.default_rng(16)
    phi = rng.normal(size=nv.shape)
    O.phi_finish(d, nv, phi)
    u = case.ucont.copy()
    u_ref = u.copy()
    O.projection(d, M, nv, phi, u_ref)
    gpu_ctx.set_field(gid, capi.FIELD_UCONT, u)
    gpu_ctx.L.vfs_set_field(gpu_ctx.h, gid, capi.FIELD_PHI, capi.dptr(phi))
    gpu_ctx.projection(gid)
    u_got = gpu_ctx.get_field(gid, capi.FIELD_UCONT, u.shape)
    assert np.array_equal(u_got, u_ref)
    assert gpu_ctx.divergence_max(gid) == O.divergence(d, u_ref, O.metric(M, d, "aj"), nv)
    # IB flux balance (mode 1) with fractional nvert
    u2 = case.ucont.copy()
    fa = O.volume_flux(d, 1, u2, nv, M)
    gpu_ctx.set_field(gid, capi.FIELD_UCONT, case.ucont)
    fa_g = gpu_ctx.volume_flux(gid)
    assert np.allclose(fa_g, fa, rtol=1e-12, atol=1e-13 * abs(fa[0]))
    assert np.abs(gpu_ctx.get_field(gid, capi.FIELD_UCONT, u.shape) - u2).max() <= 1e-14 * np.abs(u2).max()
    gpu_ctx.grid_destroy(gid)


def _faces_vs_reference(gpu_ctx, gid, d, M, nv, u, phi, dt, st, coeff):
    """vfs_projection_faces against the oracle's Projection (the reference's
    operation order) for the same phi: equal to rounding, every face the
    reference leaves alone unchanged bit for bit."""
    u_ref = u.copy()
    O.projection(d, M, nv, phi, u_ref, dt=dt, st=st, coeff=coeff)
    gpu_ctx.set_field(gid, capi.FIELD_UCONT, u)
    gpu_ctx.L.vfs_set_field(gpu_ctx.h, gid, capi.FIELD_PHI, capi.dptr(phi))
    gpu_ctx.projection(gid, dt=dt, st=st, coeff=coeff, faces=True)
    u_got = gpu_ctx.get_field(gid, capi.FIELD_UCONT, u.shape)
    # per component: FMAs and the pair sums' order against the reference's
    # left-to-right sums, relative to the flux and its correction
    scale = np.abs(u).max() + np.abs(u_ref - u).max()
    assert np.abs(u_got - u_ref).max() <= 1e-14 * scale
    untouched = u_ref == u
    assert np.array_equal(u_got[untouched], u[untouched])
    dv = O.divergence(d, u_ref, O.metric(M, d, "aj"), nv)
    dg = gpu_ctx.divergence_max(gid)
    assert abs(dg - dv) <= 1e-12 * max(dv, 1e-300) + 1e-14 * scale


def test_projection_faces_matches_reference_order(gpu_ctx, loaded):
    case, gid, d, mg = loaded
    g = case.grid
    M = O.form_metrics(d, g.coor)
    rng = np.random.default_rng(81)
    for dt, st, coeff in ((0.04, 1.0, 1.0), (0.013, 0.5, 1.5)):
        phi = rng.normal(size=g.nvert.shape) * 10.0
        O.phi_finish(d, g.nvert, phi)
        _faces_vs_reference(gpu_ctx, gid, d, M, g.nvert, case.ucont.copy(), phi, dt, st, coeff)


@pytest.mark.parametrize("kind", ["fractional", "walled", "terrain"])
def test_projection_faces_other_grids(gpu_ctx, kind):
    """The face-weight projection on grids whose regime choices differ from
    the channel's: fractional nvert (the FP64 nvert tests), walls on every
    side (no periodic seam) and the stretched terrain grid."""
    if kind == "terrain":
        case = synth.c3_terrain(scale=8)
        g = case.grid
        nv = g.nvert
    else:
        case = synth.channel_case(32, 16, 16, seed=15, spheres=[(math.pi, 0.0, math.pi / 2, 0.6)], sigma=0.5,
                                  levels=3)
        g = case.grid
        nv = g.nvert * 0.35 if kind == "fractional" else g.nvert
    desc_periodic = kind != "walled"
    if desc_periodic:
        gid = gpu_ctx.grid_create(g.coor, nv, case.levels, case.immersed)
        d = O.dims_of(g)
    else:
        gid = gpu_ctx.grid_create(g.coor, nv, case.levels, case.immersed, periodic=(0, 0, 0))
        mz, my, mx = nv.shape
        d = O.Dims(mx, my, mz, 0, 0, 0)
    try:
        gpu_ctx.poisson_lhs(gid)
        M = O.form_metrics(d, g.coor)
        rng = np.random.default_rng(82)
        phi = rng.normal(size=nv.shape)
        O.phi_finish(d, nv, phi)
        _faces_vs_reference(gpu_ctx, gid, d, M, nv, case.ucont.copy(), phi, 0.04, 1.0, 1.0)
    finally:
        gpu_ctx.grid_destroy(gid)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_fp16_operator", "mixed_fp32_assembled"])
@pytest.mark.parametrize("orth", ["cgs", "cgs2"])
def test_full_step_parity(gpu_ctx, loaded, precision, orth):
    """mixed: FP32 multigrid on FP32 stencil coefficients, in face form on
    11-slot levels (the default); mixed_fp16_operator: on the FP16
    diagonal-normalised operator; mixed_fp32_assembled: on the 19 assembled
    FP32 coefficients."""
    case, gid, d, mg = loaded
    g = case.grid
    ref = O.projection_step(g, case.ucont, levels=case.levels, immersed=case.immersed, rtol=1e-13, maxit=400, mg=mg,
                            orth=1 if orth == "cgs" else 2)
    params = capi.default_params(precision=precision.split("_")[0], rtol=1e-12, maxit=300, restart=30, orth=orth,
                                 div_tol=1e-8,
                                 mg_half={"mixed_fp16_operator": 1, "mixed_fp32_assembled": 2}.get(precision, 0))
    u = np.ascontiguousarray(case.ucont.copy())
    p = np.zeros(g.nvert.shape)
    info, divmax = gpu_ctx.projection_step(gid, params, u, p)
    assert info["converged"] and info["relres"] < 1e-11
    phi = gpu_ctx.get_field(gid, capi.FIELD_PHI, p.shape)
    fl = (g.nvert < 0.1)
    fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = False, False, False, False, False, False
    a, r = phi[fl] - phi[fl].mean(), ref["phi"][fl] - ref["phi"][fl].mean()
    assert np.linalg.norm(a - r) / np.linalg.norm(r) <= 1e-8
    assert np.abs(p[fl] - ref["p"][fl]).max() <= 1e-8 * np.abs(ref["p"][fl]).max()
    assert np.abs(u - ref["ucont"]).max() <= 1e-8 * np.abs(ref["ucont"]).max()
    ref_settings = O.projection_step(g, case.ucont, levels=case.levels, immersed=case.immersed, rtol=5e-9, maxit=10,
                                     mg=mg, orth=1)
    assert divmax <= ref_settings["divmax"]
    assert divmax < 1e-8


def test_mixed_precision_error_vs_fp64_oracle(gpu_ctx):
    """Mixed FP32-MG / FP64-FGMRES reaches the FP64 oracle's solution: the
    FP32 preconditioner only changes search directions."""
    case = synth.c2_sphere(scale=4)
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, 1)
    gpu_ctx.poisson_lhs(gid)
    ref = O.projection_step(g, case.ucont, levels=case.levels, immersed=1, rtol=1e-13, maxit=400)
    u = np.ascontiguousarray(case.ucont.copy())
    info, divmax = gpu_ctx.projection_step(gid, capi.default_params(precision="mixed", rtol=1e-12, div_tol=1e-8), u,
                                           None)
    phi = gpu_ctx.get_field(gid, capi.FIELD_PHI, g.nvert.shape)
    fl = (g.nvert < 0.1)
    fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = False, False, False, False, False, False
    a, r = phi[fl] - phi[fl].mean(), ref["phi"][fl] - ref["phi"][fl].mean()
    assert np.linalg.norm(a - r) / np.linalg.norm(r) <= 1e-8
    ref_settings = O.projection_step(g, case.ucont, levels=case.levels, immersed=1, rtol=5e-9, maxit=10)
    assert divmax <= ref_settings["divmax"] and divmax < 1e-8
    gpu_ctx.grid_destroy(gid)


def test_errors_are_reported(gpu_ctx):
    case = CASES[0][1]
    g = case.grid
    with pytest.raises(capi.VfsError) as e:
        gpu_ctx.grid_create(g.coor[:, :, :-1].copy(), g.nvert[:, :, :-1].copy(), 3, 0)  # odd i extent
    assert e.value.code == capi.VFS_ERR_ARG
    gid = gpu_ctx.grid_create(g.coor, g.nvert, 2, 0)
    with pytest.raises(capi.VfsError) as e:
        gpu_ctx.poisson_solve(gid, capi.default_params())
    assert e.value.code == capi.VFS_ERR_STATE
    gpu_ctx.poisson_lhs(gid)
    bad = case.ucont.copy()
    bad[3, 3, 3, 0] = np.nan
    gpu_ctx.set_field(gid, capi.FIELD_UCONT, bad)
    with pytest.raises(capi.VfsError) as e:
        gpu_ctx.poisson_rhs(gid)
    assert e.value.code == capi.VFS_ERR_NUMERIC
    gpu_ctx.grid_destroy(gid)
    small = capi.Context(0, hbm_budget_bytes=1 << 20)
    with pytest.raises(capi.VfsError) as e:
        small.grid_create(g.coor, g.nvert, 3, 0)
    assert e.value.code == capi.VFS_ERR_NOMEM
    small.close()
