"""Semi-coarsening on the CUDA path (the reference's -mg_i_semi, -mg_j_semi,
-mg_k_semi: isc, jsc, ksc in MyRestriction / MyInterpolation,
poisson.c:336-471, 526-669, and the coarse grids of init.c:95-127,
239-241) against the oracle, whose transfers with each flag are pinned bit
for bit to the reference's own functions (tests/test_ref_oracle.py): per
level the dimensions, the coarse nvert, the metrics and the operator
coefficients exactly; restriction and prolongation to rounding; and a whole
projection step, FP64 and mixed, to the solution criterion of the pressure
path (relative L2 of phi <= 1e-8 after removing the fluid mean, max |div u|
< 1e-8)."""
import math

import numpy as np
import pytest

import oracle as O
from vfs_v3p2_gb300 import capi, synth

pytestmark = pytest.mark.gpu

SEMIS = [(0, 1, 0), (1, 0, 0), (0, 0, 1)]


def _case():
    return synth.channel_case(32, 16, 16, seed=41, spheres=[(math.pi, 0.0, math.pi / 2, 0.6)], sigma=0.5, levels=3)


@pytest.fixture(scope="module", params=SEMIS, ids=["semi_j", "semi_i", "semi_k"])
def semi_loaded(request, gpu_ctx):
    semi = request.param
    case = _case()
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed, semi=semi)
    gpu_ctx.poisson_lhs(gid)
    d = O.dims_of(g)
    mg = O.MG(d, g.coor, g.nvert, case.levels, semi=semi)
    yield semi, case, gid, d, mg
    mg.close()
    gpu_ctx.grid_destroy(gid)


def test_semi_levels_exact(gpu_ctx, semi_loaded):
    semi, case, gid, d, mg = semi_loaded
    for l in range(case.levels):
        ld = mg.level_dims(l)
        assert gpu_ctx.level_dims(gid, l) == (ld.mx, ld.my, ld.mz), l
        assert np.array_equal(gpu_ctx.level_nvert(gid, l).ravel(), mg.level_array(l, "nvert")), l
        assert np.array_equal(gpu_ctx.metrics(gid, l), mg.level_array(l, "M")), l
        assert np.array_equal(gpu_ctx.coef(gid, l, 0).ravel(), mg.level_array(l, "coef")), l
        assert np.array_equal(gpu_ctx.coef(gid, l, 1).ravel(), mg.level_array(l, "mcoef")), l
    # the semi-coarsened axis keeps its extent down the hierarchy
    top, bottom = mg.level_dims(case.levels - 1), mg.level_dims(0)
    kept = [a for a, s in zip(("mx", "my", "mz"), semi) if s]
    assert all(getattr(top, a) == getattr(bottom, a) for a in kept)


def test_semi_transfers(gpu_ctx, semi_loaded):
    semi, case, gid, d, mg = semi_loaded
    rng = np.random.default_rng(42)
    for l in range(1, case.levels):
        fd, cd = mg.level_dims(l), mg.level_dims(l - 1)
        xf = rng.normal(size=(fd.mz, fd.my, fd.mx))
        ref = mg.restrict(l, xf)
        got = gpu_ctx.mg_restrict(gid, l, xf)
        assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max(), l
        xc = rng.normal(size=(cd.mz, cd.my, cd.mx))
        ref = mg.prolong(l, xc)
        got = gpu_ctx.mg_prolong(gid, l, xc)
        assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max(), l


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_semi_full_step(gpu_ctx, semi_loaded, precision):
    semi, case, gid, d, mg = semi_loaded
    g = case.grid
    ref = O.projection_step(g, case.ucont, levels=case.levels, immersed=case.immersed, rtol=1e-13, maxit=400, mg=mg)
    u = np.ascontiguousarray(case.ucont.copy())
    p = np.zeros(g.nvert.shape)
    info, divmax = gpu_ctx.projection_step(gid, capi.default_params(precision=precision, rtol=1e-12, maxit=300,
                                                                    div_tol=1e-8), u, p)
    assert info["converged"]
    phi = gpu_ctx.get_field(gid, capi.FIELD_PHI, p.shape)
    fl = g.nvert < 0.1
    fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = False, False, False, False, False, False
    a, r = phi[fl] - phi[fl].mean(), ref["phi"][fl] - ref["phi"][fl].mean()
    assert np.linalg.norm(a - r) <= 1e-8 * np.linalg.norm(r)
    assert np.abs(u - ref["ucont"]).max() <= 1e-8 * np.abs(ref["ucont"]).max()
    assert divmax < 1e-8
