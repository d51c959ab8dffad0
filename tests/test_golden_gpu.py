"""The CUDA path (through the C ABI) against the committed golden fixtures:
operator coefficients bit for bit, and the full projection step (FP64 and
mixed) to the solution criterion of the pressure path: relative L2 of phi
<= 1e-8 after removing the fluid mean, p and U within 1e-8, and
max |div u| < 1e-8."""
import os
import sys

import numpy as np
import pytest

from vfs_v3p2_gb300 import capi

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as MG  # noqa: E402

GOLD = np.load(os.path.join(HERE, "golden", "golden_small.npz"))
CASES = MG.cases()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_cuda_path_matches_golden(gpu_ctx, name, precision):
    case = CASES[name]
    g = case.grid
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    try:
        gpu_ctx.poisson_lhs(gid)
        assert np.array_equal(gpu_ctx.coef(gid, case.levels - 1, 0), GOLD[f"{name}/coef"])
        u = np.ascontiguousarray(case.ucont.copy())
        p = np.zeros(g.nvert.shape)
        params = capi.default_params(precision=precision, rtol=1e-12, div_tol=1e-8)
        info, divmax = gpu_ctx.projection_step(gid, params, u, p)
        phi = gpu_ctx.get_field(gid, capi.FIELD_PHI, p.shape)
        fl = g.nvert < 0.1
        fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = False, False, False, False, False, False
        a, r = phi[fl] - phi[fl].mean(), GOLD[f"{name}/phi"][fl] - GOLD[f"{name}/phi"][fl].mean()
        assert np.linalg.norm(a - r) <= 1e-8 * np.linalg.norm(r)
        for got, key in ((p, "p"), (u, "ucont")):
            ref = GOLD[f"{name}/{key}"]
            assert np.abs(got - ref).max() <= 1e-8 * np.abs(ref).max(), key
        assert info["converged"] and divmax < 1e-8
    finally:
        gpu_ctx.grid_destroy(gid)
