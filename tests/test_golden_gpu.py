"""The CUDA path (through the C ABI) against the committed golden fixtures,
which tests/golden/make_golden.py generated from the reference's own code:
the finest level's metrics and the operator's entries bit for bit (the
coefficients exported in the reference's compact fluid numbering), and the
full projection step (FP64 and mixed) to the solution criterion of the
pressure path: relative L2 of phi <= 1e-8 after removing the fluid mean, p
and U within 1e-8, and max |div u| < 1e-8."""
import os
import sys

import numpy as np
import pytest

import oracle as O
from vfs_v3p2_gb300 import capi

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as MG  # noqa: E402

GOLD = np.load(os.path.join(HERE, "golden", "golden_small.npz"))
CASES = MG.cases()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_cuda_path_matches_reference_golden(gpu_ctx, name, precision):
    case = MG.stored_case(GOLD, name)  # the inputs the reference ran on, bit for bit
    g = case.grid
    d = O.dims_of(g)
    gid = gpu_ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    try:
        gpu_ctx.poisson_lhs(gid)
        L = case.levels - 1
        assert np.array_equal(gpu_ctx.metrics(gid, L), GOLD[f"{name}/M"])
        coef = gpu_ctx.coef(gid, L, 0).reshape((19,) + g.nvert.shape)
        A, _ = O.csr(d, coef, g.nvert)  # the oracle's CSR export, as test infrastructure
        Ac = A.tocoo()
        order = np.lexsort((Ac.col, Ac.row))
        assert np.array_equal(Ac.row[order], GOLD[f"{name}/lhs_rows"])
        assert np.array_equal(Ac.col[order], GOLD[f"{name}/lhs_cols"])
        assert np.array_equal(Ac.data[order], GOLD[f"{name}/lhs_vals"])
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
