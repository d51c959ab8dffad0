"""Connected fluid regions in the oracle (CPU): a channel cut by solid walls
spanning whole k-planes has one region per stretch of fluid planes (the
stretches on either side of the periodic seam join).  The compatibility fix
of the right-hand side then zeroes the sum of b over each region, and the
oracle's projection step on such a grid reaches max |div u| < 1e-8."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
import oracle as O  # noqa: E402
from regions_cases import expected_labels, walled_channel  # noqa: E402

CASES = [(((9, 9), (25, 25)), 1, 2), (((9, 12), (25, 28)), 1, 2), (((16, 16),), 1, 1), (((16, 16),), 0, 2),
         (((5, 6), (12, 12), (20, 21)), 0, 4)]


@pytest.mark.parametrize("walls,kp,K", CASES)
def test_region_labels(walls, kp, K):
    case = walled_channel(walls, kp=kp)
    d = O.dims_of(case.grid)
    n, lab = O.fluid_regions(d, case.grid.nvert)
    assert n == K
    want = expected_labels(case, walls)
    inner = lab[1:-1, 1:-1, 1:-1]
    assert np.array_equal(inner, np.broadcast_to(want[1:-1, None, None], inner.shape))
    assert (lab[0] == -1).all() and (lab[-1] == -1).all() and (lab[:, 0] == -1).all() and (lab[:, :, -1] == -1).all()


def test_compatibility_per_region():
    walls = ((9, 9), (25, 25))
    case = walled_channel(walls)
    g = case.grid
    d = O.dims_of(g)
    u = np.array(case.ucont)
    M = O.form_metrics(d, g.coor)
    O.volume_flux(d, 0, u, g.nvert, M)
    b, _ = O.rhs(d, u, g.nvert, 0.04, 1.0, 1.0, True)
    _, lab = O.fluid_regions(d, g.nvert)
    for q in range(2):
        assert abs(b[lab == q].sum()) <= 1e-12 * np.abs(b).sum()


def test_oracle_step_on_split_grid():
    case = walled_channel(((9, 9), (25, 25)), ni=16, nj=8, nk=32)
    r = O.projection_step(case.grid, case.ucont, levels=case.levels, rtol=1e-12, maxit=200)
    assert r["info"]["converged"] and r["divmax"] < 1e-8
    d = O.dims_of(case.grid)
    _, lab = O.fluid_regions(d, case.grid.nvert)
    for q in range(2):
        assert abs(r["phi"][lab == q].mean()) <= 1e-12 * np.abs(r["phi"]).max()
