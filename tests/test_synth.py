"""Host-side checks of the seeded workload generators."""
import math

import numpy as np

from vfs_v3p2_gb300 import synth


def test_channel_grid_layout():
    c = synth.channel_coords(8, 6, 4, beta=2.0, skew=0.05)
    assert c.shape == (6, 8, 10, 3)
    assert np.isclose(c[0, 0, 0, 1], -1.0) and np.isclose(c[0, 6, 0, 1], 1.0)
    assert np.isclose(c[4, 0, 0, 2], math.pi)
    assert np.all(c[:, :, 9] == 0)  # node index ni+1 is not a grid node


def test_ucont_walls_and_periodic_ghosts():
    rng = np.random.default_rng(0)
    u = synth.gaussian_ucont(8, 6, 4, rng)
    assert np.all(u[:, 0, :, 1] == 0) and np.all(u[:, 6, :, 1] == 0)
    assert np.array_equal(u[:, :, 0, 0], u[:, :, 8, 0])
    assert np.array_equal(u[0, :, :, 2], u[4, :, :, 2])


def test_sphere_nvert_codes():
    coor = synth.channel_coords(32, 16, 16, beta=2.0, skew=0.0)
    nv = synth.sphere_nvert(coor, [(math.pi, 0.0, math.pi / 2, 0.5)])
    assert set(np.unique(nv)) == {0.0, 1.0, 4.0}
    solid = nv == 4
    # every IB cell touches a solid face neighbour
    ib = np.argwhere(nv == 1)
    for k, j, i in ib[:50]:
        assert solid[k, j, i - 1] or solid[k, j, i + 1] or solid[k, j - 1, i] or solid[k, j + 1, i] or solid[k - 1, j, i] or solid[k + 1, j, i]


def test_batch_sizes_are_coarsenable():
    cases = synth.c4_batch(count=6)
    for c in cases:
        for n in (c.grid.ni, c.grid.nj, c.grid.nk):
            assert n % 8 == 0 and 32 <= n <= 192
            assert n % (1 << (c.levels - 1)) == 0
