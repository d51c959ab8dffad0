"""Known answers on affine grids and linear fields: the metrics (FormMetrics,
metrics.c:4-1290), the operator, the projection and the transfer operators.

On a grid with node r(i, j, k) = (i dx + s k dz + t j dy, j dy, k dz) every
metric is constant: the area vectors are the cross products of the two
other edge vectors, csi = r_eta x r_zeta, eta = r_zeta x r_xi,
zet = r_xi x r_eta, and aj = 1 / det[r_xi r_eta r_zeta], at cell centres
and on every face family alike (central and one-sided differences of a
linear map are exact).  A uniform Cartesian velocity V then has face fluxes
U = V . (face area vector); Contra2Cart returns V and the divergence is
zero.  Checked on the oracle (CPU) and, through the metric hook, on the
CUDA path."""
import os
import sys

import numpy as np
import pytest

from vfs_v3p2_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
import oracle as O  # noqa: E402

GEOMS = [(8, 6, 5, 0.5, 0.25, 0.2, 0.0, 0.0), (8, 6, 5, 0.5, 0.25, 0.2, 0.3, 0.0),
         (10, 8, 6, 0.3, 0.4, 0.25, -0.2, 0.15)]


def _grid(ni, nj, nk, dx, dy, dz, s, t):
    mx, my, mz = ni + 2, nj + 2, nk + 2
    coor = np.zeros((mz, my, mx, 3))
    k, j, i = np.meshgrid(np.arange(nk + 1), np.arange(nj + 1), np.arange(ni + 1), indexing="ij")
    coor[:nk + 1, :nj + 1, :ni + 1, 0] = i * dx + s * k * dz + t * j * dy
    coor[:nk + 1, :nj + 1, :ni + 1, 1] = j * dy
    coor[:nk + 1, :nj + 1, :ni + 1, 2] = k * dz
    return synth.Grid(ni, nj, nk, coor, np.zeros((mz, my, mx)), 0, 0, 0)


def _expected(dx, dy, dz, s, t):
    rx = np.array([dx, 0.0, 0.0])
    ry = np.array([t * dy, dy, 0.0])
    rz = np.array([s * dz, 0.0, dz])
    csi, eta, zet = np.cross(ry, rz), np.cross(rz, rx), np.cross(rx, ry)
    aj = 1.0 / np.dot(rx, np.cross(ry, rz))
    return csi, eta, zet, aj


def _check_pack(M, d, geom):
    csi, eta, zet, aj = _expected(*geom[3:])
    inner = (slice(1, -1), slice(1, -1), slice(1, -1))
    want = dict(csi=csi, eta=eta, zet=zet, icsi=csi, ieta=eta, izet=zet, jcsi=csi, jeta=eta, jzet=zet,
                kcsi=csi, keta=eta, kzet=zet)
    for name, v in want.items():
        a = O.metric(M, d, name)[inner]
        assert np.allclose(a, v, rtol=0, atol=1e-13 * np.abs(v).max()), (name, np.abs(a - v).max())
    for name in ("aj", "iaj", "jaj", "kaj"):
        a = O.metric(M, d, name)[inner]
        assert np.allclose(a, aj, rtol=1e-13, atol=0), (name, np.abs(a - aj).max())


@pytest.mark.parametrize("geom", GEOMS)
def test_oracle_affine_metrics(geom):
    g = _grid(*geom)
    d = O.dims_of(g)
    _check_pack(O.form_metrics(d, g.coor), d, geom)


@pytest.mark.parametrize("geom", GEOMS)
def test_oracle_uniform_velocity(geom):
    g = _grid(*geom)
    d = O.dims_of(g)
    M = O.form_metrics(d, g.coor)
    V = np.array([0.7, -0.4, 0.25])
    u = np.zeros(g.nvert.shape + (3,))
    u[..., 0] = O.metric(M, d, "icsi") @ V
    u[..., 1] = O.metric(M, d, "jeta") @ V
    u[..., 2] = O.metric(M, d, "kzet") @ V
    ucat = O.contra2cart(d, M, g.nvert, u)
    inner = (slice(1, -1), slice(1, -1), slice(1, -1))
    assert np.allclose(ucat[inner], V, rtol=0, atol=1e-13)
    assert O.divergence(d, u, O.metric(M, d, "aj"), g.nvert) <= 1e-12
    b, _ = O.rhs(d, u, g.nvert, 0.04, 1.0, 1.0, False)
    assert np.abs(b).max() <= 1e-12


@pytest.mark.parametrize("geom", GEOMS)
def test_oracle_projection_of_a_linear_potential(geom):
    """phi = G . (cell centre): the index-space differences of a linear field
    are exact (central and one-sided alike), and sum_m r_m a_m^T = I / aj on
    an affine grid, so Projection (poisson.c:2122-2470) lowers every interior
    face flux by exactly dt st / coeff G . (face area vector), cross terms
    included.  The CUDA projection matches this oracle bit for bit
    (tests/test_parity_gpu.py)."""
    g = _grid(*geom)
    d = O.dims_of(g)
    M = O.form_metrics(d, g.coor)
    G = np.array([0.3, -0.7, 0.45])
    phi = O.metric(M, d, "cent") @ G
    u0 = np.random.default_rng(3).standard_normal(g.nvert.shape + (3,))
    for dt, st, coeff in ((0.04, 1.0, 1.0), (0.02, 1.5, 1.5)):
        u = u0.copy()
        O.projection(d, M, g.nvert, phi, u, dt, st, coeff)
        mz, my, mx = g.nvert.shape
        faces = [("icsi", 0, (slice(1, mz - 1), slice(1, my - 1), slice(1, mx - 2))),
                 ("jeta", 1, (slice(1, mz - 1), slice(1, my - 2), slice(1, mx - 1))),
                 ("kzet", 2, (slice(1, mz - 2), slice(1, my - 1), slice(1, mx - 1)))]
        for name, c, sl in faces:
            want = dt * st / coeff * (O.metric(M, d, name) @ G)
            got = (u0 - u)[..., c]
            assert np.abs(got[sl] - want[sl]).max() <= 1e-12 * np.abs(want).max(), name


@pytest.mark.parametrize("geom", GEOMS)
def test_oracle_operator_annihilates_linear_potentials(geom):
    """The assembled 19-point operator (PoissonLHSNew, poisson.c:1146-1630)
    is consistent: on an affine grid it maps a linear potential to zero on
    every cell whose stencil stays in the interior (the face fluxes of a
    uniform gradient cancel, cross terms included), and constants to zero
    everywhere.  The CUDA coefficients equal these bit for bit
    (tests/test_parity_gpu.py)."""
    g = _grid(*geom)
    d = O.dims_of(g)
    M = O.form_metrics(d, g.coor)
    coef = O.lhs(d, O.gtensor(d, M), g.nvert)
    phi = O.metric(M, d, "cent") @ np.array([0.3, -0.7, 0.45])
    y = O.matvec(d, coef, phi)
    scale = np.abs(coef).max() * np.abs(phi).max()
    assert np.abs(y[2:-2, 2:-2, 2:-2]).max() <= 1e-14 * scale
    assert np.abs(O.matvec(d, coef, np.ones_like(phi))[1:-1, 1:-1, 1:-1]).max() <= 1e-14 * np.abs(coef).max()


@pytest.mark.parametrize("geom", GEOMS)
def test_oracle_rhs_of_a_uniform_expansion(geom):
    """PoissonRHS2_hypre (poisson_hypre.c:342-429): val = -(U_i - U_i-1 + ...)
    then val *= -1 / dt * st * coeff, so b = +(net outward face flux) / dt *
    st * coeff (the opposite sign to PoissonRHS in poisson.c, paired with an
    operator of the matching sign).  For v = (a x, 0, 0) the i-face fluxes
    are a x_face times the face area vector's x part, so on an affine grid
    every cell's net flux is a times its volume and aj b = a st coeff / dt in
    every interior cell.  The CUDA right-hand side matches this oracle
    (tests/test_parity_gpu.py)."""
    g = _grid(*geom)
    d = O.dims_of(g)
    M = O.form_metrics(d, g.coor)
    a = 0.8
    u = np.zeros(g.nvert.shape + (3,))
    # the i-face of cell (i, j, k) lies on node column i with corners at
    # nodes j-1, j and k-1, k (cell j spans nodes j-1..j); only x matters
    c = g.coor
    mz, my, mx = g.nvert.shape
    xf = 0.25 * (c[0:mz - 2, 0:my - 2, :, 0] + c[1:mz - 1, 0:my - 2, :, 0] + c[0:mz - 2, 1:my - 1, :, 0] +
                 c[1:mz - 1, 1:my - 1, :, 0])
    icsi = O.metric(M, d, "icsi")
    u[1:mz - 1, 1:my - 1, :, 0] = a * xf * icsi[1:mz - 1, 1:my - 1, :, 0]
    for dt, st, coeff in ((0.04, 1.0, 1.0), (0.02, 1.5, 1.5)):
        b, _ = O.rhs(d, u, g.nvert, dt, st, coeff, False)
        aj = O.metric(M, d, "aj")
        inner = (slice(1, -1), slice(1, -1), slice(1, -1))
        want = a * st * coeff / dt
        assert np.allclose((aj * b)[inner], want, rtol=1e-12, atol=0)


def test_oracle_transfers_of_linear_fields():
    """MyInterpolation (poisson.c:526-669) is cell-centred trilinear with
    weights (27, 9, 9, 3, 9, 3, 3, 1) / 64: a field linear in the cell index
    comes back exactly away from the clamped edges.  MyRestriction
    (poisson.c:364-471) averages the 8 children: a linear fine field gives
    its value at the coarse cell centre.  The CUDA transfers match these
    within 1e-14 (tests/test_parity_gpu.py)."""
    case = synth.channel_case(16, 16, 16, seed=5, levels=2)
    g = case.grid
    d = O.dims_of(g)
    mg = O.MG(d, g.coor, g.nvert, 2)
    try:
        dc = mg.level_dims(0)
        c = np.array([1.0, 2.0, -0.5])  # coefficients of i, j, k

        def lin(shape, off, scale):
            k, j, i = np.meshgrid(*(np.arange(n) for n in shape), indexing="ij")
            return c[0] * (i + off) * scale + c[1] * (j + off) * scale + c[2] * (k + off) * scale

        xc = lin((dc.mz, dc.my, dc.mx), 0.0, 1.0)        # coarse cell index
        fine_in_coarse = lin((d.mz, d.my, d.mx), 0.5, 0.5)  # fine cell i sits at coarse (i + 0.5) / 2
        yf = mg.prolong(1, xc)
        inner = (slice(2, -2), slice(2, -2), slice(2, -2))
        assert np.abs(yf[inner] - fine_in_coarse[inner]).max() <= 1e-13 * np.abs(yf[inner]).max()
        xf = lin((d.mz, d.my, d.mx), 0.0, 1.0)
        yc = mg.restrict(1, xf)
        coarse_centre = lin((dc.mz, dc.my, dc.mx), -0.25, 2.0)  # children 2ic-1, 2ic: mean index 2ic - 0.5
        cin = (slice(1, -1), slice(1, -1), slice(1, -1))
        assert np.abs(yc[cin] - coarse_centre[cin]).max() <= 1e-13 * np.abs(yc[cin]).max()
    finally:
        mg.close()


@pytest.mark.gpu
@pytest.mark.parametrize("geom", GEOMS)
def test_cuda_affine_metrics(gpu_ctx, geom):
    g = _grid(*geom)
    d = O.dims_of(g)
    gid = gpu_ctx.grid_create(g.coor, g.nvert, 1, 0, periodic=(0, 0, 0))
    try:
        _check_pack(gpu_ctx.metrics(gid, 0), d, geom)
    finally:
        gpu_ctx.grid_destroy(gid)
