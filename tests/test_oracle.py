"""Known-answer tests of the CPU oracle (test infrastructure).

The reference ships no tests or golden data and cannot be built here (its
pressure path needs PETSc, HYPRE and MPI), so the oracle is pinned by
properties of the discretisation it restates and by a direct solve."""
import math

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

import oracle as O
from vfs_v3p2_gb300 import synth


def _setup(grid):
    d = O.dims_of(grid)
    M = O.form_metrics(d, grid.coor)
    g = O.gtensor(d, M)
    coef = O.lhs(d, g, grid.nvert)
    return d, M, g, coef


def _grid(ni, nj, nk, beta=2.0, skew=0.05, spheres=()):
    coor = synth.channel_coords(ni, nj, nk, beta, skew)
    nv = synth.sphere_nvert(coor, spheres) if spheres else np.zeros((nk + 2, nj + 2, ni + 2))
    return synth.Grid(ni, nj, nk, coor, nv)


def test_uniform_grid_eigenmodes():
    """Uniform Cartesian grid: g11 = dy dz / dx etc., no cross terms, so a
    separable cosine mode (periodic in x, z; cell-centred Neumann in y) is
    an exact eigenvector with the 7-point eigenvalue."""
    ni, nj, nk = 12, 10, 8
    grid = _grid(ni, nj, nk, beta=0.0, skew=0.0)
    d, M, g, coef = _setup(grid)
    dx, dy, dz = 2 * math.pi / ni, 2.0 / nj, math.pi / nk
    inner = (slice(1, -1),) * 3
    assert np.allclose(g[0][inner], dy * dz / dx, rtol=1e-12)
    assert np.allclose(g[4][inner], dx * dz / dy, rtol=1e-12)
    assert np.allclose(g[8][inner], dx * dy / dz, rtol=1e-12)
    for q in (1, 2, 3, 5, 6, 7):
        assert np.abs(g[q][inner]).max() < 1e-14
    for (p, qq, r) in [(1, 1, 1), (2, 3, 1), (5, 0, 3)]:
        k, j, i = np.meshgrid(np.arange(nk + 2), np.arange(nj + 2), np.arange(ni + 2), indexing="ij")
        phi = (np.cos(2 * math.pi * p * (i - 0.5) / ni) * np.cos(math.pi * qq * (j - 0.5) / nj)
               * np.cos(2 * math.pi * r * (k - 0.5) / nk))
        lam = (dy * dz / dx * (2 * math.cos(2 * math.pi * p / ni) - 2) + dx * dz / dy * (2 * math.cos(math.pi * qq / nj) - 2)
               + dx * dy / dz * (2 * math.cos(2 * math.pi * r / nk) - 2))
        y = O.matvec(d, coef, phi)
        assert np.allclose(y[inner], lam * phi[inner], atol=1e-12 * abs(lam) + 1e-13)


@pytest.mark.parametrize("spheres", [(), ((math.pi, 0.0, math.pi / 2, 0.5),)])
def test_null_space_and_conservation(spheres):
    """Rows sum to zero (A 1 = 0) and columns sum to zero (the flux form is
    conservative: 1^T A = 0), with and without an immersed body."""
    grid = _grid(20, 12, 16, spheres=spheres)
    d, M, g, coef = _setup(grid)
    A, gid = O.csr(d, coef, grid.nvert)
    one = np.ones(A.shape[0])
    scale = np.abs(A).max()
    assert np.abs(A @ one).max() < 1e-13 * scale
    assert np.abs(A.T @ one).max() < 1e-13 * scale


def test_symmetric_without_skew():
    grid = _grid(12, 10, 8, beta=2.0, skew=0.0)
    d, M, g, coef = _setup(grid)
    A, _ = O.csr(d, coef, grid.nvert)
    assert abs(A - A.T).max() < 1e-14 * abs(A).max()
    grid = _grid(12, 10, 8, beta=2.0, skew=0.05)
    d, M, g, coef = _setup(grid)
    A, _ = O.csr(d, coef, grid.nvert)
    assert abs(A - A.T).max() > 1e-6 * abs(A).max()


@pytest.mark.parametrize("spheres", [(), ((math.pi, 0.0, math.pi / 2, 0.6),)])
def test_projection_operator_consistency(spheres):
    """div(Projection(U, phi)) = div(U) - dt st / coeff * (A phi) on every
    fluid cell: Projection (poisson.c:2202-2397) applies the same gradient
    stencil whose divergence PoissonLHSNew assembles."""
    ni, nj, nk = 24, 12, 16
    grid = _grid(ni, nj, nk, spheres=spheres)
    d, M, g, coef = _setup(grid)
    rng = np.random.default_rng(7)
    u = synth.gaussian_ucont(ni, nj, nk, rng)
    phi = rng.normal(size=(nk + 2, nj + 2, ni + 2))
    O.phi_finish(d, grid.nvert, phi)
    dt, st, coeff = 0.04, 1.0, 1.0

    def div(u):
        v = np.zeros(u.shape[:3])
        v[1:-1, 1:-1, 1:-1] = (u[1:-1, 1:-1, 1:-1, 0] - u[1:-1, 1:-1, :-2, 0] + u[1:-1, 1:-1, 1:-1, 1]
                               - u[1:-1, :-2, 1:-1, 1] + u[1:-1, 1:-1, 1:-1, 2] - u[:-2, 1:-1, 1:-1, 2])
        return v

    d0 = div(u)
    u2 = u.copy()
    O.projection(d, M, grid.nvert, phi, u2, dt, st, coeff)
    d1 = div(u2)
    Aphi = O.matvec(d, coef, phi)
    fluid = np.zeros(grid.nvert.shape, bool)
    fluid[1:-1, 1:-1, 1:-1] = grid.nvert[1:-1, 1:-1, 1:-1] < 0.1
    lhs = (d1 - d0)[fluid]
    rhs = -(dt * st / coeff) * Aphi[fluid]
    assert np.abs(lhs - rhs).max() < 1e-12 * max(1.0, np.abs(rhs).max())


@pytest.mark.parametrize("orth", [1, 2])
def test_fgmres_matches_direct_solve(orth):
    """Both Gram-Schmidt variants (one classical pass, as PETSc's GMRES
    default; CGS2) reach the direct solution of the bordered system."""
    case = synth.channel_case(16, 12, 16, seed=3, spheres=[(math.pi, 0.0, math.pi / 2, 0.6)], levels=3)
    grid = case.grid
    d, M, g, coef = _setup(grid)
    u = case.ucont.copy()
    O.volume_flux(d, 1, u, grid.nvert, M)
    b, _ = O.rhs(d, u, grid.nvert)
    mg = O.MG(d, grid.coor, grid.nvert, 3)
    x, info = mg.fgmres(b, rtol=1e-13, maxit=300, orth=orth)
    assert info["converged"]
    A, gid = O.csr(d, coef, grid.nvert)
    n = A.shape[0]
    mask = gid >= 0
    mask[0, :, :] = mask[-1, :, :] = False
    mask[:, :, 0] = mask[:, :, -1] = False
    mask[:, 0, :] = mask[:, -1, :] = False
    bv = np.zeros(n)
    bv[gid[mask]] = b[mask]
    one = sp.csr_matrix(np.ones((n, 1)))
    B = sp.bmat([[A, one], [one.T, None]]).tocsc()
    xs = spl.spsolve(B, np.concatenate([bv, [0.0]]))[:n]
    xv = np.zeros(n)
    xv[gid[mask]] = x[mask]
    xv -= xv.mean()
    assert np.linalg.norm(xv - xs) / np.linalg.norm(xs) < 1e-9


def test_full_step_divergence_free():
    case = synth.c2_sphere(scale=8)
    r = O.projection_step(case.grid, case.ucont, levels=case.levels, immersed=1, rtol=1e-12)
    assert r["info"]["converged"]
    assert r["divmax"] < 1e-8
    assert abs(r["flux"][2]) < 1e-12  # IB net flux after the balance


def test_volume_flux_balance():
    case = synth.c2_sphere(scale=8)
    d = O.dims_of(case.grid)
    M = O.form_metrics(d, case.grid.coor)
    u = case.ucont.copy()
    fa = O.volume_flux(d, 1, u, case.grid.nvert, M)
    assert abs(fa[0]) > 1e-6 and fa[1] > 0
    assert abs(fa[2]) < 1e-13 * max(1.0, abs(fa[0]))
    assert np.isclose(fa[1], fa[3])


def test_transfer_operators_preserve_constants():
    grid = _grid(16, 8, 16)
    d = O.dims_of(grid)
    mg = O.MG(d, grid.coor, grid.nvert, 2)
    f = np.ones(grid.nvert.shape)
    rc = mg.restrict(1, f)
    assert np.allclose(rc[1:-1, 1:-1, 1:-1], 1.0)
    dc = mg.level_dims(0)
    pc = mg.prolong(1, np.ones((dc.mz, dc.my, dc.mx)))
    assert np.allclose(pc[1:-1, 1:-1, 1:-1], 1.0)


def test_nvert_restriction_sandwich():
    """A coarse cell becomes solid only if all 8 children are; fluid cells
    hemmed in on all three axes are filled in place in k, j, i order."""
    f = O.Dims(10, 10, 10, 0, 0, 0)
    c = O.Dims()
    O.lib().orc_coarse_dims(f, 0, 0, 0, c)
    assert (c.mx, c.my, c.mz) == (6, 6, 6)
    nf = np.zeros((10, 10, 10))
    # solid blocks at coarse cells (2,2,1), (2,2,3), (2,1,2), (2,3,2), (1,2,2), (3,2,2): ring around (2,2,2)
    for (ci, cj, ck) in [(1, 2, 2), (3, 2, 2), (2, 1, 2), (2, 3, 2), (2, 2, 1), (2, 2, 3)]:
        nf[2 * ck - 1:2 * ck + 1, 2 * cj - 1:2 * cj + 1, 2 * ci - 1:2 * ci + 1] = 4.0
    nc = np.zeros((6, 6, 6))
    O.lib().orc_nvert_restrict(f, c, 0, 0, 0, O._p(nf), O._p(nc))
    assert nc[2, 2, 1] == 1 and nc[2, 2, 3] == 1 and nc[1, 2, 2] == 1
    assert nc[2, 2, 2] == 1  # sandwiched on every axis
    assert nc[1, 1, 1] == 0
