"""The oracle restatement (oracle/vfs_oracle.c) against the reference's own
code: the path's functions compiled unmodified from the reference's sources
(oracle/ref.mk, single-rank PETSc/HYPRE/MPI stand-ins in oracle/ref_stub/)
and run on the same seeded grids.  Every comparison is bit for bit:

* FormMetrics (metrics.c:4-1290): all 17 metric fields, ghosts included;
* setup_lidx2 + PoissonLHSNew (poisson.c:187-334, 976-1691): the fluid
  numbering and every (row, column, value) handed to HYPRE;
* VolumeFlux (poisson.c:2634-2828, 2898-3240): the balanced fluxes;
* PoissonRHS2_hypre and PoissonRHS2 (poisson_hypre.c:272-477,
  poisson.c:1789-1915): the right-hand side without and with the fix;
* Convert_Phi2_Phi, UpdatePressure, Projection, Contra2Cart, Divergence
  (poisson.c:97-185, 2473-2632, 2122-2470; rhs.c:50; main.c:1244-1390);
* MyNvertRestriction, MyRestriction, MyInterpolation (poisson.c:2004-2106,
  364-471, 526-669) on every level, with and without semi-coarsening.

Then the whole step: the oracle's FGMRES + GMG solve against a direct solve
of the reference's own matrix, through the reference's post-processing.

Needs the reference's sources (the checker is built from them); skipped
where they are absent.
"""
import math

import numpy as np
import pytest

import oracle as O
import ref as R
from vfs_v3p2_gb300 import synth

import refstep

pytestmark = pytest.mark.skipif(not R.available(), reason="reference sources absent: the checker cannot be built")


def fractional(case):
    case.grid.nvert = case.grid.nvert * 0.35  # 0, 0.35 (IB band: fluid for the numbering) and 1.4 (solid)
    return case


def walled():
    case = synth.channel_case(16, 8, 12, seed=31, levels=2)
    nv = case.grid.nvert
    nv[4:8, 1:-1, 7] = 4.0  # a wall across the channel at i = 7
    synth.periodic_fill_scalar(nv)
    case.immersed = 1
    return case


CASES = {
    "channel": lambda: synth.channel_case(16, 12, 16, seed=11, levels=3),
    "sphere": lambda: synth.channel_case(16, 12, 16, seed=12, spheres=[(math.pi, 0.0, math.pi / 2, 0.6)], sigma=0.5,
                                         levels=3),
    "uniform": lambda: synth.channel_case(12, 8, 8, seed=13, beta=0.0, skew=0.0, levels=2),
    "ragged": lambda: synth.channel_case(20, 6, 12, seed=14, levels=2),
    "fractional_nvert": lambda: fractional(synth.channel_case(16, 12, 16, seed=15,
                                                              spheres=[(math.pi, 0.0, math.pi / 2, 0.6)],
                                                              sigma=0.5, levels=2)),
    "terrain": lambda: synth.c3_terrain(scale=16),
    "walled": walled,
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    return request.param, CASES[request.param]()


def fluid_interior(nvert):
    fl = nvert < 0.1
    fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = False, False, False, False, False, False
    return fl


def test_metrics_and_operator_bitexact(case):
    name, c = case
    g = c.grid
    d = O.dims_of(g)
    rg = R.RefGrid(g, immersed=c.immersed)
    Mr = rg.form_metrics()
    Mo = O.form_metrics(d, g.coor)
    assert np.array_equal(Mr, Mo)
    rows, cols, vals, gid = rg.lhs()
    coef = O.lhs(d, O.gtensor(d, Mo), g.nvert)
    A, gid_o = O.csr(d, coef, g.nvert)
    assert np.array_equal(gid_o.astype(np.float64), gid)
    Ac = A.tocoo()
    order = np.lexsort((Ac.col, Ac.row))
    assert A.nnz == len(vals)
    assert np.array_equal(Ac.row[order], rows)
    assert np.array_equal(Ac.col[order], cols)
    assert np.array_equal(Ac.data[order], vals)


def test_flux_rhs_projection_divergence_bitexact(case):
    name, c = case
    g = c.grid
    d = O.dims_of(g)
    rg = R.RefGrid(g, immersed=c.immersed)
    rg.form_metrics()
    _, _, _, gid = rg.lhs()
    M = O.form_metrics(d, g.coor)
    u_r, flux_r = rg.volume_flux(c.ucont)
    u_o = c.ucont.copy()
    flux_o = O.volume_flux(d, c.immersed, u_o, g.nvert, M)
    assert np.array_equal(u_r, u_o)
    if c.immersed:  # VolumeFlux reports the IB flux and area after its balance
        assert flux_r[1] == flux_o[3] and abs(flux_r[0] - flux_o[2]) <= 1e-12 * abs(flux_o[0]) + 1e-300
    inter = np.zeros(g.nvert.shape, bool)
    inter[1:-1, 1:-1, 1:-1] = True
    rowcells = inter & (gid >= 0)
    idx = gid[rowcells].astype(int)
    for meanfix, got in ((False, rg.rhs(u_o)), (True, rg.rhs2(u_o))):
        b, _ = O.rhs(d, u_o, g.nvert, meanfix=meanfix)
        compact = np.zeros(rg.n_fluid)
        compact[idx] = b[rowcells]
        assert np.array_equal(compact, got), f"meanfix={meanfix}"
    rng = np.random.default_rng(3)
    phi2 = rng.normal(size=rg.n_fluid)
    phi_r = rg.phi2_to_phi(phi2)
    phi_o = np.zeros(g.nvert.shape)
    phi_o[rowcells] = phi2[idx]
    O.phi_finish(d, g.nvert, phi_o)
    assert np.array_equal(phi_r, phi_o)
    p0 = rng.normal(size=g.nvert.shape)
    p_r, u2_r, ucat_r = rg.update_and_project(phi_r, p0, u_o)
    p_o = p0.copy()
    O.update_pressure(d, g.nvert, phi_o, p_o)
    u2_o = u_o.copy()
    O.projection(d, M, g.nvert, phi_o, u2_o)
    assert np.array_equal(p_r, p_o)
    assert np.array_equal(u2_r, u2_o)
    ucat_o = O.contra2cart(d, M, g.nvert, u2_o)
    fl = fluid_interior(g.nvert)
    assert np.array_equal(ucat_r[fl], ucat_o[fl])
    assert rg.divergence(u2_o) == O.divergence(d, u2_o, O.metric(M, d, "aj"), g.nvert)


@pytest.mark.parametrize("semi", [(0, 0, 0), (0, 1, 0), (1, 0, 0), (0, 0, 1)])
def test_multigrid_transfers_bitexact(semi):
    c = synth.channel_case(16, 16, 16, seed=21, spheres=[(math.pi, 0.0, math.pi / 2, 0.7)], sigma=0.5, levels=3)
    g = c.grid
    d = O.dims_of(g)
    mg = O.MG(d, g.coor, g.nvert, c.levels, semi=semi)
    fine = R.RefGrid(g, immersed=1)
    try:
        for lev in range(c.levels - 1, 0, -1):
            cd = mg.level_dims(lev - 1)
            shape = (cd.mz, cd.my, cd.mx)
            cg = synth.Grid(cd.mx - 2, cd.my - 2, cd.mz - 2, mg.level_array(lev - 1, "coor").reshape(shape + (3,)),
                            mg.level_array(lev - 1, "nvert").reshape(shape), g.i_periodic, g.j_periodic,
                            g.k_periodic)
            coarse = R.RefGrid(cg, immersed=1)
            fine.link_coarse(coarse, semi=semi, coarse_level=lev - 1)
            assert np.array_equal(fine.nvert_restrict(), mg.level_array(lev - 1, "nvert").reshape(shape))
            rng = np.random.default_rng(lev)
            xf = rng.normal(size=fine.shape)
            assert np.array_equal(fine.restrict(xf), mg.restrict(lev, xf))
            xc = rng.normal(size=coarse.shape)
            assert np.array_equal(fine.interpolate(xc), mg.prolong(lev, xc))
            fine = coarse
    finally:
        mg.close()


def test_projection_step_matches_reference(case):
    """The oracle's step (its FGMRES + GMG to rtol 1e-13) against the
    reference's functions around a direct solve of the reference's matrix."""
    name, c = case
    g = c.grid
    ref = refstep.reference_step(c)
    got = O.projection_step(g, c.ucont, levels=c.levels, immersed=c.immersed, rtol=1e-13, maxit=400, orth=2)
    fl = fluid_interior(g.nvert)
    a, r = got["phi"][fl] - got["phi"][fl].mean(), ref["phi"][fl] - ref["phi"][fl].mean()
    assert np.linalg.norm(a - r) <= 1e-10 * np.linalg.norm(r)
    assert np.abs(got["p"][fl] - ref["p"][fl]).max() <= 1e-10 * np.abs(ref["p"][fl]).max()
    assert np.abs(got["ucont"] - ref["ucont"]).max() <= 1e-10 * np.abs(ref["ucont"]).max()
    if name == "walled":
        # a wall splits the fluid in two: the reference's single mean fix
        # (poisson.c:1879-1903) leaves each region's net flux, so neither step
        # is divergence free there, and both leave the same divergence
        assert abs(got["divmax"] - ref["divmax"]) <= 1e-10 * ref["divmax"]
        return
    # both solve the reference's matrix, whose drop rule (|v| <= 1e-10 on the
    # unscaled entries, poisson.c:1607-1616) leaves a divergence floor near
    # 1e-9 where aj is large (the terrain grid's thin cells)
    assert got["divmax"] < 1e-8 and ref["divmax"] < 1e-8
