"""The oracle against the committed golden fixtures (tests/golden/golden_small.npz),
which tests/golden/make_golden.py generated from the reference's own code
(compiled unmodified from its sources): the regenerated inputs hash to the
stored digest; metrics, the operator's entries and numbering and the
right-hand side are reproduced bit for bit; the tight solve's phi, pressure
and fluxes to rounding (a direct solve stands in for the reference's HYPRE
solve, and the oracle's OpenMP reductions depend on the thread count).
These run wherever the reference's sources are absent, too."""
import os
import sys

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as MG  # noqa: E402

GOLD = np.load(os.path.join(HERE, "golden", "golden_small.npz"))
CASES = MG.cases()


def fluid_interior(nvert):
    fl = nvert < 0.1
    fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = False, False, False, False, False, False
    return fl


def golden_csr(name):
    rows, cols, vals = (GOLD[f"{name}/lhs_{k}"] for k in ("rows", "cols", "vals"))
    return rows, cols, vals


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_reference_golden(name):
    assert str(GOLD[f"{name}/digest"]) == MG.input_digest(CASES[name])  # generator drift (this machine)
    case = MG.stored_case(GOLD, name)
    g = case.grid
    d = O.dims_of(g)
    M = O.form_metrics(d, g.coor)
    assert np.array_equal(M, GOLD[f"{name}/M"])
    coef = O.lhs(d, O.gtensor(d, M), g.nvert)
    A, gid = O.csr(d, coef, g.nvert)
    assert np.array_equal(gid.astype(np.float64), GOLD[f"{name}/gid"])
    Ac = A.tocoo()
    order = np.lexsort((Ac.col, Ac.row))
    rows, cols, vals = golden_csr(name)
    assert np.array_equal(Ac.row[order], rows) and np.array_equal(Ac.col[order], cols)
    assert np.array_equal(Ac.data[order], vals)
    r = O.projection_step(g, case.ucont, levels=case.levels, immersed=case.immersed, rtol=1e-13, maxit=400, orth=1)
    inter = np.zeros(g.nvert.shape, bool)
    inter[1:-1, 1:-1, 1:-1] = True
    rowcells = inter & (gid >= 0)
    compact = np.zeros(len(GOLD[f"{name}/b"]))
    compact[gid[rowcells]] = r["b"][rowcells]
    assert np.array_equal(compact, GOLD[f"{name}/b"])
    fl = fluid_interior(g.nvert)
    a, ref = r["phi"][fl], GOLD[f"{name}/phi"][fl]
    a, ref = a - a.mean(), ref - ref.mean()
    assert np.linalg.norm(a - ref) <= 1e-10 * np.linalg.norm(ref)
    for k in ("p", "ucont"):
        gold = GOLD[f"{name}/{k}"]
        assert np.abs(r[k] - gold).max() <= 1e-10 * np.abs(gold).max(), k
    assert r["divmax"] < 1e-9 and GOLD[f"{name}/divmax"] < 1e-9
