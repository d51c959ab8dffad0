"""The committed golden fixtures (tests/golden/golden_small.npz, made by
tests/golden/make_golden.py) against the oracle: the regenerated inputs hash
to the stored digest; metrics, operator coefficients and RHS are reproduced
bit for bit; the tight solve's phi, pressure and fluxes to rounding (the
oracle's OpenMP reductions depend on the thread count)."""
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


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_golden(name):
    case = CASES[name]
    assert str(GOLD[f"{name}/digest"]) == MG.input_digest(case)
    out = MG.outputs(case)
    for k in ("aj", "coef", "b"):
        assert np.array_equal(out[k], GOLD[f"{name}/{k}"]), k
    fl = fluid_interior(case.grid.nvert)
    a, r = out["phi"][fl], GOLD[f"{name}/phi"][fl]
    a, r = a - a.mean(), r - r.mean()
    assert np.linalg.norm(a - r) <= 1e-10 * np.linalg.norm(r)
    for k in ("p", "ucont"):
        g = GOLD[f"{name}/{k}"]
        assert np.abs(out[k] - g).max() <= 1e-10 * np.abs(g).max(), k
    assert out["divmax"] < 1e-10 and GOLD[f"{name}/divmax"] < 1e-10
