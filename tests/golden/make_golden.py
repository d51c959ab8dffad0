"""Generates tests/golden/golden_small.npz from the reference's own code: the
pressure-path functions compiled unmodified from the reference's sources
(oracle/ref.mk, run through oracle/ref.py and tests/refstep.py) on small
seeded grids.  Stored per case:

* M: FormMetrics' 17 fields (metrics.c:4-1290) in the oracle's 43-array pack;
* lhs_rows, lhs_cols, lhs_vals, gid: every entry PoissonLHSNew hands to
  HYPRE (poisson.c:976-1691) in its compact fluid numbering (setup_lidx2);
* b: PoissonRHS2 of the balanced fluxes (poisson.c:1789-1915);
* phi, p, ucont, divmax: the step through the reference's Remove_Nullspace,
  Convert_Phi2_Phi, UpdatePressure, Projection and Divergence around a direct
  solve of its matrix (HYPRE itself is not part of the sources).

The inputs (node coordinates, nvert, fluxes) are stored too: the seeded
generators use numpy's exp and tanh, whose last bit may differ between
machines, so a check elsewhere runs on the stored inputs; a digest of the
inputs detects generator drift where they are regenerated.  The fixtures let the oracle (tests/test_golden_cpu.py) and the CUDA path
(tests/test_golden_gpu.py) be checked against the reference where its
sources are absent.

    python tests/golden/make_golden.py     (needs the reference's sources)
"""
import hashlib
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.dirname(HERE))


def cases():
    from vfs_v3p2_gb300 import synth
    return {
        "channel_12x8x8": synth.channel_case(12, 8, 8, seed=2101, levels=2),
        "sphere_16x8x8": synth.channel_case(16, 8, 8, seed=2102, spheres=[(math.pi, 0.0, math.pi / 2, 0.7)],
                                            sigma=0.5, levels=2),
        "terrain_16x8x8": synth.c3_terrain(scale=32),
    }


def input_digest(case) -> str:
    h = hashlib.sha256()
    for a in (case.grid.coor, case.grid.nvert, case.ucont):
        h.update(np.ascontiguousarray(a, dtype=np.float64).tobytes())
    return h.hexdigest()


def stored_case(gold, name):
    """The case with the inputs stored in the fixtures (bit-identical on any machine)."""
    c = cases()[name]
    c.grid.coor = np.array(gold[f"{name}/in_coor"])
    c.grid.nvert = np.array(gold[f"{name}/in_nvert"])
    c.ucont = np.array(gold[f"{name}/in_ucont"])
    return c


def reference_outputs(case):
    import refstep
    r = refstep.reference_step(case)
    return {"M": r["M"], "lhs_rows": r["rows"], "lhs_cols": r["cols"], "lhs_vals": r["vals"], "gid": r["gid"],
            "b": r["b"], "phi": r["phi"], "p": r["p"], "ucont": r["ucont"], "divmax": np.array(r["divmax"])}


def main():
    out = {}
    for name, c in cases().items():
        out[f"{name}/digest"] = np.array(input_digest(c))
        out[f"{name}/in_coor"] = c.grid.coor
        out[f"{name}/in_nvert"] = c.grid.nvert
        out[f"{name}/in_ucont"] = c.ucont
        for k, v in reference_outputs(c).items():
            out[f"{name}/{k}"] = v
    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **out)


if __name__ == "__main__":
    main()
