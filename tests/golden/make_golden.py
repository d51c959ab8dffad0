"""Generates tests/golden/golden_small.npz: outputs of the CPU oracle (the
restatement of the reference's pressure path) for two small seeded cases.
The reference itself cannot be built here (PETSc/HYPRE/MPI absent), so these
fixtures anchor the oracle against drift and give the CUDA path fixed
targets.  Inputs are not stored: they are regenerated from the seeded
synthetic generators, and a checksum of them is stored to detect generator
drift.

    python tests/golden/make_golden.py
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


def cases():
    from vfs_v3p2_gb300 import synth
    return {
        "channel_12x8x8": synth.channel_case(12, 8, 8, seed=2101, levels=2),
        "sphere_16x8x8": synth.channel_case(16, 8, 8, seed=2102, spheres=[(math.pi, 0.0, math.pi / 2, 0.7)],
                                            sigma=0.5, levels=2),
    }


def input_digest(case) -> str:
    h = hashlib.sha256()
    for a in (case.grid.coor, case.grid.nvert, case.ucont):
        h.update(np.ascontiguousarray(a, dtype=np.float64).tobytes())
    return h.hexdigest()


def outputs(case):
    import oracle as O
    g = case.grid
    d = O.dims_of(g)
    M = O.form_metrics(d, g.coor)
    G = O.gtensor(d, M)
    coef = O.lhs(d, G, g.nvert)
    r = O.projection_step(g, case.ucont, levels=case.levels, immersed=case.immersed, rtol=1e-13, maxit=400, orth=1)
    return {"aj": O.metric(M, d, "aj"), "coef": coef, "b": r["b"], "phi": r["phi"], "p": r["p"],
            "ucont": r["ucont"], "divmax": np.array(r["divmax"])}


def main():
    out = {}
    for name, c in cases().items():
        out[f"{name}/digest"] = np.array(input_digest(c))
        for k, v in outputs(c).items():
            out[f"{name}/{k}"] = v
    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **out)


if __name__ == "__main__":
    main()
