"""The reference's own pressure-projection step on one grid, run from its
unmodified sources (oracle/_ref, built by oracle/ref.mk): VolumeFlux,
PoissonRHS2 (with its compatibility fix), PoissonLHSNew's matrix, a direct
solve, Remove_Nullspace, Convert_Phi2_Phi, UpdatePressure, Projection (with
Contra2Cart) and Divergence, in the order of PoissonSolver_Hypre and
Flow_Solver (poisson_hypre.c:580-771, solvers.c:874-930).

The reference solves its assembled system with HYPRE's GMRES + BoomerAMG,
which is not part of its sources; a sparse direct solve of the same matrix
(bordered with the fluid indicator, which picks the mean-zero solution of
the singular system) stands in for its converged solve.  Test
infrastructure: used by tests/test_ref_oracle.py and tests/golden/make_golden.py.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import ref as R


def reference_step(case, p0=None):
    g = case.grid
    rg = R.RefGrid(g, immersed=case.immersed, dt=case.dt, st=case.st)
    M = rg.form_metrics()
    rows, cols, vals, gid = rg.lhs()
    n = rg.n_fluid
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    u, flux = rg.volume_flux(case.ucont)
    b = rg.rhs2(u)
    # numbered cells the reference does not assemble (0.1 < nvert < 1) have
    # empty rows and no couplings: their values are free and unused by the
    # projection; the solve pins them to zero
    empty = np.diff(A.indptr) == 0
    A = A + sp.diags(empty.astype(np.float64))
    rhs = np.where(empty, 0.0, b)
    e = (~empty).astype(np.float64).reshape(-1, 1)
    K = sp.bmat([[A, sp.csr_matrix(e)], [sp.csr_matrix(e.T), None]], format="csc")
    sol = spla.spsolve(K, np.concatenate([rhs, [0.0]]))
    phi2 = rg.remove_nullspace(sol[:n])
    phi = rg.phi2_to_phi(phi2)
    p = np.zeros(g.nvert.shape) if p0 is None else np.array(p0, dtype=np.float64)
    p, u_out, ucat = rg.update_and_project(phi, p, u)
    divmax = rg.divergence(u_out)
    return dict(M=M, rows=rows, cols=cols, vals=vals, gid=gid, b=b, phi2=phi2, phi=phi, p=p, ucont=u_out,
                ucont_balanced=u, ucat=ucat, divmax=divmax, flux=flux, handle=rg)
