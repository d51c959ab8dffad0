"""Grids cut into separate fluid regions by solid walls spanning whole
k-planes (shared by the region tests)."""
import dataclasses

import numpy as np

from vfs_v3p2_gb300 import synth


def walled_channel(walls, kp=1, ni=32, nj=16, nk=32, seed=41, levels=3):
    """A channel whose interior planes k0..k1 (1-based, inclusive) of each
    wall are solid (nvert 4) across every i and j; periodic in k when kp."""
    case = synth.channel_case(ni, nj, nk, seed=seed, levels=levels)
    nv = case.grid.nvert.copy()
    for k0, k1 in walls:
        nv[k0:k1 + 1, :, :] = 4.0
    grid = dataclasses.replace(case.grid, nvert=nv, k_periodic=kp)
    u = np.array(case.ucont)
    if not kp:
        # closed ends: no flux through the boundary k-faces, so every region
        # is balanced (open ends would carry the random inputs' imbalance)
        u[0, :, :, 2] = 0.0
        u[-2, :, :, 2] = 0.0
    return dataclasses.replace(case, grid=grid, ucont=u, name=f"walled_{len(walls)}_kp{kp}")


def expected_labels(case, walls):
    """Region label of every fluid interior cell, by k-plane."""
    g = case.grid
    mz = g.nvert.shape[0]
    solid = np.zeros(mz, bool)
    for k0, k1 in walls:
        solid[k0:k1 + 1] = True
    lab, cur, first = np.full(mz, -1), -1, None
    for k in range(1, mz - 1):
        if solid[k]:
            continue
        if k == 1 or solid[k - 1]:
            cur += 1
        lab[k] = cur
    if g.k_periodic and not solid[1] and not solid[mz - 2]:
        lab[lab == lab[mz - 2]] = lab[1]  # the last run wraps onto the first
        _, lab_c = np.unique(np.where(lab >= 0, lab, 10**6), return_inverse=True)
        lab = np.where(lab >= 0, lab_c, -1)
    return lab
