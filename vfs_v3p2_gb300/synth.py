"""Seeded synthetic inputs for the pressure-projection step.

The reference reads its grid from grid.dat (init.c:251-392), marks immersed
bodies with a ray-cast search (ibm.c) and produces the intermediate velocity
with its momentum solver.  None of those inputs ship with the reference, so
this module builds seeded stand-ins with the shapes of the five workloads:

* channel grid: x, z uniform on [0, 2pi] x [0, pi], tanh wall stretching in
  y on [-1, 1], x-lines skewed by ``skew * sin(z)``; periodic in x and z,
  walls in y;
* terrain grid: y-lines stretched from a Gaussian hill h(x, z) up to y = 1;
* immersed spheres marked in ``nvert`` with the reference's codes (solid
  cells 4, fluid cells touching a solid face-neighbour 1, fluid 0; the
  pressure system keeps only ``nvert < 0.1``, poisson.c:1167);
* contravariant face fluxes ``ucont`` (AoS ``[mz][my][mx][3]``), zero on the
  wall faces j = 0 and j = nj, periodic ghosts synced.

All arrays use the reference's DMDA layout: extents ``mx = ni + 2`` etc.,
i fastest, node coordinates valid for indices 0..ni (init.c:340-380).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class Grid:
    """One structured grid in the reference's ghosted layout."""

    ni: int
    nj: int
    nk: int
    coor: np.ndarray  # [mz, my, mx, 3] node coordinates
    nvert: np.ndarray  # [mz, my, mx]
    i_periodic: int = 1
    j_periodic: int = 0
    k_periodic: int = 1

    @property
    def shape(self):
        return (self.nk + 2, self.nj + 2, self.ni + 2)

    @property
    def dims(self):
        mz, my, mx = self.shape
        return mx, my, mz


def _stretch(eta: np.ndarray, beta: float) -> np.ndarray:
    """tanh stretching of eta in [0, 1] onto [-1, 1]; beta == 0 is uniform."""
    if beta == 0.0:
        return 2.0 * eta - 1.0
    return np.tanh(beta * (2.0 * eta - 1.0)) / math.tanh(beta)


def channel_coords(ni: int, nj: int, nk: int, beta: float = 2.0, skew: float = 0.05,
                   lx: float = 2 * math.pi, lz: float = math.pi) -> np.ndarray:
    """Node coordinates of the skewed, wall-stretched channel grid."""
    mz, my, mx = nk + 2, nj + 2, ni + 2
    coor = np.zeros((mz, my, mx, 3))
    x = lx * np.arange(ni + 1) / ni
    y = _stretch(np.arange(nj + 1) / nj, beta)
    z = lz * np.arange(nk + 1) / nk
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    coor[: nk + 1, : nj + 1, : ni + 1, 0] = X + skew * np.sin(Z)
    coor[: nk + 1, : nj + 1, : ni + 1, 1] = Y
    coor[: nk + 1, : nj + 1, : ni + 1, 2] = Z
    return coor


def hill(x: np.ndarray, z: np.ndarray) -> np.ndarray:
    return 0.25 * np.exp(-((x - math.pi) ** 2 + (z - math.pi / 2) ** 2) / 0.5)


def terrain_coords(ni: int, nj: int, nk: int, beta: float = 2.5) -> np.ndarray:
    """Terrain-following grid over a Gaussian hill, bottom-clustered in y."""
    mz, my, mx = nk + 2, nj + 2, ni + 2
    coor = np.zeros((mz, my, mx, 3))
    x = 2 * math.pi * np.arange(ni + 1) / ni
    z = math.pi * np.arange(nk + 1) / nk
    eta = np.arange(nj + 1) / nj
    s = 1.0 + np.tanh(beta * (eta - 1.0)) / math.tanh(beta)
    Z, E, X = np.meshgrid(z, s, x, indexing="ij")
    h = hill(X, Z)
    coor[: nk + 1, : nj + 1, : ni + 1, 0] = X
    coor[: nk + 1, : nj + 1, : ni + 1, 1] = h + (1.0 - h) * E
    coor[: nk + 1, : nj + 1, : ni + 1, 2] = Z
    return coor


def cell_centres(coor: np.ndarray) -> np.ndarray:
    """Cell centres (metrics.c:80-103) on the full ghosted extent (ghosts 0)."""
    mz, my, mx, _ = coor.shape
    c = np.zeros_like(coor)
    n = coor
    c[1:-1, 1:-1, 1:-1] = 0.125 * (
        n[1:-1, 1:-1, 1:-1] + n[1:-1, :-2, 1:-1] + n[:-2, 1:-1, 1:-1] + n[:-2, :-2, 1:-1]
        + n[1:-1, 1:-1, :-2] + n[1:-1, :-2, :-2] + n[:-2, 1:-1, :-2] + n[:-2, :-2, :-2])
    return c


def periodic_fill_scalar(a: np.ndarray, ip=1, jp=0, kp=1) -> np.ndarray:
    """Copy interior partners into periodic ghost cells (index 0 <- m-2, m-1 <- 1)."""
    if ip:
        a[:, :, 0] = a[:, :, -2]
        a[:, :, -1] = a[:, :, 1]
    if jp:
        a[:, 0, :] = a[:, -2, :]
        a[:, -1, :] = a[:, 1, :]
    if kp:
        a[0, :, :] = a[-2, :, :]
        a[-1, :, :] = a[1, :, :]
    return a


def sphere_nvert(coor: np.ndarray, spheres, ip=1, jp=0, kp=1) -> np.ndarray:
    """nvert for immersed spheres [(cx, cy, cz, r), ...]: 4 inside, 1 for fluid
    cells with a solid face-neighbour, 0 elsewhere; periodic ghosts copied."""
    mz, my, mx, _ = coor.shape
    cent = cell_centres(coor)
    solid = np.zeros((mz, my, mx), dtype=bool)
    for (cx, cy, cz, r) in spheres:
        d2 = (cent[..., 0] - cx) ** 2 + (cent[..., 1] - cy) ** 2 + (cent[..., 2] - cz) ** 2
        inside = d2 < r * r
        inside[0, :, :] = inside[-1, :, :] = False
        inside[:, 0, :] = inside[:, -1, :] = False
        inside[:, :, 0] = inside[:, :, -1] = False
        solid |= inside
    nv = np.zeros((mz, my, mx))
    nv[solid] = 4.0
    nb = np.zeros_like(solid)
    nb[:, :, 1:] |= solid[:, :, :-1]
    nb[:, :, :-1] |= solid[:, :, 1:]
    nb[:, 1:, :] |= solid[:, :-1, :]
    nb[:, :-1, :] |= solid[:, 1:, :]
    nb[1:, :, :] |= solid[:-1, :, :]
    nb[:-1, :, :] |= solid[1:, :, :]
    ib = nb & ~solid
    ib[0, :, :] = ib[-1, :, :] = False
    ib[:, 0, :] = ib[:, -1, :] = False
    ib[:, :, 0] = ib[:, :, -1] = False
    nv[ib] = 1.0
    return periodic_fill_scalar(nv, ip, jp, kp)


def face_area_vectors(coor: np.ndarray):
    """Area vectors of the i-, j- and k-faces from the node coordinates (half
    cross product of the face diagonals).  Face (k, j, i) of each family sits
    at the + side of cell (k, j, i); entries without a full face are zero."""
    n = coor
    mz, my, mx, _ = n.shape
    A = np.zeros((3, mz, my, mx, 3))
    # i-face at node plane i, spanned by nodes (j-1..j, k-1..k)
    d1 = n[1:, 1:, :] - n[:-1, :-1, :]
    d2 = n[1:, :-1, :] - n[:-1, 1:, :]
    A[0, 1:, 1:, :] = 0.5 * np.cross(d2, d1)
    # j-face at node plane j, spanned by nodes (i-1..i, k-1..k)
    d1 = n[1:, :, 1:] - n[:-1, :, :-1]
    d2 = n[:-1, :, 1:] - n[1:, :, :-1]
    A[1, 1:, :, 1:] = 0.5 * np.cross(d2, d1)
    # k-face at node plane k, spanned by nodes (i-1..i, j-1..j)
    d1 = n[:, 1:, 1:] - n[:, :-1, :-1]
    d2 = n[:, 1:, :-1] - n[:, :-1, 1:]
    A[2, :, 1:, 1:] = 0.5 * np.cross(d2, d1)
    return A


def face_centres(coor: np.ndarray):
    n = coor
    mz, my, mx, _ = n.shape
    F = np.zeros((3, mz, my, mx, 3))
    F[0, 1:, 1:, :] = 0.25 * (n[1:, 1:, :] + n[:-1, 1:, :] + n[1:, :-1, :] + n[:-1, :-1, :])
    F[1, 1:, :, 1:] = 0.25 * (n[1:, :, 1:] + n[:-1, :, 1:] + n[1:, :, :-1] + n[:-1, :, :-1])
    F[2, :, 1:, 1:] = 0.25 * (n[:, 1:, 1:] + n[:, :-1, 1:] + n[:, 1:, :-1] + n[:, :-1, :-1])
    return F


def finish_ucont(u: np.ndarray, ni: int, nj: int, nk: int, ip=1, jp=0, kp=1) -> np.ndarray:
    """Zero the flux on the y-walls and on faces outside the domain, then sync
    periodic ghost faces the way Projection does (poisson.c:2398-2437)."""
    mz, my, mx = nk + 2, nj + 2, ni + 2
    out = np.zeros_like(u)
    # valid faces: x-face i in [0, ni] for interior j, k; etc.
    out[1:-1, 1:-1, 0:mx - 1, 0] = u[1:-1, 1:-1, 0:mx - 1, 0]
    out[1:-1, 0:my - 1, 1:-1, 1] = u[1:-1, 0:my - 1, 1:-1, 1]
    out[0:mz - 1, 1:-1, 1:-1, 2] = u[0:mz - 1, 1:-1, 1:-1, 2]
    if not jp:
        out[:, 0, :, 1] = 0.0
        out[:, my - 2, :, 1] = 0.0
    if ip:
        out[:, :, 0, 0] = out[:, :, mx - 2, 0]
        out[:, :, mx - 1, 0] = out[:, :, 1, 0]
    if kp:
        out[0, :, :, 2] = out[mz - 2, :, :, 2]
        out[mz - 1, :, :, 2] = out[1, :, :, 2]
    return out


def gaussian_ucont(ni, nj, nk, rng, sigma=1.0, ip=1, jp=0, kp=1) -> np.ndarray:
    """U ~ N(0, sigma^2) drawn directly per face."""
    u = rng.normal(0.0, sigma, size=(nk + 2, nj + 2, ni + 2, 3))
    return finish_ucont(u, ni, nj, nk, ip, jp, kp)


def profile_ucont(coor: np.ndarray, ni, nj, nk, rng, profile, sigma, ip=1, jp=0, kp=1) -> np.ndarray:
    """Cartesian profile u(x, y, z) plus N(0, sigma^2) per component, turned
    into contravariant face fluxes U^xi = u . A_i (and likewise for j, k)."""
    A = face_area_vectors(coor)
    F = face_centres(coor)
    u = np.zeros(coor.shape)
    for f in range(3):
        vel = profile(F[f]) + rng.normal(0.0, sigma, size=F[f].shape)
        u[..., f] = np.sum(vel * A[f], axis=-1)
    return finish_ucont(u, ni, nj, nk, ip, jp, kp)


def poiseuille(P):
    v = np.zeros_like(P)
    v[..., 0] = 1.0 - P[..., 1] ** 2
    return v


def loglaw(P):
    v = np.zeros_like(P)
    h = hill(P[..., 0], P[..., 2])
    v[..., 0] = np.log1p(30.0 * np.maximum(P[..., 1] - h, 0.0)) / math.log(31.0)
    return v


# ---------------------------------------------------------------------------
# The named workloads.
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Case:
    name: str
    grid: Grid
    ucont: np.ndarray
    immersed: int
    levels: int
    dt: float = 0.04
    st: float = 1.0
    coeff: float = 1.0


def channel_case(ni, nj, nk, seed, beta=2.0, skew=0.05, spheres=(), sigma=1.0, levels=3,
                 profile=None, name="channel") -> Case:
    rng = np.random.default_rng(seed)
    coor = channel_coords(ni, nj, nk, beta, skew)
    nv = sphere_nvert(coor, spheres) if spheres else np.zeros((nk + 2, nj + 2, ni + 2))
    if profile is None:
        u = gaussian_ucont(ni, nj, nk, rng, sigma)
    else:
        u = profile_ucont(coor, ni, nj, nk, rng, profile, sigma)
    g = Grid(ni, nj, nk, coor, nv)
    return Case(name, g, u, 1 if spheres else 0, levels)


def c1_channel(scale: int = 1) -> Case:
    """Plain FP64 channel, 64^3 cells (scale divides each extent)."""
    n = 64 // scale
    return channel_case(n, n, n, seed=1001, levels=3, name=f"channel_{n}x{n}x{n}")


def c2_sphere(scale: int = 1) -> Case:
    """256x128x128 channel with a sphere r = 0.3 at (pi, 0, pi/2), Poiseuille
    profile plus N(0, 0.1^2) noise, 5 MG levels (scale divides each extent)."""
    ni, nj, nk = 256 // scale, 128 // scale, 128 // scale
    levels = 5
    while levels > 1 and min(ni, nj, nk) >> (levels - 1) < 4:
        levels -= 1
    return channel_case(ni, nj, nk, seed=1002, spheres=[(math.pi, 0.0, math.pi / 2, 0.3)], sigma=0.1,
                        levels=levels, profile=poiseuille, name=f"sphere_{ni}x{nj}x{nk}")


def c3_terrain(scale: int = 1) -> Case:
    """512x256x256 terrain-following grid over the Gaussian hill, log-law
    profile plus N(0, 0.05^2) noise."""
    ni, nj, nk = 512 // scale, 256 // scale, 256 // scale
    rng = np.random.default_rng(1003)
    coor = terrain_coords(ni, nj, nk, 2.5)
    u = profile_ucont(coor, ni, nj, nk, rng, loglaw, 0.05)
    levels = 5
    while levels > 1 and min(ni, nj, nk) >> (levels - 1) < 4:
        levels -= 1
    g = Grid(ni, nj, nk, coor, np.zeros((nk + 2, nj + 2, ni + 2)))
    return Case(f"terrain_{ni}x{nj}x{nk}", g, u, 0, levels)


def _round8(v):
    return max(8, int(round(v / 8.0)) * 8)


def mg_levels(ni: int, nj: int, nk: int, max_levels: int = 5, min_cells: int = 4) -> int:
    """Deepest geometric hierarchy (full coarsening) for which every axis
    halves evenly down to the coarsest level and keeps >= min_cells cells."""
    levels = 1
    while levels < max_levels and all(n % (1 << levels) == 0 and n >> levels >= min_cells for n in (ni, nj, nk)):
        levels += 1
    return levels


def c4_batch(count: int = 64, seed: int = 1004, lo=(32, 32, 32), hi=(192, 96, 96)):
    """Uneven batch: per-axis log-uniform extents in [lo, hi] rounded to a
    multiple of 8, skew U[0, 0.1], beta U[1.5, 3], 0-3 spheres r U[0.1, 0.3],
    U ~ N(0, 1)."""
    rng = np.random.default_rng(seed)
    cases = []
    for r in range(count):
        ext = [_round8(math.exp(rng.uniform(math.log(a), math.log(b)))) for a, b in zip(lo, hi)]
        skew = rng.uniform(0.0, 0.1)
        beta = rng.uniform(1.5, 3.0)
        ns = int(rng.integers(0, 4))
        sph = []
        for _ in range(ns):
            rad = rng.uniform(0.1, 0.3)
            sph.append((rng.uniform(1.0, 2 * math.pi - 1.0), rng.uniform(-0.5, 0.5), rng.uniform(0.6, math.pi - 0.6), rad))
        ni, nj, nk = ext
        levels = mg_levels(ni, nj, nk)
        cases.append(channel_case(ni, nj, nk, seed=1_000_000 + r, beta=beta, skew=skew, spheres=sph, levels=levels,
                                  name=f"batch{r}_{ni}x{nj}x{nk}"))
    return cases
