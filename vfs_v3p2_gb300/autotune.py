"""Autotuner for the batched and served solves.

Picks the smoothing schedule (pre/post y-line sweeps on the finest and on
the coarser levels, Chebyshev damping with the width of its interval, or
constant damping) and the smoother's block tile (i-columns per block).  Each
candidate is run once to warm up (graph capture) and then timed over a few
steps with U* resident; the fastest candidate whose steps all converge to
the requested max |div u| wins.

What makes a grid hard for the multigrid is mostly its wall stretching, not
its size: strongly stretched grids (tanh beta near 3) converge fastest with a
wider Chebyshev interval (the 1/16 .. 2 of a ratio of 16 and 4 + 4 sweeps cut
the worst grid of the 64-grid batch from 39 to 26 FGMRES iterations), while
the sphere and terrain grids are fastest with the default 1/3 .. 2.  Hence
the per-grid objective beside the size classes:
  tuned_params       one representative grid per size class alone (latency);
  tuned_params_grids every grid alone (latency; the per-grid settings of a
                     batch or a set of served streams);
  tuned_params_batch all of a size class's grids together as one batch
                     (vfs_projection_step_batch: throughput, where small
                     grids' launch latencies overlap and total work counts).
Results of tuned_params can be cached per class in a JSON file.
"""
from __future__ import annotations

import json
import math
import os
import time

import numpy as np

from . import capi

# (nu1, nu2, omega, smooth_cols, coarse sweeps, smoother, cheb_ratio);
# smooth_cols 0 = the kernel's own choice; coarse sweeps -1 = as on the finest
# level; omega is the damping of the "jacobi" smoother; "chebyshev" takes the
# roots on [2 / cheb_ratio, 2].  The list holds the winners of a sweep over
# the 64-grid batch, the sphere, the channel and the terrain (GB300):
# ratio 6 (the default), 10, 16 and 24 with 3 + 3 or 4 + 4 sweeps, 5 + 5
# coarse sweeps (the sphere's best), and two constant-damping schedules.
CANDIDATES = [
    (3, 3, 0.9, 0, -1, "chebyshev", 6.0), (3, 3, 0.9, 0, -1, "chebyshev", 10.0),
    (3, 3, 0.9, 0, -1, "chebyshev", 16.0), (3, 3, 0.9, 0, -1, "chebyshev", 24.0),
    (4, 4, 0.9, 0, -1, "chebyshev", 10.0), (4, 4, 0.9, 0, -1, "chebyshev", 16.0),
    (3, 3, 0.9, 0, 5, "chebyshev", 6.0), (2, 2, 0.9, 0, -1, "chebyshev", 10.0),
    (3, 3, 0.9, 0, 5, "jacobi", 6.0), (4, 4, 0.9, 16, 6, "jacobi", 6.0),
]
SMOOTHERS = {"jacobi": capi.SMOOTH_JACOBI, "chebyshev": capi.SMOOTH_CHEBYSHEV}


def apply_candidate(p: capi.SolveParams, cand):
    p.nu1, p.nu2, p.omega, p.smooth_cols = cand[:4]
    p.nu1_coarse = p.nu2_coarse = cand[4]
    p.smoother = SMOOTHERS[cand[5]]
    p.cheb_ratio = cand[6]


def candidate_entry(cand) -> dict:
    return {"nu1": cand[0], "nu2": cand[1], "omega": cand[2], "smooth_cols": cand[3], "nu_coarse": cand[4],
            "smoother": cand[5], "cheb_ratio": cand[6]}


def entry_candidate(e: dict):
    return (e["nu1"], e["nu2"], e["omega"], e["smooth_cols"], e["nu_coarse"], e.get("smoother", "jacobi"),
            float(e.get("cheb_ratio", 6.0)))


def size_class(case) -> str:
    """log2 of the interior cell count (rounded) and whether a body is present."""
    g = case.grid
    cells = g.ni * g.nj * g.nk
    body = bool((g.nvert > 0.1).any())
    return f"c{int(round(math.log2(cells)))}{'_ib' if body else ''}"


def _time_candidate(ctx, gid, case, params, steps):
    """Seconds per step, each step solving from zero: with a warm start the
    repeated step would begin at its own solution and time the cycle's cost
    alone, not the iterations a new request needs."""
    shp = case.grid.nvert.shape
    p = with_precision(params, params.precision)
    p.warm_start = 0
    ctx.set_field(gid, capi.FIELD_USTAR, case.ucont)
    ctx.set_field(gid, capi.FIELD_P, np.zeros(shp))
    info, dm = ctx.projection_step(gid, p)  # warm-up: graph capture
    if not info["converged"]:
        return math.inf
    t0 = time.perf_counter()
    for _ in range(steps):
        info, dm = ctx.projection_step(gid, p)
        if not info["converged"] or (p.div_tol > 0 and dm > p.div_tol and not info.get("div_limited")):
            return math.inf
    return (time.perf_counter() - t0) / steps


def tune_resident(ctx, gid, case, base: capi.SolveParams, candidates=CANDIDATES, steps=3):
    """Best candidate for a resident grid (LHS built) and its seconds/step;
    the grid's U* and p are reset to the case's afterwards."""
    best, best_t = None, math.inf
    for cand in candidates:
        p = capi.SolveParams()
        ctypes_copy(p, base)
        apply_candidate(p, cand)
        try:
            t = _time_candidate(ctx, gid, case, p, steps)
        except capi.VfsError:
            t = math.inf
        if t < best_t:
            best, best_t = cand, t
    _reset(ctx, [gid], [case])
    return (best if best is not None else candidates[0]), best_t


def tune_case(ctx, case, base: capi.SolveParams, candidates=CANDIDATES, steps=3):
    """Best candidate for one grid and its seconds/step."""
    g = case.grid
    gid = ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    try:
        ctx.poisson_lhs(gid)
        return tune_resident(ctx, gid, case, base, candidates, steps)
    finally:
        ctx.grid_destroy(gid)


def tuned_params_cases(ctx, cases, base: capi.SolveParams, steps=2):
    """Per-case SolveParams, every case tuned alone on a grid of its own
    (created and destroyed here); returns the list and a table by case name."""
    out, table = [], {}
    for c in cases:
        cand, t = tune_case(ctx, c, base, steps=steps)
        table[c.name] = {**candidate_entry(cand), "ms_per_step": t * 1e3}
        p = capi.SolveParams()
        ctypes_copy(p, base)
        apply_candidate(p, cand)
        out.append(p)
    return out, table


def tuned_params_grids(ctx, ids, cases, base: capi.SolveParams, steps=2):
    """Per-grid SolveParams for resident grids `ids` (created, LHS built):
    every grid tuned alone; returns the list and a table by grid name."""
    out, table = [], {}
    for gid, c in zip(ids, cases):
        cand, t = tune_resident(ctx, gid, c, base, steps=steps)
        table[c.name] = {**candidate_entry(cand), "ms_per_step": t * 1e3}
        p = capi.SolveParams()
        ctypes_copy(p, base)
        apply_candidate(p, cand)
        out.append(p)
    return out, table


def ctypes_copy(dst, src):
    for name, _ in src._fields_:
        setattr(dst, name, getattr(src, name))


def with_precision(p: capi.SolveParams, precision: int) -> capi.SolveParams:
    """A copy of p in another precision (the same smoothing settings)."""
    q = capi.SolveParams()
    ctypes_copy(q, p)
    q.precision = precision
    return q


def tuned_params(ctx, cases, base: capi.SolveParams, cache_path: str | None = None, steps=3):
    """Per-case SolveParams: each size class is tuned once (on its median-size
    member) and cached in cache_path (JSON) if given."""
    cache = {}
    if cache_path and os.path.exists(cache_path):
        with open(cache_path) as f:
            cache = json.load(f)
    classes = {}
    for q, c in enumerate(cases):
        classes.setdefault(size_class(c), []).append(q)
    for key, members in classes.items():
        if key in cache:
            continue
        cells = sorted(members, key=lambda q: cases[q].grid.ni * cases[q].grid.nj * cases[q].grid.nk)
        rep = cases[cells[len(cells) // 2]]
        cand, t = tune_case(ctx, rep, base, steps=steps)
        cache[key] = {**candidate_entry(cand), "ms_per_step": t * 1e3, "grid": rep.name}
    if cache_path:
        with open(cache_path, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
    out = []
    for c in cases:
        e = cache[size_class(c)]
        p = capi.SolveParams()
        ctypes_copy(p, base)
        apply_candidate(p, entry_candidate(e))
        out.append(p)
    return out, cache


def tuned_params_batch(ctx, ids, cases, base: capi.SolveParams, steps=2):
    """Per-grid SolveParams for resident grids `ids` (created, LHS built,
    U* set) that will run as one batch: each size class's grids are timed
    together as a sub-batch for every candidate."""
    classes = {}
    for q, c in enumerate(cases):
        classes.setdefault(size_class(c), []).append(q)
    table, out = {}, [None] * len(cases)
    for key, members in sorted(classes.items()):
        sub = [ids[q] for q in members]
        best, best_t = None, math.inf
        for cand in CANDIDATES:
            p = capi.SolveParams()
            ctypes_copy(p, base)
            apply_candidate(p, cand)
            try:
                _reset(ctx, sub, [cases[q] for q in members])
                ctx.projection_step_batch(sub, p)  # warm-up: graph capture
                t0 = time.perf_counter()
                ok = True
                for _ in range(steps):
                    infos, dm = ctx.projection_step_batch(sub, p)
                    ok = ok and all(i["converged"] for i in infos)
                t = (time.perf_counter() - t0) / steps if ok else math.inf
            except capi.VfsError:
                t = math.inf
            if t < best_t:
                best, best_t = cand, t
        table[key] = {**candidate_entry(best), "ms_per_batch_step": best_t * 1e3, "grids": len(members)}
        for q in members:
            p = capi.SolveParams()
            ctypes_copy(p, base)
            apply_candidate(p, best)
            out[q] = p
    _reset(ctx, ids, cases)
    return out, table


def _reset(ctx, ids, cases):
    for gid, c in zip(ids, cases):
        ctx.set_field(gid, capi.FIELD_USTAR, c.ucont)
        ctx.set_field(gid, capi.FIELD_P, np.zeros(c.grid.nvert.shape))
