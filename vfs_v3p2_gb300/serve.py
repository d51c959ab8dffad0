"""Serving loop for pressure-projection requests (continuous batching).

Simulation streams each own a resident grid on the device (MG hierarchy,
pressure, phi; phi is the warm start of the stream's next request).
Requests arrive as a Poisson process; the loop admits them as request slots
and HBM free up (vfs_submit reserves a grid's solver memory against the
context's budget), so a request that arrives while others are on the GPU
joins them, and vfs_poll advances every request in flight.  A stream whose
grid is not resident gets one when the budget allows, evicting idle streams'
grids least recently used first.  Latency is measured from a request's
arrival to the loop seeing its result.

Inputs follow the serving workload: stream sizes log-uniform between two
extents; each stream's successive requests are its previous intermediate
velocity plus seeded Gaussian perturbations (a few pre-drawn variants per
stream, used in turn, so the loop itself does no random-number work); every
request uploads its U* from page-locked host memory and downloads its
pressure.
"""
from __future__ import annotations

import collections
import ctypes
import dataclasses
import math
import time

import numpy as np

from . import capi, synth


@dataclasses.dataclass
class Stream:
    case: synth.Case
    inputs: list            # page-locked AoS U* variants
    p_out: np.ndarray       # page-locked pressure of the latest result
    grid: int | None = None
    params: object = None   # the stream's SolveParams (autotuned), else the server's
    last_used: float = 0.0
    served: int = 0
    busy: bool = False


def serving_streams(n_streams=16, lo=(32, 32, 32), hi=(256, 128, 128), seed=1005, variants=2, sigma=0.01,
                    levels_max=5):
    """Stream grids of log-uniform size per axis (multiples of 8), each with
    an immersed sphere or none, and `variants` perturbed copies of its U*."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(n_streams):
        ext = []
        for a, b in zip(lo, hi):
            ext.append(max(16, int(round(math.exp(rng.uniform(math.log(a), math.log(b))) / 8)) * 8))
        ni, nj, nk = ext
        levels = synth.mg_levels(ni, nj, nk, levels_max)
        sph = [(math.pi, 0.0, math.pi / 2, 0.3)] if rng.uniform() < 0.5 else []
        case = synth.channel_case(ni, nj, nk, seed=1_000_000 + s, spheres=sph, levels=levels, name=f"stream{s}")
        noise = np.random.default_rng(2_000_000 + s)
        ins = []
        for v in range(variants):
            u = case.ucont + sigma * noise.standard_normal(case.ucont.shape)
            ins.append(np.ascontiguousarray(synth.finish_ucont(u, ni, nj, nk)))
        out.append(Stream(case=case, inputs=ins, p_out=np.zeros(case.grid.nvert.shape)))
    return out


class Server:
    """Request loop over one context (one GPU)."""

    def __init__(self, ctx: capi.Context, streams, params: capi.SolveParams, dt=0.04):
        self.ctx = ctx
        self.streams = streams
        self.params = params
        self.dt = dt
        self.registered = []
        for s in streams:
            for a in s.inputs + [s.p_out]:
                ctx.host_register(a)
                self.registered.append(a)

    def close(self):
        for s in self.streams:
            if s.grid is not None and not s.busy:
                self.ctx.grid_destroy(s.grid)
                s.grid = None
        for a in self.registered:
            self.ctx.host_unregister(a)
        self.registered = []

    def _estimate(self, s: Stream) -> int:
        g = s.case.grid
        mz, my, mx = g.nvert.shape
        d = capi.GridDesc(mx, my, mz, 1, 0, 1, s.case.levels, 0, 0, 0, s.case.immersed, None, None)
        b = ctypes.c_ulonglong()
        self.ctx.check(self.ctx.L.vfs_grid_estimate(ctypes.byref(d), self.params.restart, ctypes.byref(b)))
        return b.value

    def ensure_grid(self, s: Stream) -> bool:
        """Make the stream's grid resident; False if the budget does not allow
        it now (every other resident grid is busy)."""
        if s.grid is not None:
            return True
        used, budget = self.ctx.memory()
        need = self._estimate(s)
        if budget:
            idle = sorted([o for o in self.streams if o.grid is not None and not o.busy], key=lambda o: o.last_used)
            while used + need > budget and idle:
                victim = idle.pop(0)
                self.ctx.grid_destroy(victim.grid)
                victim.grid = None
                used, _ = self.ctx.memory()
            if used + need > budget:
                return False
        g = s.case.grid
        s.grid = self.ctx.grid_create(g.coor, g.nvert, s.case.levels, s.case.immersed)
        self.ctx.poisson_lhs(s.grid)
        self.ctx.set_field(s.grid, capi.FIELD_P, np.zeros(g.nvert.shape))
        return True

    def _evict_one(self, keep: Stream) -> bool:
        idle = sorted([o for o in self.streams if o.grid is not None and not o.busy and o is not keep],
                      key=lambda o: o.last_used)
        if not idle:
            return False
        self.ctx.grid_destroy(idle[0].grid)
        idle[0].grid = None
        return True

    def submit(self, sid: int):
        s = self.streams[sid]
        if s.busy or not self.ensure_grid(s):
            return None
        u = s.inputs[s.served % len(s.inputs)]
        while True:
            try:
                t = self.ctx.submit(s.grid, s.params if s.params is not None else self.params,
                                    ucont_in=u.ctypes.data, p_out=s.p_out.ctypes.data, dt=self.dt)
                break
            except capi.VfsError as e:
                # the solver memory reserved at admission does not fit: free an
                # idle grid and retry, or wait for a running request to finish
                if e.code != capi.VFS_ERR_NOMEM or not self._evict_one(s):
                    if e.code == capi.VFS_ERR_NOMEM:
                        return None
                    raise
        if t is not None:
            s.busy = True
        return t

    def run(self, arrivals, time_limit=120.0, keep_outputs=False):
        """arrivals: list of (time_s, stream_id).  Returns per-request records
        (stream, arrival, admitted, done, iterations, divmax, status, and the
        pressure with keep_outputs) and the wall time from the first arrival
        to the last result."""
        queue = collections.deque()
        pending = {}  # ticket -> (request index)
        recs = [dict(stream=sid, arrival=t) for t, sid in arrivals]
        nxt = 0
        t0 = time.perf_counter()
        done = 0
        while done < len(arrivals):
            now = time.perf_counter() - t0
            if now > time_limit:
                raise RuntimeError(f"serving run exceeded {time_limit} s")
            while nxt < len(arrivals) and arrivals[nxt][0] <= now:
                queue.append(nxt)
                nxt += 1
            # admit in arrival order; a request of a busy stream waits its turn
            waiting = collections.deque()
            while queue:
                r = queue.popleft()
                sid = recs[r]["stream"]
                t = self.submit(sid) if all(recs[q]["stream"] != sid for q in waiting) else None
                if t is None:
                    waiting.append(r)
                else:
                    pending[t] = r
                    recs[r]["admitted"] = time.perf_counter() - t0
            queue = waiting
            got = self.ctx.poll(wait=False) if pending else None
            while got is not None:
                ticket, status, info, divmax = got
                r = pending.pop(ticket)
                s = self.streams[recs[r]["stream"]]
                s.busy = False
                s.served += 1
                s.last_used = time.perf_counter() - t0
                recs[r].update(done=s.last_used, iterations=info["iterations"], divmax=divmax, status=status)
                if keep_outputs:
                    recs[r]["p"] = s.p_out.copy()
                done += 1
                got = self.ctx.poll(wait=False) if pending else None
            if not pending and not queue and nxt < len(arrivals):
                time.sleep(max(0.0, min(arrivals[nxt][0] - (time.perf_counter() - t0), 0.002)))
        wall = max(r["done"] for r in recs) - arrivals[0][0]
        return recs, wall


def poisson_arrivals(n, rate, n_streams, seed=1005):
    rng = np.random.default_rng(1_000_000 + seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    sid = rng.integers(0, n_streams, size=n)
    return [(float(a), int(b)) for a, b in zip(t - t[0], sid)]


def summarize(recs, wall):
    lat = np.array([r["done"] - r["arrival"] for r in recs]) * 1e3
    its = [r["iterations"] for r in recs]
    return dict(solves_per_s=len(recs) / wall if wall > 0 else float("nan"),
                latency_ms={"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                            "max": float(lat.max())},
                iterations={"mean": float(np.mean(its)), "max": int(max(its))},
                divmax=float(max(r["divmax"] for r in recs)),
                failed=int(sum(1 for r in recs if r["status"] != 0)))
