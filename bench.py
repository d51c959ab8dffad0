#!/usr/bin/env python
"""Benchmark of the GB300 pressure-projection step.

One step = the pressure section of the reference's Flow_Solver
(solvers.c:871-931) on one grid: IB flux balance, PoissonRHS, the
multigrid-preconditioned FGMRES solve, UpdatePressure, Projection (with
Contra2Cart) and the divergence check.  The default workload is the
256x128x128 channel with an immersed sphere (mixed FP32-MG / FP64-FGMRES,
rtol 1e-9 and max |div u| <= 1e-8 guaranteed by the stopping test, 5
multigrid levels), seeded synthetic inputs of that shape.

value : projection steps (pressure solves) per second with U* resident in
        HBM when the timed region starts, mixed precision.
e2e   : the same through vfs_projection_step with page-locked host buffers
        (vfs_host_alloc): H2D of U* and p, the step, D2H of the corrected U
        and p, every step.
Also reported: the plain FP64 solve rate on the same grid, p50/p99 step
latency, the live-probed roofline of the dominant kernel, the CPU oracle
baseline, clocks during the timed region and the kernel launch count.

--gpus N (launched with torchrun for N > 1) runs N independent replicas,
one per GPU: the pressure step has no cross-solve exchange, so scaling is
weak and no data-path collective exists.  --impl reference times the
reference's algorithm on the host cores instead (the CPU oracle port: the
reference itself needs PETSc, HYPRE and MPI, which this image lacks).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="sphere", choices=["channel", "sphere", "terrain", "batch", "serve"])
    ap.add_argument("--requests", type=int, default=400, help="serve: timed requests")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: Poisson arrival rate, requests/s")
    ap.add_argument("--no-tune", action="store_true",
                    help="batch/serve: default solve parameters instead of the autotuner's per size class")
    ap.add_argument("--scale", type=int, default=1, help="divide each grid extent (quick runs)")
    ap.add_argument("--grid", default=None, help="NIxNJxNK override of the sphere workload (profiling sizes)")
    ap.add_argument("--rtol", type=float, default=1e-9)
    ap.add_argument("--div-tol", type=float, default=1e-8, help="max |div u| the solve must reach")
    ap.add_argument("--nu", type=int, default=3, help="pre- and post-smoothing sweeps")
    ap.add_argument("--nu1", type=int, default=None, help="pre-smoothing sweeps (overrides --nu)")
    ap.add_argument("--nu2", type=int, default=None, help="post-smoothing sweeps (overrides --nu)")
    ap.add_argument("--nu-coarse", default=None,
                    help="PRE,POST sweeps below the finest level of the single-grid workloads (-1,-1: as finest, "
                         "the default with the Chebyshev smoother; 5,5 the default with the Jacobi one)")
    ap.add_argument("--smoother", default="chebyshev", choices=["chebyshev", "jacobi"],
                    help="sweep damping: Chebyshev roots on [cheb_hi / cheb_ratio, cheb_hi], or omega on every sweep")
    ap.add_argument("--cheb-hi", type=float, default=2.0)
    ap.add_argument("--cheb-ratio", type=float, default=6.0)
    ap.add_argument("--omega", type=float, default=0.9, help="y-line Jacobi damping (--smoother jacobi)")
    ap.add_argument("--smooth-cols", type=int, default=0, help="smoother tile columns (0: automatic)")
    ap.add_argument("--mg-half", type=int, default=0, choices=[0, 1, 2],
                    help="multigrid operator storage: FP32 face form on 11-slot levels (0), FP16 normalised by "
                         "the diagonal (1), FP32 assembled coefficients (2); FP32 arithmetic in every case")
    ap.add_argument("--restart", type=int, default=30)
    ap.add_argument("--mg-stage", type=int, default=0, choices=[0, 1],
                    help="finest face-form sweeps staged in registers (0) or by tensor-memory copies (1)")
    ap.add_argument("--mg-grouped", type=int, default=0, choices=[0, 1],
                    help="batch: V-cycles as grouped launches over same-size grids (1) or each grid's own (0)")
    ap.add_argument("--orth", default="cgs", choices=["cgs", "cgs2"], help="Gram-Schmidt of the Arnoldi step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the headline phi check against the oracle")
    ap.add_argument("--no-workloads", action="store_true",
                    help="skip the compact runs of the channel, batch and serving workloads on the default line")
    return ap.parse_args()


def make_case(args):
    import math
    from vfs_v3p2_gb300 import synth
    if args.grid:
        ni, nj, nk = (int(v) for v in args.grid.lower().split("x"))
        return synth.channel_case(ni, nj, nk, seed=1002, spheres=[(math.pi, 0.0, math.pi / 2, 0.3)], sigma=0.1,
                                  levels=5, profile=synth.poiseuille, name=f"sphere_{ni}x{nj}x{nk}")
    if args.config == "channel":
        return synth.c1_channel(args.scale)
    if args.config == "terrain":
        return synth.c3_terrain(args.scale)
    return synth.c2_sphere(args.scale)


# storage of the FP32 multigrid's level operators (vfs_solve_params.mg_half)
OPERATOR = {0: "fp32 face form (3 face weights + 2 cross weights + aj carrying 4 code bits per cell; on levels with "
                "i-j or j-k cross terms 4 more cross weights carrying their own codes)",
            1: "fp16 diagonal-normalised, row sums kept (fp32 arithmetic)",
            2: "fp32 assembled coefficients (11 or 19 slots)"}

WORKLOAD = {
    "channel": "channel 64x64x64, tanh beta 2.0, skew 0.05 sin(z), no body, U ~ N(0,1) per face",
    "sphere": "channel 256x128x128 + sphere r=0.3 at (pi,0,pi/2), Poiseuille + N(0,0.1^2)",
    "terrain": "terrain 512x256x256 over a Gaussian hill, log-law + N(0,0.05^2)",
    "batch": "64 independent channel grids, extents log-uniform 32^3..192x96x96, skew U[0,0.1], beta U[1.5,3], "
             "0-3 spheres r U[0.1,0.3], U ~ N(0,1); one graph launch per FGMRES iteration for all 64",
    "serve": "Poisson arrivals from 16 streams, extents log-uniform 32^3..256x128x128, U* = previous + N(0,0.01^2), "
             "warm start from the resident phi, HBM admission budget 120 GB",
}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return dist, rank, local, ws
    return None, rank, local, ws


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons (every 200 ms)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={self.Q}", "--format=csv,noheader",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1].split()[0]))
                mx = max(mx, float(parts[2].split()[0]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel_key: str):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/traffic.json), scaled to this workload, or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            t = json.load(f)
        return t.get(kernel_key)
    except Exception:
        return None


# the oracle's multigrid settings: y-line Jacobi, 2 + 2 sweeps damped 0.8 on
# every level, 32 sweeps on the coarsest (its defaults); the GPU arm's
# Chebyshev-damped 3 + 3 sweeps change the iteration history, not the answer
ORACLE_MG = {"nu1": 2, "nu2": 2, "coarsest_sweeps": 32, "omega": 0.8, "omega_coarsest": 0.8,
             "smoother": "y-line Jacobi, constant damping"}


def oracle_module():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    import oracle as O
    O.build()
    return O


def cpu_baseline(case, args, steps=2, warmup=1):
    """The CPU oracle (same discretisation, FP64 FGMRES + GMG, OpenMP over all
    host cores) on the same workload with the GPU arm's stopping rule (rtol
    and max |div u| <= div_tol), after warmup untimed steps; returns steps/s,
    threads and the last step."""
    O = oracle_module()
    g = case.grid
    d = O.dims_of(g)
    mg = O.MG(d, g.coor, g.nvert, case.levels)
    mg.set_params(ORACLE_MG["nu1"], ORACLE_MG["nu2"], ORACLE_MG["coarsest_sweeps"], ORACLE_MG["omega"],
                  ORACLE_MG["omega_coarsest"])
    kw = dict(levels=case.levels, immersed=case.immersed, rtol=args.rtol, div_tol=args.div_tol, mg=mg)
    for _ in range(max(1, warmup)):
        O.projection_step(g, case.ucont, **kw)
    t = time.perf_counter()
    for _ in range(steps):
        r = O.projection_step(g, case.ucont, **kw)
    dt = time.perf_counter() - t
    mg.close()
    return steps / dt, O.lib().orc_num_threads(), r


def oracle_parity(case, phis):
    """Relative L2 (fluid mean removed) of each phi against a tight oracle
    solve of the same step (rtol 1e-13), outside any timed region."""
    O = oracle_module()
    g = case.grid
    ref = O.projection_step(g, case.ucont, levels=case.levels, immersed=case.immersed, rtol=1e-13, maxit=600)
    fl = g.nvert < 0.1
    fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = (False,) * 6
    r = ref["phi"][fl] - ref["phi"][fl].mean()
    out = {}
    for k, phi in phis.items():
        if phi is not None:
            a = phi[fl] - phi[fl].mean()
            out[k] = float(np.linalg.norm(a - r) / np.linalg.norm(r))
    return {"phi_rel_l2_vs_oracle": out, "oracle_rtol": 1e-13, "oracle_divmax": ref["divmax"],
            "bar": "phi rel L2 <= 1e-8 after removing the fluid mean"}


# the headline metric, identical on every line of both arms (the workload and
# what a line measures are in its config)
METRIC = "Pressure solves/s, HBM GB/s, p50/p99 latency: mixed vs FP64 at \u2016div u\u2016<1e-8"


REF_MAX_STEPS = 10


def run_reference(args):
    dist, rank, local, ws = dist_init()
    if rank != 0:
        return
    if args.config in ("batch", "serve"):
        # the oracle on a sample of the workload's own grids (its median-size ones)
        from vfs_v3p2_gb300 import serve, synth
        if args.config == "batch":
            pool = synth.c4_batch(64, seed=1004)
        else:
            pool = [s.case for s in serve.serving_streams(16)]
        pool.sort(key=lambda c: c.grid.nvert.size)
        sample = pool[len(pool) // 2 - 1:len(pool) // 2 + 1]
        nwarm = max(1, args.warmup)
        runs = [cpu_baseline(c, args, steps=1, warmup=nwarm) for c in sample]
        rates = [r[0] for r in runs]
        val = float(len(rates) / sum(1.0 / r for r in rates))
        cores = os.cpu_count()
        line = {"metric": METRIC, "value": val, "unit": "solves/s",
                "impl": "reference", "n_gpus": args.gpus, "steps": len(sample), "warmup": nwarm,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded)",
                "config": {"workload": WORKLOAD[args.config], "rtol": args.rtol, "div_tol": args.div_tol,
                           "oracle_mg": ORACLE_MG,
                           "measures": "pressure projection steps/s of the CPU oracle (FP64 FGMRES + GMG, the "
                                       "GPU arm's stopping rule)"},
                "divmax": max(r[2]["divmax"] for r in runs),
                "cpu_baseline": {"value": val, "unit": "solves/s", "cores": cores, "kind": "port",
                                 "sample": f"two median-size grids of the workload, one step each after {nwarm} "
                                           f"warm-up steps"},
                "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "the reference links PETSc/HYPRE/MPI, absent here: its CPU algorithm is timed as the "
                        "oracle restatement, which matches the reference's own compiled path functions bit for bit"}
        print(json.dumps(line), flush=True)
        return
    case = make_case(args)
    # the timed steps are capped at REF_MAX_STEPS (a full-size CPU step takes
    # seconds), the warm-up steps are the arm's own
    nsteps, nwarm = max(1, min(args.steps, REF_MAX_STEPS)), max(1, args.warmup)
    val, cores, r = cpu_baseline(case, args, steps=nsteps, warmup=nwarm)
    line = {
        "metric": METRIC, "value": val, "unit": "solves/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": nsteps, "warmup": nwarm, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD[args.config], "grid": case.name, "cells": int(case.grid.ni * case.grid.nj *
                                                                                   case.grid.nk),
                   "mg_levels": case.levels, "rtol": args.rtol, "div_tol": args.div_tol, "oracle_mg": ORACLE_MG,
                   "measures": "pressure projection steps/s of the CPU oracle (FP64 FGMRES + GMG, the GPU arm's "
                               "stopping rule)"},
        "cpu_baseline": {"value": val, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": f"{WORKLOAD[args.config]}: {nsteps} full-size steps timed after {nwarm} "
                                   f"warm-up steps"},
        "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "divmax": r["divmax"], "iterations": r["info"]["iterations"], "div_rounds": r["info"]["rounds"],
        "same_config_note": "same grid, inputs, rtol and div_tol as the GPU arm; its own smoother settings "
                            "(oracle_mg) and step count, so iteration histories differ",
        "note": "the reference links PETSc/HYPRE/MPI, absent here: its CPU algorithm is timed as the oracle "
                "restatement, which matches the reference's own compiled path functions bit for bit",
    }
    print(json.dumps(line), flush=True)


def base_line(args, ws):
    return {"n_gpus": ws, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32-mg/f64-krylov", "data": "synthetic (seeded)"}


def main_batch(args, dist, rank, local, ws):
    line = run_batch(args, dist, local, ws)
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_batch(args, dist, local, ws):
    from vfs_v3p2_gb300 import autotune, capi, synth
    sc = max(1, args.scale)
    cases = synth.c4_batch(64, seed=1004, lo=(32 // sc, 32 // sc, 32 // sc), hi=(192 // sc, 96 // sc, 96 // sc))
    ctx = capi.Context(local)
    base = capi.default_params(precision="mixed", rtol=args.rtol, div_tol=args.div_tol, maxit=400, restart=args.restart,
                               mg_grouped=args.mg_grouped)
    ids = []
    for c in cases:
        gid = ctx.grid_create(c.grid.coor, c.grid.nvert, c.levels, c.immersed)
        ctx.poisson_lhs(gid)
        ctx.set_field(gid, capi.FIELD_USTAR, c.ucont)
        ctx.set_field(gid, capi.FIELD_P, np.zeros(c.grid.nvert.shape))
        ids.append(gid)
    tuned, tune_s = None, 0.0
    if not args.no_tune:  # every grid tuned alone (its smoothing schedule), before the timed steps
        t0 = time.perf_counter()
        plist, tuned = autotune.tuned_params_grids(ctx, ids, cases, base)
        tune_s = time.perf_counter() - t0
    else:
        plist = [base] * len(ids)
    for _ in range(args.warmup):
        ctx.projection_step_batch(ids, plist)
    clk = Clocks(local)
    barrier(dist)
    n0 = capi.launch_count()
    per, its, dms = [], [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        infos, dm = ctx.projection_step_batch(ids, plist)
        per.append(time.perf_counter() - t0)
        its += [i["iterations"] for i in infos]
        dms.append(float(dm.max()))
    nl = capi.launch_count() - n0
    clocks = clk.stop()
    barrier(dist)
    total = allmax(dist, sum(per))
    cells = sum(c.grid.ni * c.grid.nj * c.grid.nk for c in cases)
    value = ws * len(ids) * args.steps / total
    fp64 = None
    if not args.no_fp64:
        # the same grids in plain FP64 (each with its mixed run's smoothing
        # settings): batched, and one grid at a time through the single-grid step
        p64 = [autotune.with_precision(p, capi.VFS_FP64) for p in plist]
        ctx.projection_step_batch(ids, p64)
        K64 = max(2, args.steps // 2)
        t0 = time.perf_counter()
        its64, dm64 = [], []
        for _ in range(K64):
            infos, dm = ctx.projection_step_batch(ids, p64)
            its64 += [i["iterations"] for i in infos]
            dm64.append(float(dm.max()))
        t_b = allmax(dist, time.perf_counter() - t0)
        for gid, p in zip(ids, p64):
            ctx.projection_step(gid, p)
        t0 = time.perf_counter()
        dm1 = []
        for gid, p in zip(ids, p64):
            _, dm = ctx.projection_step(gid, p)
            dm1.append(dm)
        t_1 = allmax(dist, time.perf_counter() - t0)
        r_b, r_1 = ws * len(ids) * K64 / t_b, ws * len(ids) / t_1
        fp64 = {"batched": {"value": r_b, "iterations_mean": float(np.mean(its64)), "divmax": max(dm64)},
                "one_grid_at_a_time": {"value": r_1, "divmax": max(dm1)},
                "mixed_batched_over_fp64_batched": value / r_b, "mixed_batched_over_fp64_one_at_a_time": value / r_1}
    line = {"metric": METRIC,
            "value": value, "unit": "solves/s", "steps": args.steps,
            "ms_per_step": 1e3 * total / args.steps, **base_line(args, ws),
            "config": {"workload": WORKLOAD["batch"], "grids": len(ids), "cells_total": int(cells),
                       "measures": "batched pressure projection steps/s (64 uneven grids, one graph launch per "
                                   "FGMRES iteration), mixed FP32-MG/FP64-FGMRES",
                       "rtol": args.rtol, "div_tol": args.div_tol, "autotuned": not args.no_tune,
                       "autotune_s": tune_s, "mg_grouped": args.mg_grouped,
                       "mg_operator": OPERATOR[base.mg_half],
                       "timer": "host wall clock around synchronous batch calls (results on the host)",
                       "parallelism": f"replicas x{ws}"},
            "e2e": None, "iterations": {"mean": float(np.mean(its)), "max": int(max(its))}, "divmax": max(dms),
            "latency_ms": {"p50": float(np.percentile(per, 50) * 1e3), "p99": float(np.percentile(per, 99) * 1e3)},
            "clocks": clocks, "gpu_launches": int(nl), "fp64": fp64}
    if tuned:
        line["autotune"] = tuned
    for gid in ids:
        ctx.grid_destroy(gid)
    ctx.close()
    return line


def main_serve(args, dist, rank, local, ws):
    line = run_serve(args, dist, local, ws)
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_serve(args, dist, local, ws):
    from vfs_v3p2_gb300 import autotune, capi, serve
    sc = max(1, args.scale)
    streams = serve.serving_streams(16, lo=(32 // sc,) * 3, hi=(256 // sc, 128 // sc, 128 // sc))
    ctx = capi.Context(local, hbm_budget_bytes=120 * 10**9, max_inflight=16)
    params = capi.default_params(precision="mixed", rtol=args.rtol, div_tol=args.div_tol, maxit=400,
                                 restart=args.restart, warm_start=1)
    tuned, tune_s = None, 0.0
    if not args.no_tune:  # every stream's grid tuned alone, single-grid latency objective
        t0 = time.perf_counter()
        plist, tuned = autotune.tuned_params_cases(ctx, [s.case for s in streams], params)
        tune_s = time.perf_counter() - t0
        for s, p in zip(streams, plist):
            s.params = p
    srv = serve.Server(ctx, streams, params)
    for s in streams:  # resident hierarchies of the 16 streams (admission)
        srv.ensure_grid(s)
    # warm-up: every stream serves a few requests (graph capture, warm phi)
    warm = serve.poisson_arrivals(max(48, 16 * args.warmup), args.rate, 16, seed=7)
    srv.run(warm)
    arr = serve.poisson_arrivals(args.requests, args.rate, 16)
    clk = Clocks(local)
    barrier(dist)
    n0 = capi.launch_count()
    recs, wall = srv.run(arr)
    nl = capi.launch_count() - n0
    clocks = clk.stop()
    barrier(dist)
    wall = allmax(dist, wall)
    summ = serve.summarize(recs, wall)
    cells = [streams[r["stream"]].case.grid.nvert.size for r in recs]
    h2d = float(np.mean([24 * c for c in cells]))
    d2h = float(np.mean([8 * c for c in cells]))
    fp64 = None
    if not args.no_fp64:
        # capacity: the same number of requests arriving at once, mixed and
        # plain FP64 (same smoother settings); then FP64 at the offered rate
        burst = serve.poisson_arrivals(args.requests, 1e6, 16, seed=11)
        rb, wb = srv.run(burst)
        cap = serve.summarize(rb, allmax(dist, wb))
        srv.params = autotune.with_precision(params, capi.VFS_FP64)
        for s in streams:
            if s.params is not None:
                s.params = autotune.with_precision(s.params, capi.VFS_FP64)
        srv.run(warm)
        rb64, wb64 = srv.run(burst)
        cap64 = serve.summarize(rb64, allmax(dist, wb64))
        recs64, wall64 = srv.run(arr)
        s64 = serve.summarize(recs64, allmax(dist, wall64))
        fp64 = {"value": ws * s64["solves_per_s"], "latency_ms": s64["latency_ms"], "divmax": s64["divmax"],
                "failed": s64["failed"],
                "capacity_solves_per_s": {"mixed": ws * cap["solves_per_s"], "fp64": ws * cap64["solves_per_s"],
                                          "mixed_over_fp64": cap["solves_per_s"] / cap64["solves_per_s"],
                                          "divmax": {"mixed": cap["divmax"], "fp64": cap64["divmax"]},
                                          "requests": len(burst)}}
    line = {"metric": METRIC,
            "value": ws * summ["solves_per_s"], "unit": "solves/s", "steps": len(recs),
            "ms_per_step": 1e3 * wall / len(recs), **base_line(args, ws),
            "config": {"workload": WORKLOAD["serve"], "streams": 16, "rate_req_s": args.rate,
                       "measures": "served pressure projection steps/s with p50/p99 latency (Poisson arrivals, "
                                   "continuous batching), mixed FP32-MG/FP64-FGMRES",
                       "requests": len(recs), "hbm_budget_gb": 120, "max_inflight": 16,
                       "mg_operator": OPERATOR[params.mg_half], "rtol": args.rtol,
                       "div_tol": args.div_tol, "autotuned": not args.no_tune, "autotune_s": tune_s,
                       "timer": "host wall clock, first arrival to last result",
                       "parallelism": f"replicas x{ws}"},
            "e2e": {"value": ws * summ["solves_per_s"], "unit": "solves/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "latency_ms": summ["latency_ms"], "iterations": summ["iterations"], "divmax": summ["divmax"],
            "failed": summ["failed"], "clocks": clocks, "gpu_launches": int(nl), "fp64": fp64}
    if tuned:
        line["autotune"] = tuned
    srv.close()
    ctx.close()
    return line


def kernel_table(recs, top):
    """Per kernel (finest level / coarser levels): launches, device ms,
    algorithmic GB and achieved GB/s, largest time first."""
    agg = {}
    for name, lv, ms, by in recs:
        key = (name, "finest" if lv == top else "coarser levels")
        a = agg.setdefault(key, [0, 0.0, 0.0])
        a[0] += 1
        a[1] += ms
        a[2] += by
    out = []
    for (name, where), (n, ms, by) in sorted(agg.items(), key=lambda kv: -kv[1][1]):
        out.append({"kernel": name, "levels": where, "launches": n, "ms": ms, "alg_gb": by / 1e9,
                    "achieved_gbs": (by / (ms / 1e3) / 1e9) if ms > 0 else 0.0})
    return out


def nu_coarse(args) -> str:
    if args.nu_coarse is not None:
        return args.nu_coarse
    return "-1,-1" if args.smoother == "chebyshev" else "5,5"


def smoother_config(args) -> dict:
    if args.smoother == "chebyshev":
        return {"smoother": "chebyshev", "cheb_interval": [args.cheb_hi / args.cheb_ratio, args.cheb_hi]}
    return {"smoother": "jacobi", "omega": args.omega}


def compact_single(args, dist, local, ws, config):
    """Mixed and plain FP64 steps/s of one single-grid workload (U* resident,
    the headline's stopping rule; the smoothing schedule the autotuner picks
    for the grid, the same in both precisions), for the default line."""
    from vfs_v3p2_gb300 import autotune, capi
    a = argparse.Namespace(**vars(args))
    a.config, a.grid, a.scale = config, None, 1
    case = make_case(a)
    g = case.grid
    ctx = capi.Context(local)
    gid = ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    ctx.poisson_lhs(gid)
    ctx.set_field(gid, capi.FIELD_USTAR, case.ucont)
    ctx.set_field(gid, capi.FIELD_P, np.zeros(g.nvert.shape))
    out = {"workload": WORKLOAD[config], "grid": case.name, "mg_levels": case.levels}
    base = capi.default_params(precision="mixed", rtol=args.rtol, div_tol=args.div_tol, maxit=400)
    t0 = time.perf_counter()
    cand, _ = autotune.tune_resident(ctx, gid, case, base, steps=2)
    out["autotuned"] = {**autotune.candidate_entry(cand), "autotune_s": time.perf_counter() - t0}
    autotune.apply_candidate(base, cand)
    K = 20 if g.nvert.size < 2**24 else 5
    phis = {}
    for prec in ("mixed", "fp64"):
        params = autotune.with_precision(base, capi.VFS_MIXED if prec == "mixed" else capi.VFS_FP64)
        for _ in range(3):
            ctx.projection_step(gid, params)
        barrier(dist)
        ctx.mark(gid, 0)
        its, dms = [], []
        for _ in range(K):
            info, dm = ctx.projection_step(gid, params)
            its.append(info["iterations"])
            dms.append(dm)
        ctx.mark(gid, 1)
        t = allmax(dist, ctx.elapsed(0, 1))
        out[prec] = {"value": ws * K / (t / 1e3), "unit": "solves/s", "iterations": statistics.mean(its),
                     "divmax": max(dms), "steps": K}
        phis[prec] = ctx.get_field(gid, capi.FIELD_PHI, g.nvert.shape)
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    # the two solutions of the same step (fluid interior, means removed)
    fl = g.nvert < 0.1
    fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = False, False, False, False, False, False
    a = phis["mixed"][fl] - phis["mixed"][fl].mean()
    r = phis["fp64"][fl] - phis["fp64"][fl].mean()
    out["phi_rel_l2_mixed_vs_fp64"] = float(np.linalg.norm(a - r) / np.linalg.norm(r))
    ctx.grid_destroy(gid)
    ctx.close()
    return out


def compact_workloads(args, dist, local, ws):
    """The channel, terrain, batched and served workloads in short runs, so
    that one default bench line records every configuration; --config batch / serve
    give the full runs.  Every grid runs the smoothing schedule the autotuner
    picks for it (tuned once, before the timed steps; the FP64 runs use the
    same schedules)."""
    out = {"channel_64x64x64": compact_single(args, dist, local, ws, "channel"),
           "terrain_512x256x256": compact_single(args, dist, local, ws, "terrain")}
    b = argparse.Namespace(**vars(args))
    b.steps, b.warmup, b.no_tune, b.no_fp64, b.scale = 3, 1, False, False, 1
    bl = run_batch(b, dist, local, ws)
    out["batch_64_grids"] = {"workload": WORKLOAD["batch"], "value": bl["value"], "unit": "solves/s",
                             "steps": bl["steps"], "latency_ms": bl["latency_ms"], "divmax": bl["divmax"],
                             "iterations": bl["iterations"], "autotuned": True,
                             "autotune_s": bl["config"]["autotune_s"],
                             "fp64_batched": bl["fp64"]["batched"]["value"],
                             "mixed_over_fp64_batched": bl["fp64"]["mixed_batched_over_fp64_batched"],
                             "fp64_divmax": bl["fp64"]["batched"]["divmax"]}
    v = argparse.Namespace(**vars(args))
    v.requests, v.warmup, v.no_tune, v.no_fp64, v.scale = 200, 1, False, False, 1
    sl = run_serve(v, dist, local, ws)
    out["serve_16_streams"] = {"workload": WORKLOAD["serve"], "value": sl["value"], "unit": "solves/s",
                               "requests": sl["steps"], "rate_req_s": v.rate, "latency_ms": sl["latency_ms"],
                               "divmax": sl["divmax"], "failed": sl["failed"], "autotuned": True,
                               "autotune_s": sl["config"]["autotune_s"],
                               "fp64_latency_ms": sl["fp64"]["latency_ms"], "fp64_divmax": sl["fp64"]["divmax"],
                               "capacity_solves_per_s": sl["fp64"]["capacity_solves_per_s"]}
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.config in ("batch", "serve"):
        dist, rank, local, ws = dist_init()
        (main_batch if args.config == "batch" else main_serve)(args, dist, rank, local, ws)
        if dist is not None:
            dist.destroy_process_group()
        return
    dist, rank, local, ws = dist_init()
    from vfs_v3p2_gb300 import capi
    case = make_case(args)
    g = case.grid
    N = g.nvert.size
    ctx = capi.Context(local)
    gid = ctx.grid_create(g.coor, g.nvert, case.levels, case.immersed)
    ctx.poisson_lhs(gid)
    ctx.set_field(gid, capi.FIELD_USTAR, case.ucont)
    ctx.set_field(gid, capi.FIELD_P, np.zeros(g.nvert.shape))
    nu1 = args.nu if args.nu1 is None else args.nu1
    nu2 = args.nu if args.nu2 is None else args.nu2
    nuc = [int(v) for v in nu_coarse(args).split(",")]
    smooth = dict(smoother=args.smoother, cheb_hi=args.cheb_hi, cheb_ratio=args.cheb_ratio, omega=args.omega)
    mixed = capi.default_params(precision="mixed", rtol=args.rtol, nu1=nu1, nu2=nu2, restart=args.restart,
                                div_tol=args.div_tol, maxit=400, orth=args.orth, **smooth,
                                nu1_coarse=nuc[0], nu2_coarse=nuc[1], smooth_cols=args.smooth_cols,
                                mg_half=args.mg_half, mg_stage=args.mg_stage)
    other = capi.default_params(precision="mixed", rtol=args.rtol, nu1=nu1, nu2=nu2, restart=args.restart,
                                div_tol=args.div_tol, maxit=400, orth=args.orth, **smooth,
                                nu1_coarse=nuc[0], nu2_coarse=nuc[1], smooth_cols=args.smooth_cols,
                                mg_half=2 if args.mg_half == 0 else 0)
    fp64 = capi.default_params(precision="fp64", rtol=args.rtol, nu1=nu1, nu2=nu2, restart=args.restart,
                               div_tol=args.div_tol, maxit=400, orth=args.orth, **smooth,
                               nu1_coarse=nuc[0], nu2_coarse=nuc[1], smooth_cols=args.smooth_cols)

    def steps(params, K, base_slot):
        infos, divs = [], []
        ctx.mark(gid, base_slot)
        for s in range(K):
            info, dm = ctx.projection_step(gid, params)
            ctx.mark(gid, base_slot + 1 + s)
            infos.append(info)
            divs.append(dm)
        total = ctx.elapsed(base_slot, base_slot + K)
        per = [ctx.elapsed(base_slot + s, base_slot + s + 1) for s in range(K)]
        return total, per, infos, divs

    # ---- mixed precision, U* resident: the headline ----
    steps(mixed, args.warmup, 0)
    clk = Clocks(local)
    barrier(dist)
    ctx.sync()
    n0 = capi.launch_count()
    total_ms, per_ms, infos, divs = steps(mixed, args.steps, 100)
    ctx.sync()
    nl = capi.launch_count() - n0
    clocks = clk.stop()
    barrier(dist)
    tmax = allmax(dist, total_ms)
    value = ws * args.steps / (tmax / 1e3)
    phi_mixed = ctx.get_field(gid, capi.FIELD_PHI, g.nvert.shape)
    # dominant kernel: CUDA events around each of its launches, on its own
    # stream, over a repeat of the timed steps (per-launch events run the
    # iteration uncaptured; kernel durations do not depend on that)
    ctx.probe_begin(capi.PROBE_SMOOTH)
    steps(mixed, min(args.steps, 5), 600)
    plaunch, pms, pbytes = ctx.probe_end()
    # every instrumented kernel of the step, likewise, for the per-kernel
    # achieved GB/s and the step's algorithmic bytes
    KP = 3
    ctx.probe_begin(capi.PROBE_ALL)
    steps(mixed, KP, 650)
    n_all, _, bytes_all = ctx.probe_end()
    per_kernel = kernel_table(ctx.probe_records(n_all), case.levels - 1)

    # ---- the same mixed solve with the other multigrid operator storage ----
    alt = None
    if not args.no_fp64:
        steps(other, 2, 700)
        Ka = max(3, args.steps // 2)
        ta, _, infa, diva = steps(other, Ka, 710)
        alt = {"mg_operator": OPERATOR[other.mg_half], "value": ws * Ka / (allmax(dist, ta) / 1e3),
               "iterations": statistics.mean(i["iterations"] for i in infa), "divmax": max(diva)}

    # ---- plain FP64 on the same grid ----
    fp64_rate, fp64_iters, fp64_div, mix_vs_fp64_err, phi64 = None, None, None, None, None
    if not args.no_fp64:
        steps(fp64, 2, 200)
        K64 = max(3, args.steps // 2)
        t64, _, inf64, div64 = steps(fp64, K64, 300)
        fp64_rate = ws * K64 / (allmax(dist, t64) / 1e3)
        fp64_iters = statistics.mean(i["iterations"] for i in inf64)
        fp64_div = max(div64)
        phi64 = ctx.get_field(gid, capi.FIELD_PHI, g.nvert.shape)
        fl = g.nvert < 0.1
        fl[0], fl[-1], fl[:, 0], fl[:, -1], fl[:, :, 0], fl[:, :, -1] = (False,) * 6
        a, r = phi_mixed[fl] - phi_mixed[fl].mean(), phi64[fl] - phi64[fl].mean()
        mix_vs_fp64_err = float(np.linalg.norm(a - r) / np.linalg.norm(r))

    # ---- end to end through the C ABI with page-locked host buffers ----
    e2e = None
    if not args.no_e2e:
        # page-locked step buffers from cudaHostAlloc (vfs_host_alloc)
        u_host = ctx.host_alloc(case.ucont.shape)
        p_host = ctx.host_alloc(g.nvert.shape)
        p_host[...] = 0.
        hbytes = int(u_host.nbytes + p_host.nbytes)
        e_ms = []
        for s in range(2 + args.steps):
            np.copyto(u_host, case.ucont)
            ctx.mark(gid, 400)
            ctx.projection_step_ptr(gid, mixed, u_host.ctypes.data, p_host.ctypes.data)
            ctx.mark(gid, 401)
            if s >= 2:
                e_ms.append(ctx.elapsed(400, 401))
        ctx.host_free(u_host)
        ctx.host_free(p_host)
        del u_host, p_host
        et = allmax(dist, sum(e_ms))
        e2e = {"value": ws * len(e_ms) / (et / 1e3), "unit": "solves/s", "h2d_bytes_per_step": hbytes,
               "d2h_bytes_per_step": hbytes}

    peak, peak_kind = measured_peak()
    # algorithmic bytes of one finest sweep: the FP32 smoother's 53 bytes per
    # interior cell (9 FP32 metric coefficients, a case byte, x, b, the line
    # diagonal and the new x), whatever the storage streams
    n_int = g.ni * g.nj * g.nk
    alg = 53.0 * n_int
    avg_ms = pms / plaunch if plaunch else None
    achieved = alg / (avg_ms / 1e3) / 1e9 if plaunch else None
    kname = {0: "k_smooth<float, FaceOp>", 1: "k_smooth<float, __half>", 2: "k_smooth<float, float>"}[args.mg_half]
    if args.mg_half == 0 and args.config == "terrain":
        # i-j and j-k cross terms (the hill): the general face form
        kname = "k_smooth<float, FaceOp, general>"
    elif args.mg_half == 0:
        # the face form's full-width sweeps run the warp-row kernel (30-column
        # tiles), or with --mg-stage 1 the tensor-copy one
        kname = "k_smooth_tma" if args.mg_stage else "k_smooth_w<2>"
    traffic = ncu_traffic(kname + ":" + case.name)
    roof = {"kernel": kname + " (finest-level y-line sweep, x != 0)", "bound": "hbm", "achieved": achieved,
            "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
            "traffic": traffic, "launches": plaunch, "avg_launch_ms": avg_ms,
            "timing": "CUDA event pair around each run of consecutive finest sweeps on their stream, over repeats "
                      "of the timed steps (iterations issued uncaptured, convergence read after each)",
            "alg_bytes_per_launch": alg, "alg_bytes_per_cell": 53.0,
            "streamed_bytes_per_launch": pbytes / plaunch if plaunch else None,
            "streamed_frac": ((pbytes / plaunch) / (avg_ms / 1e3) / 1e9 / peak) if plaunch else None}

    step_bytes = bytes_all / KP
    solve_hbm = {"alg_bytes_per_step": step_bytes, "achieved_gbs": step_bytes / (tmax / args.steps / 1e3) / 1e9,
                 "unit": "GB/s", "peak": peak, "frac": step_bytes / (tmax / args.steps / 1e3) / 1e9 / peak,
                 "note": "algorithmic bytes of every instrumented launch of a step (probed run) over the unprobed "
                         "device time of a step"}
    kernels = [dict(k, frac=k["achieved_gbs"] / peak) for k in per_kernel]

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cval, cores, _ = cpu_baseline(case, args, steps=2)
        cpu = {"value": cval, "unit": "solves/s", "cores": cores, "kind": "port",
               "sample": f"2 full-size steps of {case.name} after 1 warm-up (FP64 FGMRES + GMG, OpenMP)"}

    parity = None
    if rank == 0 and not args.no_parity:
        parity = oracle_parity(case, {"mixed": phi_mixed, "fp64": phi64})

    line = None
    if rank == 0:
        its = [i["iterations"] for i in infos]
        line = {
            "metric": METRIC,
            "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": tmax / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32-mg/f64-krylov", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD[args.config], "grid": case.name, "cells": int(g.ni * g.nj * g.nk),
                       "measures": "pressure projection steps/s with U* resident, mixed FP32-MG/FP64-FGMRES",
                       "mg_levels": case.levels, "rtol": args.rtol, "div_tol": args.div_tol, "nu": [nu1, nu2], "nu_coarse": nuc,
                       "restart": args.restart, "orth": args.orth, **smoother_config(args),
                       "mg_operator": OPERATOR[args.mg_half], "mg_stage": args.mg_stage,
                       "l2": "working set > L2 (129 MB) per step", "parallelism": f"replicas x{ws}"},
            "e2e": e2e,
            "latency_ms": {"p50": float(np.percentile(per_ms, 50)), "p99": float(np.percentile(per_ms, 99))},
            "iterations": {"mean": statistics.mean(its), "max": max(its)},
            "divmax": max(divs), "relres_max": max(i["relres"] for i in infos),
            "fp64": {"value": fp64_rate, "iterations": fp64_iters, "divmax": fp64_div,
                     "mixed_over_fp64": (value / fp64_rate) if fp64_rate else None,
                     "phi_rel_l2_mixed_vs_fp64": mix_vs_fp64_err},
            "mixed_other_operator": alt,
            "roofline": roof, "solve_hbm": solve_hbm, "kernels": kernels,
            "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": int(nl), "parity": parity,
        }
    ctx.close()
    if not args.no_workloads and args.config == "sphere" and not args.grid and args.scale == 1:
        workloads = compact_workloads(args, dist, local, ws)
        if line is not None:
            line["workloads"] = workloads
    if line is not None:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
