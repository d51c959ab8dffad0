"""The N > 1 path of bench.py on CPU: two ranks (gloo, 127.0.0.1) run the
bench's own rendezvous, barrier and max-over-ranks timing helpers, as
torchrun launches them for replicas on N GPUs (no data-path collective)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    dist, r, local, ws = bench.dist_init()
    bench.barrier(dist)
    t = bench.allmax(dist, 10.0 * (rank + 1))   # per-rank timed region, ms
    bench.barrier(dist)
    q.put((r, local, ws, t))
    dist.destroy_process_group()


def test_two_rank_timing_helpers():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 0, 2, 20.0), (1, 1, 2, 20.0)]


def _rank_replica(rank, world, port, q):
    """Each rank builds its replica's workload as bench.py does (seeded,
    independent of the rank: weak scaling, the same work per GPU) and the
    reference arm's gate (rank 0 alone runs the CPU baseline)."""
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import argparse

    import numpy as np

    import bench
    args = argparse.Namespace(config="sphere", grid=None, scale=16)
    case = bench.make_case(args)
    digest = float(np.sum(case.grid.coor)) + float(np.sum(case.ucont)) + float(np.sum(case.grid.nvert))
    if rank == 0:
        dist, r, local, ws = bench.dist_init()
        ran = None
    else:
        # the reference arm under torchrun: ranks other than 0 return at once
        ref_args = argparse.Namespace(config="sphere", gpus=world)
        ran = bench.run_reference(ref_args)
        import torch.distributed as dist
    dist.barrier()
    q.put((rank, digest, ran))
    dist.destroy_process_group()


def test_replicas_do_the_same_work_and_reference_runs_on_rank_0():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_replica, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][1] == out[1][1]   # identical replica inputs on both ranks
    assert out[1][2] is None        # rank 1 did no reference work
