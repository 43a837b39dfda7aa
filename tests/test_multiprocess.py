"""Multi-process tests of bench.py's replica path, on CPU with the gloo
backend and world size 2 (the GPU runs use one process per GPU over NCCL).

A gridding call has no exchange step, so N GPUs run N replicas: the slowest
rank's time is the job's, the whole-job rate counts every rank's
visibilities, replicas of a seeded workload grid identically, and the
reference arm prints its line from rank 0 only.
"""
from __future__ import annotations

import importlib
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sys.path.insert(0, ROOT)
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import bench
        import oracle
        synthetic = importlib.import_module("gpu-gridding_gb300.synthetic")
        # Rank r "took" 1.5 + r seconds: the job takes the slowest.
        t = bench.max_over_ranks(1.5 + rank, dist)
        # Every replica grids the same seeded workload.
        wl = synthetic.random_uniform_workload("replica", 3000, 128, 8, 1, 6,
                                               seed=4, cell_size_rad=4e-4)
        g, ns, nm = oracle.grid_f(wl)
        digest = (float(np.abs(g).astype(np.float64).sum()), int(ns),
                  float(nm), wl.num_points)
        gathered = [None] * world
        dist.all_gather_object(gathered, digest)
        out.put((rank, t, gathered))
    finally:
        dist.destroy_process_group()


def test_replicas_gloo_world2():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica, args=(r, 2, port, out))
             for r in range(2)]
    for p in procs:
        p.start()
    results = [out.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    results.sort()
    for rank, t, gathered in results:
        assert t == 2.5
        assert gathered[0] == gathered[1]
    sys.path.insert(0, ROOT)
    import bench
    n = results[0][2][0][3]
    # Two replicas of n visibilities in the slowest rank's 2.5 s.
    assert bench.replica_throughput(2, n, 2.5) == pytest.approx(
        2 * n / 2.5 / 1e6)
    assert bench.max_over_ranks(3.25) == 3.25   # one process


@pytest.mark.parametrize("rank", [0, 1])
def test_reference_arm_prints_from_rank0_only(rank):
    env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank),
               WORLD_SIZE="2")
    r = subprocess.run(
        [sys.executable, "bench.py", "--impl", "reference", "--gpus", "2",
         "--workload", "cfg0", "--steps", "1", "--warmup", "0"],
        cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    if rank:
        assert r.stdout.strip() == ""
    else:
        line = json.loads(r.stdout.strip().splitlines()[-1])
        assert line["impl"] == "reference" and line["n_gpus"] == 2
        assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
