"""The multi-GPU form of the bench (replicas, weak scaling) on the CPU: two gloo ranks.

Under torchrun every rank serves its own requests; the job's time is the
slowest rank's, and its value counts the units of all ranks.  Here each rank
runs the CPU oracle on its own small requests and the bench's bookkeeping
(seeds, max over ranks, whole-job rate) is checked across the two processes.
"""

from __future__ import annotations

import os
import socket
import sys
import time
from pathlib import Path

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out) -> None:
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from oracle import oracle
        from torchhull_gb300 import scenes

        seeds = bench.replica_seeds(rank, 2, base=70)
        t0 = time.perf_counter()
        faces = 0
        for seed in seeds:
            r = scenes.make_request(seed, 4, 64, 4, False)
            res = oracle.visual_hull(r.masks, r.transforms, r.level, r.cube_corner_bfl, r.cube_length,
                                     r.masks_partial, r.transforms_convention, True, nthreads=1)
            faces += int(res.faces.shape[0])
        dt = time.perf_counter() - t0
        slowest = bench.max_over_ranks(dt, world, torch.device("cpu"))
        units = torch.tensor([len(seeds)], dtype=torch.int64)
        dist.all_reduce(units)
        out.put((rank, seeds, dt, slowest, int(units.item()), bench.whole_job_rate(len(seeds), world, slowest),
                 faces))
    finally:
        dist.destroy_process_group()


def test_two_replica_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(out.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, dt0, max0, n0, v0, f0), (r1, s1, dt1, max1, n1, v1, f1) = results
    assert (r0, r1) == (0, 1)
    assert not set(s0) & set(s1)  # each rank serves its own scenes
    assert max0 == max1 == pytest.approx(max(dt0, dt1))
    assert n0 == n1 == 4  # units of the whole job
    assert v0 == v1 == pytest.approx(4 / max(dt0, dt1))
    assert f0 > 0 and f1 > 0
