"""The replica path of bench.py with two ranks (world_size 2, gloo on the CPU): every rank
reads its place from the launcher's environment, meets the others at the barriers, and the
elapsed time is the maximum over ranks."""
from __future__ import annotations

import multiprocessing as mp
import os
import queue
import socket
import time


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, port: int, out) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE="2", LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=2)
    world, r, local = bench.dist_env()
    bench.barrier(world)
    elapsed = bench.max_over_ranks(1.5 * (rank + 1), world)
    bench.barrier(world)
    dist.destroy_process_group()
    out.put((r, world, local, elapsed))


def test_two_replicas_agree_on_the_slowest_rank():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    results = []
    deadline = time.monotonic() + 120
    try:
        # stop waiting as soon as both ranks reported, or both exited (a rank that raised)
        while len(results) < 2 and time.monotonic() < deadline:
            try:
                results.append(out.get(timeout=1))
            except queue.Empty:
                if not any(p.is_alive() for p in procs) and out.empty():
                    break
        results.sort()
    finally:
        for p in procs:
            p.join(timeout=30)
            if p.is_alive():
                p.kill()
    assert results == [(0, 2, 0, 3.0), (1, 2, 1, 3.0)]
    assert all(p.exitcode == 0 for p in procs)
