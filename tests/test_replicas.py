"""bench.py's multi-GPU mode: independent replicas, one process per GPU, with no collective on the data path. The
timed regions start after a barrier and report the slowest replica's time (max over ranks); the whole-job value is
the views of all ranks over that time. Checked on the CPU with gloo, world size 2."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank: int, world: int, port: int, times, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier()
        slowest = bench.max_over_ranks(times[rank], device="cpu")
        q.put((rank, slowest))
    finally:
        dist.destroy_process_group()


def test_single_process_timing_is_its_own():
    """Without a process group the barrier does nothing and the time is the process's own."""
    sys.path.insert(0, str(ROOT))
    import bench

    bench.barrier()
    assert bench.max_over_ranks(0.125) == 0.125


@pytest.mark.parametrize("times", [(1.5, 2.5), (3.0, 0.75)])
def test_two_replicas_report_the_slowest(times):
    """Two gloo ranks with different step times both report the larger one, so that rank 0's whole-job value
    (world x views per rank / time) is set by the slowest replica."""
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = sorted(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert got == [(0, max(times)), (1, max(times))]
    assert all(p.exitcode == 0 for p in procs)
