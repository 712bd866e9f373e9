"""The multi-GPU form of the bench is replicas only (one independent copy of
the workload per rank, no data-path collective): its host logic -- the MAX
reduction of the per-step time over ranks and the whole-job value -- runs
here on two gloo ranks on the CPU (127.0.0.1 rendezvous)."""
import multiprocessing as mp
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


def _worker(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        ms = bench.replica_reduce(1.5 + rank, world)  # rank 1 is the slowest
        q.put((rank, ms, bench.replica_value(ms, world)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_reduction_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert [g[1] for g in got] == [2.5, 2.5]
    sys.path.insert(0, str(ROOT))
    import bench

    expect = 3 * bench.nn_flops() * 2 / 2.5e-3 / 1e12
    assert all(abs(g[2] - expect) < 1e-9 * expect for g in got)


def test_single_rank_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.replica_reduce(3.0, 1) == 3.0
    assert bench.replica_value(1.0, 1) == pytest.approx(3 * bench.nn_flops() / 1e-3 / 1e12)
