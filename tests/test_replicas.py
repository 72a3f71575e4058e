"""Several GPUs: replicas only (each rank fits or evaluates its own datasets,
no collective on the data path). The bench's aggregation -- the slowest
rank's time by an all-reduce MAX, world x steps per second of it -- runs
here as two gloo processes on the CPU."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w, local = bench.dist_env()
    ms, value = bench.replica_value(10.0 + 5.0 * rank, 100)
    q.put((r, w, local, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_report_the_slowest_rank():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[:3] for g in got] == [(0, 2, 0), (1, 2, 1)]
    for _, _, _, ms, value in got:
        assert ms == 15.0
        assert value == pytest.approx(2 * 100 / 0.015)


def test_single_process_needs_no_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.replica_value(4.0, 8) == (4.0, 2000.0)
