"""The multi-rank path of bench.py (replicas, no data-path collective): max-over-ranks timing and
whole-job throughput, exercised with world_size 2 over gloo on the CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 10.0 + 5.0 * rank          # rank 1 is the slow replica
    ms = bench.reduce_max(local_ms, dist)
    q.put((rank, ms, bench.job_throughput(1e6, world, ms)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_max_time_and_total_points():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=5) for _ in range(2))
    for rank, ms, thr in res:
        assert ms == pytest.approx(15.0)
        assert thr == pytest.approx(2 * 1e6 / 15e-3)


def test_single_process_is_identity():
    assert bench.reduce_max(3.0, None) == 3.0
    assert bench.job_throughput(5.0, 1, 1000.0) == pytest.approx(5.0)
