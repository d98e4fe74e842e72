"""The replicas-only multi-GPU path of bench.py on CPU: two gloo ranks.

Every rank aligns its own reads with no collective on the data path; the
only cross-rank steps are the barrier around the timed region and the
maximum of the ranks' times, from which the whole-job throughput follows.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    r, w, local = bench.dist_env()
    dist.init_process_group("gloo", rank=r, world_size=w)
    try:
        dist.barrier()
        slowest = bench.max_over_ranks(10.0 + rank)       # rank 1 took longer
        value = bench.job_throughput(1000, w, 5, slowest)
        q.put((r, w, local, slowest, value))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_and_throughput():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for r, (rank, world, local, slowest, value) in enumerate(got):
        assert (rank, world, local) == (r, 2, r)
        assert slowest == 11.0                       # every rank reports the max
        assert value == pytest.approx(1000 * 2 * 5 / 11.0)


def test_single_rank_defaults(monkeypatch):
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench.dist_env() == (0, 1, 0)
    assert bench.job_throughput(1_000_000, 1, 5, 0.125) == 40_000_000
