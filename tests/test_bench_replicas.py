"""The N > 1 path of bench.py on the CPU: world_size-2 `gloo` ranks run the
replica aggregation (MAX over ranks, whole-job elements / slowest rank's
time) and the reference arm's rank gating.  No GPU, no NCCL."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      LOCAL_RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    local_ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
    value, max_ms = bench.job_throughput(local_ms, 1 << 24, 20, world)
    dist.barrier()
    q.put((rank, value, max_ms, bench.replica_seed(rank)))
    dist.destroy_process_group()


def test_two_rank_aggregation_uses_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    expect = (1 << 24) * 2 * 20 / 0.150 / 1e9  # both ranks' elements over the max (150 ms)
    for rank, value, max_ms, seed in res:
        assert max_ms == pytest.approx(150.0)
        assert value == pytest.approx(expect)
    assert res[0][3] != res[1][3]  # replicas draw different inputs


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    value, ms = bench.job_throughput(10.0, 1 << 20, 5, 1)
    assert ms == 10.0 and value == pytest.approx((1 << 20) * 5 / 0.010 / 1e9)


def test_reference_arm_other_ranks_exit_without_work(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = type("A", (), {"field": "BabyBear", "log_n": 24, "steps": 3, "warmup": 3, "gpus": 2})()
    assert bench.run_reference(args) is None  # returns at once: rank 0 alone runs and prints
