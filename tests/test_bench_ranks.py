"""bench.py's multi-rank host logic on the CPU: a world-size-2 gloo process group on 127.0.0.1
(the GPU runs use NCCL with one replica per GPU and no collective on the data path; only the
timing is reduced).  Replicas report the slowest rank's time and the units of all ranks."""
import argparse
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(times[rank], dist, "cpu")
    rate = bench.whole_job_rate(world, 1000, t)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, rate))


def test_max_over_ranks_and_rate_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [0.0125, 0.01725]
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = sorted(q.get(timeout=180) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    for rank, t, rate in got:
        assert t == max(times)                       # every rank sees the slowest replica's time
        assert rate == pytest.approx(2 * 1000 / max(times))
    assert all(p.exitcode == 0 for p in procs)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.whole_job_rate(1, 10, 2.0) == 5.0


def test_reference_arm_other_ranks_do_no_work(monkeypatch):
    """Under torchrun only rank 0 times the reference's CPU path; the others exit 0 at once."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    args = argparse.Namespace(warmup=3, steps=5, gpus=2, config="C2")
    assert bench.run_reference(args) == 0
