"""bench.py's multi-rank path without a GPU: two gloo ranks (one process
each, rendezvous on 127.0.0.1) pass the barrier, agree on the slowest rank's
time (max over ranks) and report the whole-job rate over both replicas; under
torchrun the reference arm runs on rank 0 alone and the other ranks exit 0
without output.  The hot path itself does not shard: N GPUs run N replicas."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, REPO)
    import bench

    bench.barrier(world)
    t = bench.max_over_ranks(1.0 + rank, world)  # rank r "took" 1 + r seconds
    q.put((rank, t, bench.job_throughput(10.0, world, 5, t)))
    bench.barrier(world)
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_time_and_rate():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = sorted(q.get(timeout=120) for _ in range(2))
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert [r for r, _, _ in res] == [0, 1]
    assert all(t == 2.0 for _, t, _ in res)           # the slowest replica
    assert all(v == 10.0 * 2 * 5 / 2.0 for _, _, v in res)  # both replicas' units over that time
    assert all(p.exitcode == 0 for p in procs)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, REPO)
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1"])
    assert bench.main() == 0
    assert capsys.readouterr().out == ""
