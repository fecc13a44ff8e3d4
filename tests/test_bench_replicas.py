"""bench.py's multi-rank host logic on CPU: world size 2 over gloo (127.0.0.1).  Every rank steps
its own replica ("replicas only": the step has no exchange), the job's time is the slowest
rank's, and the reference arm runs on rank 0 alone."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, loc = bench.dist_env()
    t = bench.max_over_ranks(0.25 + 0.5 * r, w, torch.device("cpu"))   # rank 1 is the slower one
    v = bench.job_throughput(1000, 10, w, t)
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, w, loc, t, v))


def test_two_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1] and all(g[1] == 2 and g[2] == g[0] for g in got)
    assert all(g[3] == pytest.approx(0.75) for g in got)                  # max over ranks
    assert all(g[4] == pytest.approx(1000 * 10 * 2 / 0.75) for g in got)   # whole-job particle-steps/s


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    called = []
    monkeypatch.setattr(bench, "cpu_baseline", lambda *a, **k: called.append(a))

    class Args:
        steps, warmup, gpus, workload = 3, 3, 2, "fluid_1m"
    assert bench.run_reference(Args()) == 0
    assert called == [] and capsys.readouterr().out == ""
