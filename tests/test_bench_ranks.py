"""The replica path of bench.py on CPU: two gloo ranks on 127.0.0.1.

bench.py runs one replica of the workload per GPU (weak scaling, no
data-path collective): the job's time is the slowest rank's and its value
every rank's pairs over that time; the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 + 5.0 * rank  # rank 1 is slower
    total = bench.max_over_ranks(ms, world, device="cpu")
    value = bench.job_value(1e9, 4, world, total)
    r, w, loc = bench.dist_env()
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, total, value, (r, w, loc)))


def test_two_gloo_ranks_take_the_slowest_time():
    mp = pytest.importorskip("torch.multiprocessing")
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
    for rank, total, value, env in res:
        assert total == 15.0
        assert value == pytest.approx(1e9 * 4 * 2 / 15e-3)
        assert env == (rank, 2, rank)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        workload = "trihedral60"
        warmup = 1
        steps = 1
        cpu_seconds = 1.0

    bench.run_reference(Args())
    assert capsys.readouterr().out == ""
