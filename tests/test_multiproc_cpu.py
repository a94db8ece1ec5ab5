"""bench.py's N-rank path on CPU: two gloo ranks (127.0.0.1) agree on the
slowest rank's time and on the whole-job rate, and the reference arm's
non-zero ranks exit at once without work."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env() == (rank, world, rank)
        t_local = 1.0 + rank                      # rank 1 is the slowest
        t = bench.max_over_ranks(torch, t_local, world, torch.device("cpu"))
        out[rank] = (t, bench.job_rate(2048, 10, world, t))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_max_time_and_rate():
    world, port = 2, _free_port()
    out = mp.Manager().dict()
    mp.start_processes(_rank_main, args=(world, port, out), nprocs=world, join=True,
                       start_method="spawn")
    assert out[0] == out[1]
    t, rate = out[0]
    assert t == 2.0
    assert rate == pytest.approx(2048 * 10 * 2 / 2.0)


def test_reference_arm_other_ranks_exit_without_work(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        workload, steps, warmup, gpus = "c1", 1, 0, 2

    called = []
    monkeypatch.setattr(bench, "cpu_oracle_rate", lambda *a, **k: called.append(a))
    assert bench.run_reference(Args()) == 0
    assert called == []
