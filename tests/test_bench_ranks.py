"""bench.py under torchrun (N > 1): every rank renders its own replica, the job's time is the
slowest rank's (MAX) and its work the rays of all ranks (SUM); only rank 0 prints. Two gloo
ranks on the CPU, rendezvous on 127.0.0.1; the reference arm runs on rank 0 alone."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    # rank k: (100 + 50 k) ms for (k + 1) M rays
    t_ms, rays = bench.aggregate_over_ranks(100.0 + 50.0 * rank, 1e6 * (rank + 1), ws)
    out.put((rank, t_ms, rays, bench.mrays_per_s(rays, t_ms)))
    bench._finish_ranks(ws)


def test_two_ranks_take_the_slowest_time_and_all_rays():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    try:
        res = sorted(q.get(timeout=180) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
    assert [p.exitcode for p in procs] == [0, 0]
    for rank, t_ms, rays, v in res:
        assert t_ms == 150.0 and rays == 3e6
        assert v == pytest.approx(3e6 / 0.150 / 1e6)


def test_one_rank_keeps_its_own_numbers():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.aggregate_over_ranks(12.5, 7e6, 1) == (12.5, 7e6)
    assert bench.mrays_per_s(7e6, 12.5) == pytest.approx(560.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    """Ranks other than 0 leave the reference arm at once with status 0 and print nothing."""
    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    called = []
    monkeypatch.setattr(bench, "cpu_baseline_sample", lambda **kw: called.append(kw))

    class Args:
        steps, warmup, gpus = 3, 3, 2

    assert bench.run_reference(Args()) == 0
    assert called == []
