"""bench.py over several processes, on the CPU: the replicas' figures are
combined over two gloo ranks (segments summed, each time the slowest
rank's), and the reference arm runs on rank 0 alone."""
import os
import socket
from types import SimpleNamespace

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        seg, times = bench.job_totals(dist, 1000 * (rank + 1), [1.0 + rank, 5.0 - rank])
        q.put((rank, seg, times))
    finally:
        dist.destroy_process_group()


def test_job_totals_over_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = {}
    try:
        for _ in procs:
            rank, seg, times = q.get(timeout=120)
            results[rank] = (seg, times)
    finally:
        for p in procs:
            p.join(timeout=30)
            if p.is_alive():
                p.kill()
    assert all(p.exitcode == 0 for p in procs)
    # every rank gets the job's figures: 1000 + 2000 segments, max(1, 2), max(5, 4)
    assert results == {0: (3000.0, [2.0, 5.0]), 1: (3000.0, [2.0, 5.0])}


def test_job_totals_without_a_process_group():
    import bench
    assert bench.job_totals(None, 7, [1.5, 2.5]) == (7.0, [1.5, 2.5])


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = SimpleNamespace(seed=1, scale=1.0, paints=False, d3d11=False, warmup=3, steps=1, gpus=2)
    bench.run_reference(args)  # returns at once: no work, no line
    assert capsys.readouterr().out == ""
