"""The multi-GPU form is replicas only (pixels, samples and scenes are independent; no collective on the
data path): bench.py times each replica, reduces the timings to their maximum over the ranks and reports
all ranks' work over that time.  Checked here with two gloo ranks on the CPU; the reference arm runs on
rank 0 only."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        got = bench.reduce_max_over_ranks([1.0 + rank, 10.0 * (world - rank)], "cpu")
        q.put((rank, got, bench.replica_throughput(world, 1000, got[0])))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_replica():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, thr in res:
        assert got == [2.0, 20.0]              # max over ranks, per entry
        assert thr == pytest.approx(2 * 1000 / 2.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    args = type("A", (), {"cpu_sample": 1024, "warmup": 0, "steps": 1})()
    assert bench.run_reference(args) is None
