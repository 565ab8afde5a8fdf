"""The multi-GPU path is replicas only (every rank runs its own copy of the
workload, no collective on the data path); what the ranks share is the timing
reduction of bench.py: the job time is the slowest rank's, the throughput
counts every rank's units.  Checked with two gloo ranks on the CPU, and the
reference arm's rule that only rank 0 runs."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q):
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        ms, value = bench.replica_throughput(10.0 + 5.0 * rank, 1.0e6, world, device="cpu")
        q.put((rank, ms, value))
    finally:
        dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in got:
        assert ms == 15.0                       # the slower rank
        assert value == pytest.approx(2.0e6 / 15e-3)


def test_single_rank_needs_no_group():
    sys.path.insert(0, str(ROOT))
    import bench
    ms, value = bench.replica_throughput(20.0, 1.0e6, 1)
    assert ms == 20.0 and value == pytest.approx(5.0e7)


def test_reference_arm_runs_on_rank0_only(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.run_reference(None) is None   # other ranks exit without work
