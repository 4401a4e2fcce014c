"""The N > 1 path of bench.py (replicas: one independent SpMV per rank,
no data-path collective) on CPU with gloo, world size 2: the timing
reduction takes the slowest rank's time for every figure, the whole-job rate
counts every rank's units, and the reference arm runs on rank 0 only."""
from __future__ import annotations

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


def _worker(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=ws)
    # rank r pretends its three timings were (1 + r, 10 - r, 5) ms
    got = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 5.0], ws, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, got))


def test_max_over_ranks_gloo_world_size_2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0] == res[1] == [2.0, 10.0, 5.0]


def test_replica_throughput_and_single_rank():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.replica_throughput(4, 1000.0, 2.0) == pytest.approx(2.0e6)
    assert bench.max_over_ranks([3.0, 4.0], 1, "cpu") == [3.0, 4.0]


def test_reference_arm_prints_only_on_rank_0(capsys, monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        workload, dtype, scale_rows, steps, warmup, gpus = "poisson16k", "f32", 0, 1, 1, 2
    bench.cpu_reference_arm(A())
    assert capsys.readouterr().out == ""
