"""The bench's multi-rank timing on the CPU: world_size 2 over gloo. Each rank is an
independent replica of the frame; the step time every rank reports is the slowest
rank's, and the whole-job rate counts the units of all ranks over that time."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out_dir: str):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        own_ms = 2.0 + 3.0 * rank                     # rank 1 is the slow replica
        ms = bench.max_over_ranks(own_ms)
        rate = bench.whole_job_rate(world, 1.0e7, ms)
        dist.barrier()
    finally:
        dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"ms": ms, "rate": rate}, f)


def test_max_over_ranks_and_whole_job_rate_world2(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    for r in res:
        assert r["ms"] == 5.0                          # the slowest rank's step
        assert r["rate"] == pytest.approx(world * 1.0e7 / 5.0e-3 / 1e9)


def test_max_over_ranks_without_a_process_group():
    import bench

    assert bench.max_over_ranks(3.25) == 3.25
    assert bench.whole_job_rate(1, 2.0e9, 1000.0) == pytest.approx(2.0)
