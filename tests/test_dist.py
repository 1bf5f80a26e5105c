"""Replica path of bench.py with two gloo ranks on CPU: the barrier, the maximum over ranks, the
whole-job rate and the reference arm's rank-0-only rule. Replicas exchange no data."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    w, r, local = bench.dist_init("gloo")
    bench.barrier(w)
    slowest = bench.max_over_ranks(w, 100.0 + 10.0 * r)  # this rank's milliseconds
    rate = bench.whole_job_rate(w, 5, slowest)
    # the reference arm: ranks other than 0 return at once (rank 0 would time the CPU reference)
    ref_rc = bench.run_reference(None) if r != 0 else None
    with open(os.path.join(out_dir, f"rank{r}.json"), "w") as f:
        json.dump({"world": w, "rank": r, "local": local, "slowest": slowest, "rate": rate, "ref_rc": ref_rc}, f)
    bench.barrier(w)
    dist.destroy_process_group()


def test_replicas_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    for r, d in enumerate(res):
        assert d["world"] == world and d["rank"] == r and d["local"] == r
        assert d["slowest"] == 110.0  # every rank sees the slowest rank's time
        assert d["rate"] == pytest.approx(world * 5 / 0.110)
    assert res[1]["ref_rc"] == 0
    del torch


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    env = {k: os.environ.pop(k, None) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    try:
        assert bench.dist_init() == (1, 0, 0)
        assert bench.max_over_ranks(1, 3.5) == 3.5
        assert bench.whole_job_rate(1, 4, 2000.0) == 2.0
    finally:
        for k, v in env.items():
            if v is not None:
                os.environ[k] = v
