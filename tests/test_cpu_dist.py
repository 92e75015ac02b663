"""The N>1 host path of bench.py on CPU: two gloo ranks.

The path does not shard within one system ("replicas only"): each rank runs
its own seeded replica, ranks meet at barriers around the timed region, and
the slowest rank's time sets the whole-job figure.  These tests run that
host logic with world_size 2 on the gloo backend; no GPU is involved.
"""
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


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    t = bench.max_over_ranks(1.5 * (rank + 1), world, device="cpu")
    seed = bench.replica_seed(3, rank)
    seeds = [None] * world
    dist.all_gather_object(seeds, seed)
    bench.barrier(world)
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"max": t, "seeds": seeds}, f)


def test_two_gloo_ranks_max_time_and_distinct_replicas(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    for r in res:
        assert r["max"] == 3.0                       # the slowest rank's time on every rank
        assert r["seeds"] == [3, 4]                  # independent replicas, one per rank


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(2.5, 1) == 2.5
    assert bench.replica_seed(3, 0) == 3


def test_reference_arm_prints_only_on_rank_zero(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        steps, warmup, gpus, seed = 2, 3, 2, 3
    assert bench.run_reference(A()) == 0
    assert capsys.readouterr().out == ""
