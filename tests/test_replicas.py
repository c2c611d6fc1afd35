"""The multi-GPU form is replicas: each rank runs its own right-hand sides on
its own copy of the grid with no exchange on the data path; the benchmark
only synchronises ranks around the timed region and takes the slowest.
That host logic runs here as two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), WAVEY_BENCH_GLOO="1")
    sys.path.insert(0, str(ROOT))
    import bench

    r, w = bench.dist_init()
    bench.barrier(w)
    slowest = bench.max_over_ranks(1.0 + r, w)  # rank r "took" 1 + r seconds
    q.put((r, w, slowest))
    dist.destroy_process_group()


def test_two_replicas_agree_on_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get() for _ in range(2))
    assert res == [(0, 2, 2.0), (1, 2, 2.0)]


def test_reference_arm_runs_on_rank_zero_only():
    sys.path.insert(0, str(ROOT))
    import bench

    class A:
        workload, warmup, steps, sample_steps = "room_small", 3, 1, 5

    # Rank 1 returns at once with no output; rank 0's work is tested by the
    # bench itself.
    assert bench.run_reference(A(), 1, 2) is None


def test_reference_arm_line(capsys):
    """Rank 0 of the reference arm times the reference's CPU loop (the
    oracle's restatement of run_cpu) on a bounded sample and prints one JSON
    line with the contract's keys."""
    import json

    sys.path.insert(0, str(ROOT))
    import bench

    class A:
        workload, warmup, steps, sample_steps = "room_small", 3, 2, 20

    bench.run_reference(A(), 0, 1)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["value"] > 0 and line["higher_is_better"] is True and line["steps"] == 2 and line["warmup"] == 3
    assert line["config"]["workload"] == "room_small"
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and "20 of" in cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def _shard_rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), WAVEY_BENCH_GLOO="1")
    sys.path.insert(0, str(ROOT))
    import bench

    r, w = bench.dist_init()
    sc = bench.make_scene("room_pillars", r)
    mine = (r, sc.grid.n, sc.grid.air, [tuple(t) for comp in sc.sources for t in comp], sc.notes["shard"])
    shards = [None] * w
    dist.all_gather_object(shards, mine)  # the host gather of per-rank results, the only exchange
    q.put(shards)
    dist.destroy_process_group()


def test_room_pillars_is_source_sharded_over_ranks():
    """bench --gpus 2 on room_pillars: each rank builds the same grid and runs
    its own speaker's four right-hand sides; rank 0's share is the
    single-GPU workload's source, and no two ranks share a right-hand side."""
    sys.path.insert(0, str(ROOT))
    from wavey_gb300 import workloads as W

    one = W.room_pillars(seed=2)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    shards = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    (r0, n0, air0, taps0, s0), (r1, n1, air1, taps1, s1) = shards
    assert (r0, r1) == (0, 1) and n0 == n1 == one.grid.n and air0 == air1 == one.grid.air
    assert taps0 == [tuple(t) for comp in one.sources for t in comp]
    assert len(taps1) == len(taps0) == 7 and not set(taps0) & set(taps1)
    assert (s0, s1) == ("speaker 0 of 2", "speaker 1 of 2")
