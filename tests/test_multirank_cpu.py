"""The multi-rank path of bench.py on CPU: two gloo ranks on 127.0.0.1.

bench.py runs one process per GPU (replicas: each rank steps its own batch,
seeded by its rank, no collective on the data path) and reports the whole
job's voxel-steps/s timed by the slowest rank.  These tests run that logic
with world_size 2 on the host."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_body(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        # each rank "took" a different time; every rank must see the slowest
        secs = bench.max_over_ranks(1.0 + rank, torch)
        insts, cfg = bench.workload_instances("sweep", rank)
        phases = [i.sources[0].phase for i in insts]
        value = bench.job_value(sum(i.grid.voxels for i in insts), 10, ws, secs)
        out.put((rank, secs, cfg["seed"], len(insts), phases[:3], value))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_and_value():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_body, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, seed0, n0, ph0, v0), (r1, s1, seed1, n1, ph1, v1) = res
    assert (r0, r1) == (0, 1)
    assert s0 == s1 == 2.0                 # max over ranks, on every rank
    assert (seed0, seed1) == (0, 1)        # batches seeded by rank
    assert n0 == n1 == 96 and ph0 != ph1   # same shapes, different draws
    voxels = 32 * (96 ** 3 + 128 ** 3 + 192 ** 3)
    assert v0 == v1 == pytest.approx(voxels * 10 * 2 / 2.0)


def test_single_rank_needs_no_process_group():
    assert not dist.is_initialized()
    assert bench.max_over_ranks(3.5, torch) == 3.5
    assert bench.job_value(100, 10, 1, 2.0) == 500.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    bench.run_reference(bench.parse([]))  # rank 1: returns at once, prints nothing
    assert capsys.readouterr().out == ""
