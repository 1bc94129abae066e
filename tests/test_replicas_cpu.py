"""Replicas across ranks (lightning-lite-quantum-simulator_gb300/replicas.py), run as world-size-2
gloo process groups on the CPU: shards partition the units, the job rate uses the slowest rank,
and a trajectory ensemble split over two ranks gives the single-process mean and standard error.
The per-trajectory values come from the oracle's restatement of the trajectory step, which the
GPU path matches choice for choice in the GPU tests."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

import oracle
import replicas
import workloads

N, GAMMA, LAM, SEED, TOTAL = 6, 0.02, 0.01, 77, 41


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ops = workloads.noisy_layers(N, 2)
        begin, count = replicas.shard(TOTAL, rank, world)
        z0, _, _, _ = oracle.traj_run(N, ops, GAMMA, LAM, SEED, begin, begin + count)
        mean, se, cnt = replicas.combine_moments(z0, dist)
        rate, slowest = replicas.job_rate(count, 0.5 * (rank + 1), dist)
        out.put((rank, begin, count, mean, se, cnt, rate, slowest))
    finally:
        dist.destroy_process_group()


def test_shards_partition_the_units():
    for total in (0, 1, 5, 41, 4096):
        for world in (1, 2, 3, 8):
            got = [replicas.shard(total, r, world) for r in range(world)]
            assert got[0][0] == 0 and sum(c for _, c in got) == total
            assert all(got[r][0] + got[r][1] == got[r + 1][0] for r in range(world - 1))
            assert max(c for _, c in got) - min(c for _, c in got) <= 1
    with pytest.raises(ValueError):
        replicas.shard(10, 2, 2)


def test_single_process_moments():
    x = np.array([0.25, -0.5, 1.0, 0.125])
    mean, se, n = replicas.combine_moments(x)
    assert n == 4 and mean == pytest.approx(np.mean(x), abs=1e-15)
    assert se == pytest.approx(np.std(x, ddof=1) / 2.0, abs=1e-15)
    assert replicas.combine_moments([0.3])[1] == 0.0  # one sample: 0, as the reference reports
    rate, slowest = replicas.job_rate(100, 2.0)
    assert rate == 50.0 and slowest == 2.0


def test_two_gloo_ranks_match_one_process():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ops = workloads.noisy_layers(N, 2)
    z_all, _, _, _ = oracle.traj_run(N, ops, GAMMA, LAM, SEED, 0, TOTAL)
    want_mean, want_se = float(np.mean(z_all)), float(np.std(z_all, ddof=1) / np.sqrt(TOTAL))
    assert [r[1:3] for r in res] == [(0, 21), (21, 20)]
    for _, _, _, mean, se, cnt, rate, slowest in res:
        assert cnt == TOTAL
        assert abs(mean - want_mean) <= 1e-14 and abs(se - want_se) <= 1e-14
        assert slowest == 1.0 and rate == pytest.approx(TOTAL / 1.0)
    # the shards' trajectories are the single-process ensemble's, unit for unit
    z0, _, _, _ = oracle.traj_run(N, ops, GAMMA, LAM, SEED, 21, 41)
    assert np.array_equal(z0, z_all[21:])
