"""Replicas across ranks: one process per GPU, each with its own state, or its own shard of
independent units (trajectories, circuits of a mixed batch, parameter sets of the adjoint).

The state-vector path does not shard (one state per GPU), so nothing here touches amplitudes and
there is no collective on the data path.  What crosses ranks is host-side bookkeeping only:

* the timing of a job: the slowest rank's elapsed time, and the whole job's throughput from it;
* the moments of a sharded ensemble: count, sum and sum of squares, summed over ranks, give the
  ensemble mean and its standard error, sample standard deviation over sqrt(n) and 0 for a single
  sample, as the reference reports them (src/TrajectorySolver.h:273-277, src/Mitigation.h:359-371).

Units are split into contiguous shards, so unit i (trajectory i, keyed by its own Philox counter)
gives the same value whatever the number of ranks.  Every function takes the process group module
(`torch.distributed`, already initialised) or None for a single process, and works with any
backend: nccl between GPUs, gloo in the CPU tests.
"""
from __future__ import annotations

import os

import numpy as np


def rank_env() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the launcher's environment (torchrun sets all three)."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def shard(total: int, rank: int, world: int) -> tuple[int, int]:
    """(begin, count) of rank's contiguous share of `total` units; shares differ by at most one."""
    if world < 1 or not 0 <= rank < world or total < 0:
        raise ValueError("shard: need 0 <= rank < world and total >= 0")
    base, extra = divmod(total, world)
    begin = rank * base + min(rank, extra)
    return begin, base + (1 if rank < extra else 0)


def _reduce(values, op: str, dist, device):
    """Element-wise sum or max of a float64 vector over ranks (identity for a single process)."""
    v = np.asarray(values, dtype=np.float64)
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return v
    import torch

    t = torch.tensor(v, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM if op == "sum" else dist.ReduceOp.MAX)
    return t.cpu().numpy()


def job_rate(units_this_rank: float, elapsed_s: float, dist=None, device: str = "cpu") -> tuple[float, float]:
    """(whole-job units per second, slowest rank's elapsed seconds).  The job ends when its slowest
    rank does, so the rate is every rank's units over the maximum elapsed time."""
    units, = _reduce([units_this_rank], "sum", dist, device)
    slowest, = _reduce([elapsed_s], "max", dist, device)
    return float(units / slowest) if slowest > 0 else float("inf"), float(slowest)


def combine_moments(samples, dist=None, device: str = "cpu") -> tuple[float, float, int]:
    """(mean, standard error of the mean, count) of the union of every rank's samples."""
    x = np.asarray(samples, dtype=np.float64).reshape(-1)
    cnt, s1, s2 = _reduce([x.size, float(np.sum(x)), float(np.sum(x * x))], "sum", dist, device)
    n = int(round(cnt))
    if n == 0:
        return float("nan"), float("nan"), 0
    mean = s1 / n
    var = max(0.0, (s2 - n * mean * mean) / (n - 1)) if n > 1 else 0.0
    return float(mean), float(np.sqrt(var / n)), n


def traj_ensemble(n: int, ops, gamma: float, lam: float, seed: int, total: int, dist=None, device: str = "cpu",
                  precision: str = "complex128") -> dict:
    """A trajectory ensemble of `total` trajectories split across the ranks: each rank runs its
    shard on its own GPU, and the moments are combined on the host.  Every rank gets the result."""
    import llgpu

    rank = dist.get_rank() if dist is not None and dist.is_initialized() else 0
    world = dist.get_world_size() if dist is not None and dist.is_initialized() else 1
    begin, count = shard(total, rank, world)
    z0, jumps, _, margin = llgpu.traj_run(n, ops, gamma, lam, seed, count, begin=begin, precision=precision)
    mean, se, cnt = combine_moments(z0, dist, device)
    jump_sum, = _reduce([float(np.sum(jumps))], "sum", dist, device)
    return {"mean_z0": mean, "std_error": se, "trajectories": cnt, "jumps_per_traj": jump_sum / max(1, cnt),
            "shard": (begin, count), "min_margin": margin}
