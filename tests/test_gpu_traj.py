"""Batched noisy trajectories on the GPU against the oracle's restatement of the Kraus-jump step.

Jump choices must be bit-identical to the oracle's for the same Philox stream (complex128
precisions); the oracle reports the smallest |u - survive| margin of all draws, and a decision
closer than 1e-12 would count as a tie (none occur in these cases).  Final <Z_0> per trajectory
to 1e-10.  Complex64 trajectories are checked statistically.  Means are checked against the
exact density-matrix evolution within 5 standard errors."""
from __future__ import annotations

import numpy as np
import pytest

import llgpu
import oracle
import workloads
from llgpu import OP_CNOT, OP_CZ, OP_H, OP_MCZ, OP_RX, OP_RZ, make_ops

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    assert llgpu.device_count() > 0


def check_exact(n, ops, gamma, lam, seed, count, precision, begin=0):
    sites = llgpu.noise_sites(ops)
    z, j, log, margin = llgpu.traj_run(n, ops, gamma, lam, seed, count, begin, precision, log=True)
    zo, jo, logo, margin_o = oracle.traj_run(n, ops, gamma, lam, seed, begin, begin + count, log_sites=sites)
    assert margin_o > 1e-12, "a near-tie decision: choose another seed"
    assert np.array_equal(log, logo)
    assert np.array_equal(j, jo)
    assert np.max(np.abs(z - zo)) <= 1e-10
    assert abs(margin - margin_o) <= 1e-9
    return z, j


@pytest.mark.parametrize("precision", ["df64", "fp64"])
def test_config4_circuit_jumps_bit_exact_14_qubits(precision):
    # 14 qubits of complex128 need a 2-CTA cluster: exercises the cross-CTA paths
    ops = workloads.noisy_layers(14, 8)
    z, j = check_exact(14, ops, 0.01, 0.005, seed=2024, count=48, precision=precision)
    assert j.sum() > 0


@pytest.mark.parametrize("precision", ["df64", "fp64"])
@pytest.mark.parametrize("n", [3, 7, 10])
def test_strong_noise_jumps_bit_exact(n, precision):
    ops = workloads.noisy_layers(n, 3, seed=n)
    check_exact(n, ops, 0.25, 0.15, seed=77, count=256, precision=precision)


@pytest.mark.parametrize("precision", ["df64", "fp64"])
def test_every_gate_kind_and_cross_cta_sites(precision):
    rng = np.random.default_rng(5)
    n = 14
    recs = []
    for _ in range(40):
        k = rng.integers(5)
        q = int(rng.integers(n))
        if k == 0:
            recs.append((OP_H, q))
        elif k == 1:
            recs.append((OP_RX, q, 0, float(rng.uniform(0, 6))))
        elif k == 2:
            recs.append((OP_RZ, q, 0, float(rng.uniform(0, 6))))
        elif k == 3:
            a, b = rng.choice(n, 2, replace=False)
            recs.append(((OP_CNOT, OP_CZ)[int(rng.integers(2))], int(a), int(b)))
        else:
            qs = rng.choice(n, 3, replace=False)
            recs.append((OP_MCZ, 0, 0, 0.0, int(sum(1 << int(x) for x in qs))))
    # make sure the top qubit (the one split across the cluster) is hit as target and control
    recs += [(OP_H, 13), (OP_CNOT, 13, 2), (OP_CNOT, 4, 13), (OP_RZ, 13, 0, 0.3), (OP_CZ, 13, 0)]
    ops = make_ops(recs)
    check_exact(n, ops, 0.3, 0.2, seed=9, count=32, precision=precision)


def test_trajectory_ranges_are_reproducible():
    ops = workloads.noisy_layers(12, 4, seed=1)
    z_all, j_all, log_all, _ = llgpu.traj_run(12, ops, 0.05, 0.05, 3, 64, 0, log=True)
    z_b, j_b, log_b, _ = llgpu.traj_run(12, ops, 0.05, 0.05, 3, 32, 32, log=True)
    assert np.array_equal(z_all[32:], z_b) and np.array_equal(log_all[32:], log_b)


def test_mean_matches_density_matrix():
    n = 6
    ops = workloads.noisy_layers(n, 3, seed=6)
    gamma, lam = 0.1, 0.05
    exact = oracle.density_z0(n, ops, gamma, lam)
    for precision in ("df64", "complex64"):
        z, _, _, _ = llgpu.traj_run(n, ops, gamma, lam, 123, 8192, precision=precision)
        se = z.std(ddof=1) / np.sqrt(z.size)
        assert abs(z.mean() - exact) < 5 * se, (precision, z.mean(), exact, se)


def test_complex64_trajectories_track_complex128():
    ops = workloads.noisy_layers(14, 8)
    z128, _, log128, _ = llgpu.traj_run(14, ops, 0.01, 0.005, 2024, 256, log=True)
    z64, _, log64, _ = llgpu.traj_run(14, ops, 0.01, 0.005, 2024, 256, precision="complex64", log=True)
    same = np.all(log64 == log128, axis=1)
    assert same.mean() > 0.95
    assert np.max(np.abs(z64[same] - z128[same])) <= 1e-4


def test_full_config4_ensemble():
    """4096 trajectories x 14 qubits x 328 gates, complex128: mean <Z_0> with its standard error;
    the first trajectories are checked against the oracle bit for bit."""
    ops = workloads.noisy_layers(14, 8)
    z, j, log, margin = llgpu.traj_run(14, ops, 0.01, 0.005, 2024, 4096, log=True)
    assert margin > 1e-12
    assert np.all(np.isfinite(z)) and np.all(np.abs(z) <= 1 + 1e-12)
    sites = llgpu.noise_sites(ops)
    zo, jo, logo, _ = oracle.traj_run(14, ops, 0.01, 0.005, 2024, 0, 16, log_sites=sites)
    assert np.array_equal(log[:16], logo) and np.max(np.abs(z[:16] - zo)) <= 1e-10
    assert j.sum() > 100


def test_shards_reproduce_the_ensemble():
    """Trajectory i depends only on (seed, i): two shards run separately equal the single run
    unit for unit, and replicas.traj_ensemble on one process reports the run's moments."""
    import replicas

    n, total, seed = 12, 300, 31
    ops = workloads.noisy_layers(n, 3)
    z_all, j_all, _, _ = llgpu.traj_run(n, ops, 0.02, 0.01, seed, total)
    b, c = replicas.shard(total, 1, 2)
    z_lo, j_lo, _, _ = llgpu.traj_run(n, ops, 0.02, 0.01, seed, b, begin=0)
    z_hi, j_hi, _, _ = llgpu.traj_run(n, ops, 0.02, 0.01, seed, c, begin=b)
    assert np.array_equal(np.concatenate([z_lo, z_hi]), z_all)
    assert np.array_equal(np.concatenate([j_lo, j_hi]), j_all)
    r = replicas.traj_ensemble(n, ops, 0.02, 0.01, seed, total)
    assert r["trajectories"] == total and r["shard"] == (0, total)
    assert abs(r["mean_z0"] - float(np.mean(z_all))) <= 1e-14
    assert abs(r["std_error"] - float(np.std(z_all, ddof=1) / np.sqrt(total))) <= 1e-14
