"""Density matrices on the GPU (llg_dm_apply_op / llg_dm_apply_kraus): rho against the oracle's
KrausChannel restatement through random circuits with interleaved channels, the channel
contract, and the Kraus-trajectory ensemble mean against the exact rho."""
from __future__ import annotations

import numpy as np
import pytest

import llgpu
import oracle
import workloads
from llgpu import OP_CNOT, OP_CZ, OP_H, OP_MCZ, OP_RX, OP_RY, OP_RZ, OP_U2, OP_X, make_ops

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    assert llgpu.device_count() > 0


def random_cptp(m, nk, rng):
    d = 1 << m
    a = rng.normal(size=(nk * d, d)) + 1j * rng.normal(size=(nk * d, d))
    q, _ = np.linalg.qr(a)  # isometry: stacked Kraus operators with sum K^+ K = I
    return [q[k * d:(k + 1) * d] for k in range(nk)]


@pytest.mark.parametrize("precision,tol", [("df64", 1e-12), ("fp64", 1e-12), ("complex64", 5e-6)])
@pytest.mark.parametrize("n", [3, 5, 7])
def test_rho_matches_oracle(precision, tol, n):
    rng = np.random.default_rng(40 + n)
    dm = llgpu.DensityMatrix(n, precision)
    want = oracle.dm_zero(n)
    for step in range(12):
        k = step % 6
        q = int(rng.integers(n))
        if k < 3:
            recs = [(OP_H, q), (OP_RX, q, 0, float(rng.uniform(-3, 3))), (OP_RZ, q, 0, float(rng.uniform(-3, 3)))]
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            recs += [(OP_CNOT, a, b), (OP_CZ, b, a), (OP_RY, a, 0, 0.7), (OP_X, b)]
            if n >= 3:
                recs.append((OP_MCZ, 0, 0, 0.0, 0b101))
            u, _ = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))
            recs.append((OP_U2, q, 0, 0.0, None, u.reshape(4)))
            ops = make_ops(recs)
            dm.apply_ops(ops)
            want = oracle.dm_apply_ops(want, n, ops)
        else:
            if k == 3:
                ch, tg = llgpu.amplitude_damping(0.2), [q]
            elif k == 4:
                ch, tg = llgpu.depolarizing(0.1, 2), [int(x) for x in rng.choice(n, 2, replace=False)]
            else:
                ch, tg = random_cptp(2, 3, rng), [int(x) for x in rng.choice(n, 2, replace=False)]
            dm.kraus(ch, tg)
            want = oracle.kraus_apply(want, n, ch, tg)
    got = dm.rho()
    assert np.max(np.abs(got - want)) <= tol
    assert abs(dm.trace() - 1) <= 10 * tol
    dm.close()


def test_channel_contract():
    dm = llgpu.DensityMatrix(3)
    with pytest.raises(ValueError):
        dm.kraus([np.eye(2) * 0.9], [0])  # not trace preserving
    with pytest.raises(ValueError):
        dm.kraus(llgpu.depolarizing(0.1, 2), [1, 1])  # repeated target
    with pytest.raises(ValueError):
        dm.kraus(llgpu.amplitude_damping(0.1), [3])  # outside the register
    with pytest.raises(ValueError):
        dm.kraus(random_cptp(3, 2, np.random.default_rng(0)), [0, 1, 2])  # 3 targets
    with pytest.raises(ValueError):
        dm.apply_ops(make_ops([(OP_H, 3)]))
    dm.close()


def test_trajectory_mean_matches_exact_rho():
    n, g, lam = 6, 0.05, 0.03
    ops = workloads.noisy_layers(n, 2, seed=8)
    dm = llgpu.DensityMatrix(n)
    for op in ops:
        dm.apply_ops(np.array([op]))
        qs = [int(op["q0"]), int(op["q1"])] if op["kind"] in (OP_CNOT, OP_CZ) else [int(op["q0"])]
        for q in qs:
            dm.kraus(llgpu.amplitude_damping(g), [q])
            dm.kraus(llgpu.phase_damping(lam), [q])
    p = dm.probabilities()
    z_exact = float(np.sum(p * (1 - 2 * (np.arange(1 << n) & 1))))
    assert abs(z_exact - oracle.density_z0(n, ops, g, lam)) < 1e-12
    z, _, _, _ = llgpu.traj_run(n, ops, g, lam, 31, 8192)
    se = z.std(ddof=1) / np.sqrt(z.size)
    assert abs(z.mean() - z_exact) < 5 * se
    dm.close()
