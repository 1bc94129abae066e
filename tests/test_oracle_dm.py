"""The KrausChannel restatement (oracle/dm_oracle.c) against the closed forms the reference
states for its channels (src/Noise.h:80-84, :149-167) and against the trajectory oracle's own
density-matrix evolution (oracle/traj_oracle.c)."""
from __future__ import annotations

import numpy as np
import pytest

import llgpu
import oracle
import workloads


def test_amplitude_and_phase_damping_closed_forms():
    g, lam = 0.3, 0.2
    one = np.zeros((2, 2), dtype=complex)
    one[1, 1] = 1.0
    out = oracle.kraus_apply(one, 1, llgpu.amplitude_damping(g), [0])
    np.testing.assert_allclose(out, np.diag([g, 1 - g]), atol=1e-15)
    plus = np.full((2, 2), 0.5, dtype=complex)
    ad = oracle.kraus_apply(plus, 1, llgpu.amplitude_damping(g), [0])
    assert abs(ad[0, 1] - 0.5 * np.sqrt(1 - g)) < 1e-15
    pd = oracle.kraus_apply(plus, 1, llgpu.phase_damping(lam), [0])
    np.testing.assert_allclose(np.diag(pd), [0.5, 0.5], atol=1e-15)
    assert abs(pd[0, 1] - 0.5 * np.sqrt(1 - lam)) < 1e-15


def test_depolarizing_closed_forms():
    p = 0.12
    rng = np.random.default_rng(2)
    v = rng.normal(size=2) + 1j * rng.normal(size=2)
    v /= np.linalg.norm(v)
    rho = np.outer(v, v.conj())
    out = oracle.kraus_apply(rho, 1, llgpu.depolarizing(p, 1), [0])
    for P in llgpu._PAULI[1:]:
        assert abs(np.trace(out @ P) - (1 - 4 * p / 3) * np.trace(rho @ P)) < 1e-14
    # two qubits: every non-identity Pauli expectation shrinks by 1 - 16p/15; on a 3-qubit rho
    # with targets (2, 0) the untouched qubit is unchanged
    w = rng.normal(size=8) + 1j * rng.normal(size=8)
    w /= np.linalg.norm(w)
    rho3 = np.outer(w, w.conj())
    out3 = oracle.kraus_apply(rho3, 3, llgpu.depolarizing(p, 2), [2, 0])
    Z = np.diag([1.0, -1.0])
    I2 = np.eye(2)
    zz = np.kron(Z, np.kron(I2, Z))  # Z on qubits 2 and 0 (qubit 0 is the last factor)
    assert abs(np.trace(out3 @ zz) - (1 - 16 * p / 15) * np.trace(rho3 @ zz)) < 1e-14
    z1 = np.kron(I2, np.kron(Z, I2))
    assert abs(np.trace(out3 @ z1) - np.trace(rho3 @ z1)) < 1e-14


def test_trace_preservation_check():
    assert oracle.kraus_trace_preserving(llgpu.amplitude_damping(0.4))
    assert oracle.kraus_trace_preserving(llgpu.depolarizing(0.3, 2))
    assert not oracle.kraus_trace_preserving([np.eye(2) * 0.99])


def test_agrees_with_the_trajectory_oracle_density_path():
    n, g, lam = 4, 0.05, 0.03
    ops = workloads.noisy_layers(n, 2, seed=8)
    rho = oracle.dm_zero(n)
    for op in ops:
        rho = oracle.dm_apply_ops(rho, n, np.array([op]))
        qs = [int(op["q0"]), int(op["q1"])] if op["kind"] in (llgpu.OP_CNOT, llgpu.OP_CZ) else [int(op["q0"])]
        for q in qs:
            rho = oracle.kraus_apply(rho, n, llgpu.amplitude_damping(g), [q])
            rho = oracle.kraus_apply(rho, n, llgpu.phase_damping(lam), [q])
    z0 = float(np.real(np.sum(np.diag(rho) * (1 - 2 * (np.arange(1 << n) & 1)))))
    assert abs(z0 - oracle.density_z0(n, ops, g, lam)) < 1e-13
    assert abs(np.trace(rho) - 1) < 1e-13
