"""The TrajectorySolver restatement (oracle/tsolver_oracle.c + oracle.tsolver_plan) against the
closed forms the reference checks its solver with (src/TrajectorySolver.h:588-653): T1 decay,
T2 decay, and the ensemble rho against an exact RK4 integration of the Lindblad equation."""
from __future__ import annotations

import numpy as np
import pytest

import oracle

SX = np.array([[0, 1], [1, 0]], dtype=complex)
SZ = np.diag([1.0, -1.0]).astype(complex)
SM = np.array([[0, 1], [0, 0]], dtype=complex)  # |0><1|


def test_expm_matches_scipy():
    scipy_linalg = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(4)
    for d in (2, 4, 16):
        a = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) * 0.7
        assert np.max(np.abs(oracle.expm(a) - scipy_linalg.expm(a))) < 1e-12 * max(1.0, np.abs(scipy_linalg.expm(a)).max())


def test_pauli_like_detection():
    assert oracle.pauli_like(SZ)[0] and oracle.pauli_like(np.kron(SX, SX))[0]
    assert not oracle.pauli_like(SM)[0]


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_t1_decay(kind):
    t1, t = 2.0, 2.0
    dt = 0.005 if kind == 2 else 0.02
    plan = oracle.tsolver_plan(np.zeros((2, 2), dtype=complex), [(SM, 1.0 / t1)], kind, t, dt)
    st = oracle.tsolver_run(plan, [0, 1], 101, 0, 3000)
    p1 = np.abs(st[:, 1]) ** 2
    se = p1.std(ddof=1) / np.sqrt(p1.size)
    assert abs(p1.mean() - np.exp(-t / t1)) <= 4 * se + (0.01 if kind == 2 else 0.0)


def test_t2_decay_projector():
    t1, tphi = 2.0, 1.5
    t2 = 1.0 / (0.5 / t1 + 1.0 / tphi)
    plan = oracle.tsolver_plan(np.zeros((2, 2), dtype=complex), [(SM, 1.0 / t1), (SZ, 0.5 / tphi)], 1, t2, 0.02)
    st = oracle.tsolver_run(plan, np.array([1, 1]) / np.sqrt(2), 202, 0, 3000)
    x = 2 * np.real(np.conj(st[:, 0]) * st[:, 1])
    se = x.std(ddof=1) / np.sqrt(x.size)
    assert abs(x.mean() - np.exp(-1.0)) <= 4 * se + 0.002


def test_ensemble_rho_matches_exact_lindblad():
    h = 0.3 * np.kron(SZ, np.eye(2)) + 0.2 * np.kron(np.eye(2), SZ) + 0.5 * np.kron(SX, SX)
    ch = [(np.kron(SM, np.eye(2)), 0.3), (np.kron(np.eye(2), SM), 0.2), (np.kron(SZ, np.eye(2)), 0.25),
          (np.kron(SX, SX), 0.1)]
    psi0 = np.array([1.0, 0.5, -0.3j, 0.2 + 0.1j])
    psi0 /= np.linalg.norm(psi0)
    exact = oracle.lindblad_exact(h, ch, np.outer(psi0, psi0.conj()), 1.5, 1500)
    for kind in (0, 1):
        plan = oracle.tsolver_plan(h, ch, kind, 1.5, 0.01)
        st = oracle.tsolver_run(plan, psi0, 501 + kind, 0, 4000)
        rho = st.T @ st.conj() / st.shape[0]
        assert np.max(np.abs(rho - exact)) < 0.03
        assert abs(np.trace(rho) - 1) < 1e-12
