"""The dense trajectory solver on the GPU (llg_tsolver_*): plan and trajectories against the
oracle's restatement on the same Philox stream, and the closed forms of the reference's own
checks (src/TrajectorySolver.h:588-770): T1 / T2 decay, the projector variance ratio
1 + exp(4 gamma t), rho against exact Lindblad integration (constant and driven H), and the
input contract."""
from __future__ import annotations

import numpy as np
import pytest

import llgpu
import oracle

pytestmark = pytest.mark.gpu

SX = np.array([[0, 1], [1, 0]], dtype=complex)
SZ = np.diag([1.0, -1.0]).astype(complex)
SM = np.array([[0, 1], [0, 0]], dtype=complex)
PLUS = np.array([1, 1]) / np.sqrt(2)


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    assert llgpu.device_count() > 0


def two_qubit_model():
    h = 0.3 * np.kron(SZ, np.eye(2)) + 0.2 * np.kron(np.eye(2), SZ) + 0.5 * np.kron(SX, SX)
    ch = [(np.kron(SM, np.eye(2)), 0.3), (np.kron(np.eye(2), SM), 0.2), (np.kron(SZ, np.eye(2)), 0.25),
          (np.kron(SX, SX), 0.1)]
    psi0 = np.array([1.0, 0.5, -0.3j, 0.2 + 0.1j])
    return h, ch, psi0 / np.linalg.norm(psi0)


@pytest.mark.parametrize("kind", ["STANDARD", "PROJECTOR", "ANALOG"])
def test_plan_and_trajectories_match_the_oracle(kind):
    h, ch, psi0 = two_qubit_model()
    s = llgpu.TrajectorySolver(2)
    s.set_hamiltonian(h)
    for l, g in ch:
        s.add_lindblad(l, g)
    dt = 0.004 if kind == "ANALOG" else 0.01
    st = s.states(psi0, 0.6, dt, 256, kind, seed=7)
    plan = s.plan()
    want_plan = oracle.tsolver_plan(h, ch, llgpu.UNRAVEL[kind], 0.6, dt)
    assert plan["steps"] == want_plan["steps"] and abs(plan["h"] - want_plan["h"]) < 1e-15
    assert np.max(np.abs(plan["prop"] - want_plan["prop"])) < 1e-13
    for a, b in zip(plan["ops"], want_plan["ops"]):
        assert np.max(np.abs(a - b)) < 1e-14
    want = oracle.tsolver_run(plan, psi0, 7, 0, 256)
    # same plan, same Philox draws: jump choices agree, states to rounding (ANALOG: the
    # Box-Muller increments go through the device and host math libraries)
    tol = 1e-9 if kind == "ANALOG" else 1e-11
    assert np.max(np.abs(st - want)) < tol
    s.close()


def test_driven_hamiltonian_rk4_matches_the_oracle():
    om, rabi = 1.3, 2.0
    hf = lambda t: 0.5 * rabi * np.sin(om * t) * SX + 0.25 * SZ  # noqa: E731
    s = llgpu.TrajectorySolver(1)
    s.set_hamiltonian(hf)
    s.add_lindblad(SM, 0.2)
    s.add_lindblad(SZ, 0.1)
    st = s.states([1, 0], 1.0, 0.01, 128, "STANDARD", seed=3)
    plan = s.plan()
    assert not plan["constant"] and plan["nodes"].shape[0] == 2 * plan["steps"] + 1
    want_plan = oracle.tsolver_plan(None, [(SM, 0.2), (SZ, 0.1)], 0, 1.0, 0.01, h_fn=hf)
    assert np.max(np.abs(plan["nodes"] - np.array(want_plan["nodes"]))) < 1e-14
    want = oracle.tsolver_run(plan, [1, 0], 3, 0, 128)
    assert np.max(np.abs(st - want)) < 1e-11
    s.close()


@pytest.mark.parametrize("kind", ["STANDARD", "PROJECTOR", "ANALOG"])
def test_t1_and_t2_closed_forms(kind):
    an = kind == "ANALOG"
    s = llgpu.TrajectorySolver(1)
    s.add_lindblad(SM, 0.5)
    assert not s.projector_applies(0)
    p1 = np.diag([0.0, 1.0])
    for f in (0.5, 1.0, 2.0):
        t = f * 2.0
        e = s.estimate_observable([0, 1], t, 0.005 if an else 0.02, 8000 if an else 20000, kind, p1, seed=101)
        assert abs(e["mean"] - np.exp(-t / 2.0)) <= 4 * e["std_error"] + (0.01 if an else 0.0)
    s.close()
    t1, tphi = 2.0, 1.5
    t2 = 1.0 / (0.5 / t1 + 1.0 / tphi)
    s = llgpu.TrajectorySolver(1)
    s.add_lindblad(SM, 1.0 / t1)
    s.add_lindblad(SZ, 0.5 / tphi)
    assert s.projector_applies(1) and not s.projector_applies(0)
    for f in (0.5, 1.0, 2.0):
        t = f * t2
        e = s.estimate_observable(PLUS, t, 0.005 if an else 0.02, 8000 if an else 20000, kind, SX, seed=202)
        assert abs(e["mean"] - np.exp(-t / t2)) <= 4 * e["std_error"] + (0.01 if an else 0.002)
    s.close()


def test_projector_variance_reduction():
    s = llgpu.TrajectorySolver(1)
    s.add_lindblad(SZ, 1.0)
    n, gt = 20000, 0.75
    es = s.estimate_observable(PLUS, gt, 0.005, n, "STANDARD", SX, seed=404)
    ep = s.estimate_observable(PLUS, gt, 0.005, n, "PROJECTOR", SX, seed=405)
    ratio = (es["std_error"] / ep["std_error"]) ** 2
    assert abs(ratio / (1 + np.exp(4 * gt)) - 1) < 0.10
    assert abs(ep["mean"] - np.exp(-2 * gt)) < 4 * ep["std_error"]
    # the callable form of the observable gives the same statistics
    ec = s.estimate_observable(PLUS, gt, 0.005, 2000, "PROJECTOR", lambda p: 2 * np.real(np.conj(p[0]) * p[1]), seed=9)
    em = s.estimate_observable(PLUS, gt, 0.005, 2000, "PROJECTOR", SX, seed=9)
    assert abs(ec["mean"] - em["mean"]) < 1e-12
    s.close()


def test_ensemble_rho_matches_exact_lindblad():
    h, ch, psi0 = two_qubit_model()
    exact = oracle.lindblad_exact(h, ch, np.outer(psi0, psi0.conj()), 1.5, 3000)
    s = llgpu.TrajectorySolver(2)
    s.set_hamiltonian(h)
    for l, g in ch:
        s.add_lindblad(l, g)
    for kind, dt, n, tol in (("STANDARD", 0.01, 20000, 0.02), ("PROJECTOR", 0.01, 20000, 0.02),
                             ("ANALOG", 0.004, 10000, 0.03)):
        rho = s.evolve_ensemble(psi0, 1.5, dt, n, kind, seed=501)
        assert np.max(np.abs(rho - exact)) < tol, kind
        assert abs(np.trace(rho) - 1) < 1e-12 and np.linalg.norm(rho - rho.conj().T) < 1e-12
        assert np.min(np.linalg.eigvalsh(0.5 * (rho + rho.conj().T))) > -1e-12
    s.close()


def test_reproducibility_and_contract():
    s = llgpu.TrajectorySolver(2)
    s.add_lindblad(np.kron(SM, np.eye(2)), 0.5)
    psi0 = np.array([0, 1, 1, 0], dtype=complex)
    a = s.evolve_ensemble(psi0, 1.0, 0.01, 300, "STANDARD", seed=7)
    b = s.evolve_ensemble(psi0, 1.0, 0.01, 300, "STANDARD", seed=7)
    assert np.array_equal(a, b)
    p1 = s.run_one(psi0, 1.0, 0.01, 7)
    assert np.array_equal(p1, s.run_one(psi0, 1.0, 0.01, 7)) and abs(np.linalg.norm(p1) - 1) < 1e-12
    single = s.evolve_ensemble(psi0, 1.0, 0.01, 1, "STANDARD", seed=7)
    assert np.linalg.norm(single - np.outer(p1, p1.conj())) < 1e-14
    with pytest.raises(ValueError):
        llgpu.TrajectorySolver(0)
    with pytest.raises(ValueError):
        llgpu.TrajectorySolver(11)
    with pytest.raises(ValueError):
        s.add_lindblad(SZ, 1.0)  # wrong size
    with pytest.raises(ValueError):
        s.add_lindblad(np.eye(4), -1.0)
    with pytest.raises(ValueError):
        s.set_hamiltonian(np.kron(SM, np.eye(2)))  # not Hermitian
    with pytest.raises(ValueError):
        s.run_one(psi0, 1.0, 0.0, 1)
    with pytest.raises(ValueError):
        s.evolve_ensemble(psi0, 1.0, 0.01, 0, "STANDARD", 1)
    with pytest.raises(ValueError):
        s.run_one([1, 0], 1.0, 0.01, 1)
    with pytest.raises(ValueError):
        s.run_one(np.zeros(4), 1.0, 0.01, 1)
    s.close()


def test_ten_qubit_dense_propagation():
    # dim = 1024: random Hermitian H and two jump channels, against the oracle on a few trajectories
    rng = np.random.default_rng(11)
    d = 1024
    a = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    h = (a + a.conj().T) / (4 * np.sqrt(d))
    l1 = np.kron(np.eye(d // 2), SM)  # sigma_- on qubit 0
    l2 = np.diag(np.where(np.arange(d) & 2, -1.0, 1.0)).astype(complex)  # Z on qubit 1
    s = llgpu.TrajectorySolver(10)
    s.set_hamiltonian(h)
    s.add_lindblad(l1, 0.4)
    s.add_lindblad(l2, 0.3)
    psi0 = rng.normal(size=d) + 1j * rng.normal(size=d)
    st = s.states(psi0, 0.2, 0.02, 64, "PROJECTOR", seed=5)
    plan = s.plan()
    want = oracle.tsolver_run(plan, psi0, 5, 0, 8)
    assert np.max(np.abs(st[:8] - want)) < 1e-10
    assert np.max(np.abs(np.linalg.norm(st, axis=1) - 1)) < 1e-12
    s.close()
