"""Batched ll::NoisyBackend (depolarizing Pauli noise with gate folding) and ZNE on the GPU,
against the oracle's restatement on the same Philox stream (oracle/noise_oracle.c, itself pinned to
the reference's NoisyBackend / ZNE in tests/test_oracle_noise.py), and against the closed forms
of src/Mitigation.h:17-20 and :56-60."""
from __future__ import annotations

import numpy as np
import pytest

import llgpu
import oracle
import workloads
from llgpu import OP_CNOT, OP_H, OP_RX, OP_RY, OP_RZ, make_ops

pytestmark = pytest.mark.gpu

TERMS3 = [(0, 1, 1.0), (2, -1, 0.5)]
TOL = {"df64": 1e-12, "fp64": 1e-12, "complex64": 2e-5}


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    assert llgpu.device_count() > 0


@pytest.mark.parametrize("precision", ["df64", "fp64", "complex64"])
@pytest.mark.parametrize("scale", [1, 3])
def test_pauli_choices_match_the_oracle(golden, precision, scale):
    ops = golden("noisy_zne")["three_ops"]
    h = llgpu.NoisyTraj(3, ops, 0.05, scale, 500, TERMS3, precision)
    obs, paulis, _ = h.launch(2024, 500, begin=100)
    want, wpaulis = oracle.noisy_run(3, ops, 0.05, scale, 2024, 100, 600, TERMS3)
    assert np.array_equal(paulis, wpaulis)
    assert np.max(np.abs(obs - want)) <= TOL[precision]
    h.close()


@pytest.mark.parametrize("n,precision", [(14, "df64"), (14, "complex64"), (10, "df64")])
def test_wide_states_with_cross_cta_paulis(n, precision):
    # 14-qubit complex128 states span a 2-CTA cluster: Paulis on the top qubit cross CTAs
    ops = workloads.noisy_layers(n, 2)
    terms = [(0, n - 1, 1.0), (n - 1, -1, -0.25), (3, 4, 1.0)]
    h = llgpu.NoisyTraj(n, ops, 0.02, 3, 64, terms, precision)
    obs, paulis, _ = h.launch(7, 64)
    want, wpaulis = oracle.noisy_run(n, ops, 0.02, 3, 7, 0, 64, terms)
    assert np.array_equal(paulis, wpaulis) and paulis.sum() > 50
    assert np.max(np.abs(obs - want)) <= TOL[precision]
    if n == 14 and precision == "df64":
        assert h.config()["cluster"] == 2
    h.close()


def test_noiseless_folding_is_the_identity(golden):
    ops = golden("noisy_zne")["three_ops"]
    ideal = oracle.expect_zz(oracle.run_ops(3, ops), 3, [0, 2], [1, -1], [1.0, 0.5])
    h = llgpu.NoisyTraj(3, ops, 0.0, 5, 4, TERMS3)
    obs, paulis, _ = h.launch(1, 4)
    assert np.all(paulis == 0) and np.max(np.abs(obs - ideal)) <= 1e-12
    h.close()


def test_depolarizing_decay_closed_forms():
    # 1 qubit, 3 gates: E(l) = z0 (1 - 4p/3)^(3 l); Bell pair: <ZZ>(l) = (1 - 16p/15)^l
    one = make_ops([(OP_RY, 0, 0, 0.9), (OP_RZ, 0, 0, -0.6), (OP_RX, 0, 0, 0.35)])
    z0 = oracle.expect_zz(oracle.run_ops(1, one), 1, [0], [-1], [1.0])
    p = 0.02
    for scale in (1, 3, 5):
        h = llgpu.NoisyTraj(1, one, p, scale, 60000)
        obs, _, _ = h.launch(2024 + scale, 60000)
        se = obs.std(ddof=1) / np.sqrt(obs.size)
        assert abs(obs.mean() - z0 * (1 - 4 * p / 3) ** (3 * scale)) < 5 * se
        h.close()
    bell = make_ops([(OP_H, 0), (OP_CNOT, 0, 1)])
    p2 = 0.03
    for scale in (1, 3):
        h = llgpu.NoisyTraj(2, bell, p2, scale, 40000, [(0, 1, 1.0)])
        obs, _, _ = h.launch(99 + scale, 40000)
        se = obs.std(ddof=1) / np.sqrt(obs.size)
        assert abs(obs.mean() - (1 - 16 * p2 / 15) ** scale) < 5 * se
        h.close()


@pytest.mark.parametrize("precision", ["df64", "complex64"])
def test_zne_matches_the_oracle(golden, precision):
    ops = golden("noisy_zne")["three_ops"]
    r = llgpu.zne(3, ops, 0.03, [1, 3, 5], 2000, 77, TERMS3, precision)
    w = oracle.zne(3, ops, 0.03, [1, 3, 5], 2000, 77, TERMS3)
    assert r["trajectories"] == w["trajectories"] == 2000
    np.testing.assert_array_equal(r["weights"], w["weights"])
    tol = TOL[precision]
    np.testing.assert_allclose(r["values"], w["values"], rtol=0, atol=tol)
    np.testing.assert_allclose(r["std_errors"], w["std_errors"], rtol=1e-6 if precision == "complex64" else 1e-9)
    assert abs(r["value"] - w["value"]) <= 4 * tol


def test_zne_extrapolates_towards_the_ideal():
    one = make_ops([(OP_RY, 0, 0, 0.9), (OP_RZ, 0, 0, -0.6), (OP_RX, 0, 0, 0.35)])
    z0 = oracle.expect_zz(oracle.run_ops(1, one), 1, [0], [-1], [1.0])
    p, r1 = 0.02, 1 - 4 * 0.02 / 3
    r = llgpu.zne(1, one, p, [1, 3, 5], 60000, 5)
    ana = sum(c * z0 * r1 ** (3 * s) for c, s in zip([15 / 8, -5 / 4, 3 / 8], [1, 3, 5]))
    assert abs(r["value"] - ana) < 5 * r["std_error"]
    assert abs(r["value"] - z0) < abs(r["values"][0] - z0)  # mitigated error below unmitigated
    # p = 0: one trajectory per scale, exact value, zero error
    r0 = llgpu.zne(1, one, 0.0, [1, 3], 100, 5)
    assert r0["trajectories"] == 1 and r0["std_error"] == 0.0 and abs(r0["value"] - z0) <= 1e-12
    # one noisy trajectory: the error is not estimable (NaN), as in the reference
    r1t = llgpu.zne(1, one, 0.02, [1, 3], 1, 5)
    assert np.isnan(r1t["std_error"])


def test_noisy_contract():
    one = make_ops([(OP_RY, 0, 0, 0.9)])
    for p in (-0.1, 1.2, float("nan")):
        with pytest.raises(ValueError):
            llgpu.NoisyTraj(1, one, p, 1, 4)
    for scale in (0, 2, 101):
        with pytest.raises(ValueError):
            llgpu.NoisyTraj(1, one, 0.1, scale, 4)
    with pytest.raises(ValueError):
        llgpu.NoisyTraj(1, one, 0.1, 1, 4, [(0, 0, 1.0)])  # a ZZ term on one qubit
    with pytest.raises(ValueError):
        llgpu.NoisyTraj(2, one, 0.1, 1, 4, [(0, 1, 1.0), (0, -1, 2.0), (1, -1, 3.0), (0, 1, 4.0)])  # 4 classes
    with pytest.raises(ValueError):
        llgpu.zne(1, one, 0.1, [1, 4], 10)
    with pytest.raises(llgpu.LLGError):
        llgpu.zne(1, one[:0], 0.1, [1, 3], 10)
