"""The NoisyBackend / ZNE restatement (oracle/noise_oracle.c) pinned to the reference's own
ll::NoisyBackend and ll::ZNE (fixtures written by tests/golden/gen_golden.py from the reference
build), and the Richardson algebra of src/Mitigation.h:287-301."""
from __future__ import annotations

import numpy as np
import pytest

import oracle

MT = oracle.RNG_MT
TERMS3 = [(0, 1, 1.0), (2, -1, 0.5)]


def test_mt19937_64_known_answer():
    # the C++ standard's check value for std::mt19937_64: the 10000th draw from the default seed
    assert oracle.lib().orc_mt64_first(5489, 9999) == 9981545732273789042


def test_noisy_backend_observables_match_the_reference(golden):
    g = golden("noisy_zne")
    ops = g["three_ops"]
    for key, p, scale, seed, ntraj in (("obs3_p05_s1", 0.05, 1, 2024, 200), ("obs3_p05_s3", 0.05, 3, 2024, 200),
                                       ("obs3_p0_s5", 0.0, 5, 1, 3)):
        obs, _ = oracle.noisy_run(3, ops, p, scale, seed, 0, ntraj, TERMS3, rng=MT)
        assert np.max(np.abs(obs - g[key])) <= 1e-12, key


@pytest.mark.parametrize("case,n,p,seed,scales,ntraj,terms", [
    ("zne3", 3, 0.03, 77, [1, 3, 5], 300, TERMS3),
    ("zne1", 1, 0.02, 2024, [1, 3], 2000, [(0, -1, 1.0)]),
    ("zne_bell", 2, 0.03, 99, [1, 3], 1000, [(0, 1, 1.0)]),
    ("zne_p0", 3, 0.0, 5, [1, 3, 5], 7, TERMS3),
    ("zne_single", 1, 0.02, 3, [1, 3], 1, [(0, -1, 1.0)]),
])
def test_zne_matches_the_reference(golden, case, n, p, seed, scales, ntraj, terms):
    g = golden("noisy_zne")
    ops = g["bell_ops"] if "bell" in case else (g["three_ops"] if n == 3 else g["one_ops"])
    want = g[case]
    ns = len(scales)
    r = oracle.zne(n, ops, p, scales, ntraj, seed, terms, rng=MT)
    assert r["trajectories"] == int(want[2])
    np.testing.assert_allclose(r["values"], want[3:3 + ns], rtol=0, atol=1e-12)
    np.testing.assert_allclose(r["weights"], want[3 + 2 * ns:3 + 3 * ns], rtol=0, atol=1e-15)
    if np.isnan(want[1]):
        assert np.isnan(r["std_error"]) and np.all(np.isnan(r["std_errors"]) == np.isnan(want[3 + ns:3 + 2 * ns]))
    else:
        np.testing.assert_allclose(r["std_errors"], want[3 + ns:3 + 2 * ns], rtol=1e-9, atol=1e-15)
        assert abs(r["std_error"] - want[1]) <= 1e-9 * max(1.0, want[1])
    assert abs(r["value"] - want[0]) <= 1e-12


def test_zne_contract_matches_the_reference(golden):
    g = golden("noisy_zne")
    assert int(g["zne_rc_bad_scale"]) == 1 and int(g["zne_rc_no_gates"]) == 3
    with pytest.raises(ValueError):
        oracle.zne(1, g["one_ops"], 0.02, [1, 4], 10, 1, rng=MT)
    with pytest.raises(RuntimeError):
        oracle.zne(1, g["one_ops"][:0], 0.02, [1, 3], 10, 1, rng=MT)
    for bad in ([1], [1, 3, 3], [1, 2.5], [-1, 1], [1, 101], list(range(1, 19, 2))):
        with pytest.raises(ValueError):
            oracle.zne(1, g["one_ops"], 0.02, bad, 10, 1, rng=MT)


def test_richardson_weights_and_moments():
    np.testing.assert_allclose(oracle.richardson_weights([1, 3, 5]), [15 / 8, -5 / 4, 3 / 8], atol=1e-15)
    w4 = oracle.richardson_weights([1, 3, 5, 7])
    np.testing.assert_allclose(w4, [2.1875, -2.1875, 1.3125, -0.3125], atol=1e-13)
    s = np.array([1.0, 3.0, 5.0, 7.0])
    for m in range(1, 4):
        assert abs(np.sum(w4 * s ** m)) < 1e-10
    assert abs(np.sum(w4) - 1) < 1e-12
    with pytest.raises(ValueError):
        oracle.richardson_weights([2.0, 2.0])


def test_philox_stream_reproduces_analytic_decay():
    # 1 qubit, 3 rotations: E(lambda) = z0 (1 - 4p/3)^(3 lambda) exactly (src/Mitigation.h:56-60)
    from llgpu import OP_RX, OP_RY, OP_RZ, make_ops

    ops = make_ops([(OP_RY, 0, 0, 0.9), (OP_RZ, 0, 0, -0.6), (OP_RX, 0, 0, 0.35)])
    z0 = oracle.noisy_run(1, ops, 0.0, 1, 1, 0, 1)[0][0]
    p, r1 = 0.02, 1 - 4 * 0.02 / 3
    for scale in (1, 3):
        obs, _ = oracle.noisy_run(1, ops, p, scale, 11, 0, 40000)
        se = obs.std(ddof=1) / np.sqrt(obs.size)
        assert abs(obs.mean() - z0 * r1 ** (3 * scale)) < 5 * se
