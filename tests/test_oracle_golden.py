"""The oracle (oracle/*.c) pinned against outputs of the reference's own code (tests/golden,
written by tests/golden/gen_golden.py from the reference build) and against the closed forms
and published numbers the reference states.  CPU only."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import workloads
from conftest import split, split_states
from llgpu import OP_CNOT, OP_CZ, OP_DTYPE, OP_H, OP_MCZ, OP_RX, OP_RY, OP_RZ, OP_X, make_ops


def test_random_2024_matches_reference_backends(golden):
    # tests/test_backends.cpp:205-232 recipe; the oracle restates StateVectorBackend's arithmetic,
    # so it must agree with it bit for bit and with ReferenceBackend to 1e-12
    g = golden("random_2024")
    circuits = split(g["ops"], g["offsets"])
    refs = split_states(g["ref_states"], g["state_offsets"])
    svs = split_states(g["sv_states"], g["state_offsets"])
    for n, ops, ref, sv in zip(g["n"], circuits, refs, svs):
        psi = oracle.run_ops(int(n), ops)
        assert np.array_equal(psi, sv)
        assert np.max(np.abs(psi - ref)) < 1e-12


def test_config1_matches_reference(golden):
    g = golden("config1_h_cnot")
    for n, ops, ref in zip(g["n"], split(g["ops"], g["offsets"]), split_states(g["states"], g["state_offsets"])):
        assert np.array_equal(oracle.run_ops(int(n), ops), ref)


def test_config1_workload_is_the_recipe():
    ops = workloads.mixed_h_cnot(12, 1000, seed=1234)
    assert len(ops) == 1000
    kinds = ops["kind"]
    assert set(np.unique(kinds)) <= {OP_H, OP_CNOT}
    cn = ops[kinds == OP_CNOT]
    assert np.all(cn["q0"] != cn["q1"])
    assert 400 < np.sum(kinds == OP_H) < 600


def test_config2_matches_reference(golden):
    g = golden("config2_layered")
    for n, ops, ref in zip(g["n"], split(g["ops"], g["offsets"]), split_states(g["states"], g["state_offsets"])):
        assert np.array_equal(oracle.run_ops(int(n), ops), ref)


def test_config2_gate_counts():
    ops = workloads.layered_rotations(30, layers=20)
    assert np.sum(ops["kind"] == OP_CNOT) == 290
    assert np.sum(np.isin(ops["kind"], [OP_RX, OP_RY, OP_RZ])) == 1800


def test_v3_gate_semantics_match_reference(golden):
    g = golden("v3_gates")
    n = int(g["n"])
    for label, fn, skip_oob in (("v3_cache", oracle.apply_gate_v3, False),
                                ("v3_standard", oracle.apply_gate_standard, True),
                                ("v2", oracle.apply_gate_standard, True)):
        psi = g["init"].copy()
        for t, gate in zip(g["targets"], g["gates"]):
            if skip_oob and t >= n:
                continue
            fn(psi, n, int(t), gate)
        assert np.array_equal(psi, g[label]), label


def test_gate_fuser_matches_reference(golden):
    from gate_fusion import GATES, GateFuser

    g = golden("gate_fusion")
    for label in ("bench", "mixed"):
        circuit = list(zip(g[label + "_in_targets"].tolist(), [list(x) for x in g[label + "_in_gates"]]))
        fused = GateFuser.fuse_circuit(circuit)
        assert [t for t, _ in fused] == g[label + "_targets"].tolist()
        assert np.array_equal(np.array([np.asarray(x) for _, x in fused]), g[label + "_gates"])
    assert GATES["S"] == [1 + 0j, 0j, 0j, 1j]


def grover_ops(n, marked, iterations):
    """The gate sequence of ll::Grover::run (src/Algorithms.h:85-90, :111-124)."""
    rec = [(OP_H, q) for q in range(n)]
    full = (1 << n) - 1
    for _ in range(iterations):
        for m in marked:
            rec += [(OP_X, q) for q in range(n) if not (m >> q) & 1]
            rec.append((OP_MCZ, 0, 0, 0.0, full))
            rec += [(OP_X, q) for q in range(n) if not (m >> q) & 1]
        for q in range(n):
            rec += [(OP_H, q), (OP_X, q)]
        rec.append((OP_MCZ, 0, 0, 0.0, full))
        for q in range(n):
            rec += [(OP_X, q), (OP_H, q)]
    return make_ops(rec)


def test_grover_matches_reference_and_published(golden):
    g = golden("grover")
    # README.md:509: n = 8, marked 85, 12 iterations, P = 0.99994704
    assert int(g["n8_m85_iterations"]) == 12 and int(g["n8_m85_marked_index"]) == 85
    for key, n in (("n8_m85", 8), ("n10_i10", 10), ("n12_i10", 12)):
        probs = oracle.probabilities(oracle.run_ops(n, grover_ops(n, g[key + "_marked"].tolist(),
                                                                   int(g[key + "_iterations"]))), n)
        assert np.max(np.abs(probs - g[key + "_probs"])) < 1e-12
    assert abs(g["n8_m85_probs"][85] - 0.99994704) < 5e-9
    # docs/library_comparison.json:39 (n = 10, 10 iterations, marked 2^n // 3)
    assert abs(g["n10_i10_probs"][(1 << 10) // 3] - 0.37238643309688396) < 1e-12


def vqe_ops(n, layers, theta):
    """ll::VQE::prepare (src/Algorithms.h:240-252): RY layer then CNOT ring, per layer."""
    rec = []
    for l in range(layers):
        rec += [(OP_RY, q, 0, float(theta[l * n + q]), None, None, l * n + q) for q in range(n)]
        if n == 2:
            rec.append((OP_CNOT, 0, 1))
        elif n > 2:
            rec += [(OP_CNOT, q, (q + 1) % n) for q in range(n)]
    return make_ops(rec)


def test_vqe_parameter_shift_matches_reference(golden):
    g = golden("vqe_param_shift")
    for n, layers in ((4, 2), (6, 3)):
        key = f"n{n}_l{layers}"
        theta = g[key + "_theta"]
        ops = vqe_ops(n, layers, theta)
        assert np.array_equal(oracle.run_ops(n, ops), g[key + "_state"])
        a, b = list(range(n)), [(i + 1) % n for i in range(n)]
        e, grad = oracle.param_shift(n, ops, theta, a, b, [1.0] * n)
        assert abs(e - g[key + "_energy"]) < 1e-12
        assert np.max(np.abs(grad - g[key + "_grad"])) < 1e-12


def test_hea_parameter_shift_matches_reference(golden):
    g = golden("hea_param_shift")
    n = int(g["n"])
    a, b = list(range(n)), [(i + 1) % n for i in range(n)]
    for params, e_ref, g_ref in zip(g["params"], g["energies"], g["grads"]):
        e, grad = oracle.param_shift(n, g["ops"], params, a, b, [1.0] * n)
        assert abs(e - e_ref) < 1e-12
        assert np.max(np.abs(grad - g_ref)) < 1e-12


def test_closed_forms():
    # tests/test_backends.cpp:148-203
    r = 1 / np.sqrt(2)
    p = oracle.probabilities(oracle.run_ops(4, make_ops([(OP_X, 2)])), 4)
    assert p[4] > 1 - 1e-14
    p = oracle.probabilities(oracle.run_ops(2, make_ops([(OP_H, 0), (OP_CNOT, 0, 1)])), 2)
    assert abs(p[0] - 0.5) < 1e-14 and abs(p[3] - 0.5) < 1e-14
    assert oracle.probabilities(oracle.run_ops(3, make_ops([(OP_X, 2), (OP_CNOT, 2, 0)])), 3)[5] > 1 - 1e-14
    assert oracle.probabilities(oracle.run_ops(3, make_ops([(OP_X, 0), (OP_CNOT, 0, 2)])), 3)[5] > 1 - 1e-14
    assert oracle.probabilities(oracle.run_ops(1, make_ops([(OP_RY, 0, 0, np.pi)])), 1)[1] > 1 - 1e-14
    assert abs(oracle.run_ops(1, make_ops([(OP_RX, 0, 0, np.pi)]))[1] - (-1j)) < 1e-14
    s = oracle.run_ops(1, make_ops([(OP_H, 0), (OP_RZ, 0, 0, 0.7)]))
    assert abs(s[0] - r * np.exp(-0.35j)) < 1e-14 and abs(s[1] - r * np.exp(0.35j)) < 1e-14
    m = oracle.run_ops(3, make_ops([(OP_H, 0), (OP_H, 1), (OP_H, 2), (OP_MCZ, 0, 0, 0.0, 7)]))
    assert abs(m[7] + r ** 3) < 1e-14 and np.all(np.abs(m[:7] - r ** 3) < 1e-14)


def test_oracle_rejects_what_the_reference_rejects():
    # tests/test_backends.cpp:282-302 contract, through the oracle's op runner
    nan = float("nan")
    for rec in [(OP_H, -1), (OP_X, 3), (OP_RX, 0, 0, nan), (OP_RY, 0, 0, float("inf")), (OP_RZ, 5, 0, 0.1),
                (OP_CNOT, 1, 1), (OP_CNOT, 0, 3), (OP_MCZ, 0, 0, 0.0, 0), (OP_MCZ, 0, 0, 0.0, 0b10001)]:
        with pytest.raises(ValueError):
            oracle.run_ops(3, make_ops([rec]))


def test_philox_known_answers():
    # Philox4x32-10 known-answer vectors (Salmon et al., SC'11; Random123 distribution)
    assert oracle.philox([0, 0, 0, 0], [0, 0]).tolist() == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert oracle.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2).tolist() == [0x408F276D, 0x41C83B0E, 0xA20BC7C6,
                                                                           0x6D5451FD]
    assert oracle.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]).tolist() == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_uniform_rule_is_53_bit():
    u1, u2 = oracle.uniform_pair(7, 3, 11)
    for u in (u1, u2):
        assert 0.0 <= u < 1.0
        assert u * 2 ** 53 == int(u * 2 ** 53)


def test_trajectory_mean_matches_density_matrix():
    n = 4
    ops = workloads.noisy_layers(n, layers=2, seed=9)
    gamma, lam = 0.2, 0.1  # strong noise so jumps happen often in a short test
    z_exact = oracle.density_z0(n, ops, gamma, lam)
    z, jumps, _, _ = oracle.traj_run(n, ops, gamma, lam, seed=99, begin=0, end=6000)
    se = z.std(ddof=1) / np.sqrt(z.size)
    assert jumps.sum() > 0
    assert abs(z.mean() - z_exact) < 5 * se


def test_trajectory_is_reproducible_and_splittable():
    ops = workloads.noisy_layers(5, layers=2, seed=3)
    z_all, j_all, _, _ = oracle.traj_run(5, ops, 0.05, 0.02, seed=5, begin=0, end=64)
    z_b, j_b, _, _ = oracle.traj_run(5, ops, 0.05, 0.02, seed=5, begin=32, end=64)
    assert np.array_equal(z_all[32:], z_b) and np.array_equal(j_all[32:], j_b)
