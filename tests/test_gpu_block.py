"""Dense k-qubit blocks (llg_apply_matrix, k <= 5) against the oracle's restatement
(orc_apply_matrix), interleaved with queued gates, through the C ABI and the drop-in module."""
from __future__ import annotations

import numpy as np
import pytest

import llgpu
import oracle
import workloads

pytestmark = pytest.mark.gpu
TOL = {"df64": 1e-12, "fp64": 1e-12, "complex64": 5e-5}


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    assert llgpu.device_count() > 0


def rand_unitary(d, rng):
    q, r = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("precision", ["df64", "fp64", "complex64"])
@pytest.mark.parametrize("n,k", [(4, 1), (6, 2), (8, 3), (11, 4), (13, 5), (5, 5), (3, 2), (16, 5)])
def test_block_matches_oracle(precision, n, k):
    ops = workloads.layered_rotations(n, 2, seed=n)
    st2 = llgpu.State(n, precision)
    st2.apply_ops(ops)
    want = oracle.run_ops(n, ops)
    rng = np.random.default_rng(1000 * n + k)
    for rep in range(3):
        qs = [int(x) for x in rng.choice(n, size=k, replace=False)]
        m = rand_unitary(1 << k, rng)
        q = int(rng.integers(n))
        st2.apply_matrix(qs, m)
        st2.rx(q, 0.3)
        oracle.apply_matrix(want, n, qs, m)
        want = oracle.run_ops(n, llgpu.make_ops([(llgpu.OP_RX, q, 0, 0.3)]), want)
    assert np.max(np.abs(st2.state() - want)) <= TOL[precision]
    st2.close()


@pytest.mark.parametrize("precision", ["df64", "fp64", "complex64"])
@pytest.mark.parametrize("n,k", [(5, 1), (9, 2), (10, 3), (13, 4)])
def test_sparse_block_matches_oracle(precision, n, k):
    # blocks with at most a quarter of their cost in nonzero entries run the sparse kernel: real and
    # complex entries, an empty row, a full row
    ops = workloads.layered_rotations(n, 2, seed=n)
    st = llgpu.State(n, precision)
    st.apply_ops(ops)
    want = oracle.run_ops(n, ops)
    rng = np.random.default_rng(50 * n + k)
    d = 1 << k
    for rep in range(3):
        m = np.zeros((d, d), dtype=complex)
        for r in range(d):
            for c in rng.choice(d, size=min(d, 1 + (r % 2)), replace=False):
                m[r, c] = rng.normal() + (1j * rng.normal() if (r + c) % 3 == 0 else 0.0)
        m[d - 1, :] = 0.0
        if k == 1:
            m[0, :] = [0.6, 0.0]
        qs = [int(x) for x in rng.choice(n, size=k, replace=False)]
        st.apply_matrix(qs, m)
        oracle.apply_matrix(want, n, qs, m)
    scale = max(1.0, float(np.max(np.abs(want))))
    assert np.max(np.abs(st.state() - want)) <= TOL[precision] * scale
    st.close()


def test_non_unitary_block_and_high_qubits():
    rng = np.random.default_rng(3)
    n = 20
    st = llgpu.State(n)
    psi = (rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)) / 1000.0
    st.load(psi)
    want = psi.copy()
    for qs in ([19, 18, 17], [0, 19], [5, 1, 12, 19, 0]):
        m = rng.normal(size=(1 << len(qs),) * 2) + 1j * rng.normal(size=(1 << len(qs),) * 2)
        st.apply_matrix(qs, m)
        oracle.apply_matrix(want, n, qs, m)
    got = st.state()
    assert np.max(np.abs(got - want)) <= 1e-12 * max(1.0, np.max(np.abs(want)))
    st.close()


@pytest.mark.parametrize("precision", ["df64", "fp64"])
@pytest.mark.parametrize("n,k", [(12, 5), (14, 5), (11, 4), (13, 4), (10, 3), (12, 3), (10, 2), (13, 2)])
def test_tensor_core_block_edge_values(precision, n, k):
    # 4- and 5-qubit blocks on double-float states, and 3- to 5-qubit blocks on IEEE complex128
    # states, of k + 7 or more qubits run on the tensor cores (exact 8-bit slices against a scale
    # per group of 2^k amplitudes: six for double-float, eight for FP64); an IEEE complex128 2-qubit
    # block runs there as a 3-qubit one with the identity on another qubit: zero groups, tiny
    # groups, 20 orders of magnitude inside one group, a non-unitary matrix with large entries and
    # a zero row
    rng = np.random.default_rng(40 + n + k)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    qs = [0, 3, n - 5, n - 2, n - 1][5 - k:]
    d = 1 << k
    tmask = sum(1 << q for q in qs)
    free = [i for i in range(1 << n) if i & tmask == 0]
    offs = [sum(((j >> b) & 1) << q for b, q in enumerate(qs)) for j in range(d)]
    psi[[free[0] | o for o in offs]] = 0.0                       # an all-zero group
    psi[[free[1] | o for o in offs]] *= 1e-25                    # a tiny group
    psi[[free[2] | o for o in offs[1:]]] *= 1e-20                # one large amplitude, the rest tiny
    psi[free[3] | offs[min(5, d - 1)]] = 3.0 - 4.0j
    st = llgpu.State(n, precision)
    st.load(psi)
    want = psi.copy()
    m = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) * 4.0
    m[min(7, d - 1), :] = 0.0
    m[:, min(9, d - 2)] *= 1e-12
    st.apply_matrix(qs, m)
    oracle.apply_matrix(want, n, qs, m)
    u = rand_unitary(d, rng)
    st.apply_matrix(qs[::-1], u)
    oracle.apply_matrix(want, n, qs[::-1], u)
    got = st.state()
    # error bound per group: ~2^-46 of the group's largest amplitude times the matrix norm
    scale = np.max(np.abs(want))
    assert np.max(np.abs(got - want)) <= 1e-12 * scale
    assert np.all(got[[free[0] | o for o in offs]] == 0)
    tiny = np.array([free[1] | o for o in offs])
    assert np.max(np.abs(got[tiny] - want[tiny])) <= 1e-12 * np.max(np.abs(want[tiny]))
    st.close()


@pytest.mark.parametrize("precision", ["df64", "fp64"])
@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_blocks_after_cancellation(precision, k):
    """Pairs along qubit 0 equal to 1e-9: after H the differences are stored as unnormalised
    double-float pairs whose low part outweighs the high part (double-float), or as doubles 1e-9
    below their neighbours (FP64).  Every block kernel (a thread per group for k <= 3, the tensor
    cores for k = 4, 5 on 12 qubits) must read them at full value."""
    n = 12
    rng = np.random.default_rng(700 + k)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    even = np.arange(0, 1 << n, 2)
    psi[even + 1] = psi[even] * (1.0 + 1e-9 * rng.normal(size=even.size))
    st = llgpu.State(n, precision)
    st.load(psi)
    st.set_fusion("tile", 10)
    ops = llgpu.make_ops([(llgpu.OP_H, 0)])
    st.apply_ops(ops)
    want = oracle.run_ops(n, ops, psi)
    qs = [0, 3, 6, 9, 11][:k]
    m = rand_unitary(1 << k, rng)
    st.apply_matrix(qs, m)
    oracle.apply_matrix(want, n, qs, m)
    got = st.state()
    assert np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want))
    st.close()


def test_block_contract():
    st = llgpu.State(4)
    eye = np.eye(4)
    with pytest.raises(ValueError):
        st.apply_matrix([0, 0], eye)  # repeated qubit
    with pytest.raises(ValueError):
        st.apply_matrix([0, 4], eye)  # outside the register
    with pytest.raises(ValueError):
        st.apply_matrix([0, 1], np.full((4, 4), np.nan))
    with pytest.raises(ValueError):
        st.apply_matrix([0, 1, 2, 3, 0, 1], np.eye(64))  # k > 5
    st.close()


def test_drop_in_module_apply_matrix():
    import quantum_sim_v3

    rng = np.random.default_rng(8)
    sv = quantum_sim_v3.StateVector(7)
    m = rand_unitary(8, rng)
    sv.h(0)
    sv.apply_matrix([2, 0, 5], m)
    want = oracle.zero_state(7)
    want = oracle.run_ops(7, llgpu.make_ops([(llgpu.OP_H, 0)]), want)
    oracle.apply_matrix(want, 7, [2, 0, 5], m)
    assert np.max(np.abs(sv.get_numpy_view() - want)) <= 1e-12
