"""Mixed-size circuit batches in one persistent launch, against the oracle per circuit; complex64
fidelity against complex128; the bounded dependency wait reporting LLG_ETIMEOUT."""
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


def random_batch(count, lo, hi, depth, seed):
    rng = np.random.default_rng(seed)
    nq, circuits = [], []
    for _ in range(count):
        n = int(rng.integers(lo, hi + 1))
        recs = []
        for _ in range(depth):
            k = rng.integers(9)
            q = int(rng.integers(n))
            if k == 0:
                recs.append((OP_H, q))
            elif k == 1:
                recs.append((OP_X, q))
            elif k < 5:
                recs.append(((OP_RX, OP_RY, OP_RZ)[k - 2], q, 0, float(rng.uniform(0, 2 * np.pi))))
            elif k < 7 and n > 1:
                a, b = rng.choice(n, 2, replace=False)
                recs.append(((OP_CNOT, OP_CZ)[k - 5], int(a), int(b)))
            elif k == 7:
                recs.append((OP_MCZ, 0, 0, 0.0, int(rng.integers(1, 1 << n))))
            else:
                u, _ = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))
                recs.append((OP_U2, q, 0, 0.0, None, u.reshape(4)))
        nq.append(n)
        circuits.append(make_ops(recs))
    offsets = np.concatenate([[0], np.cumsum([len(c) for c in circuits])])
    return np.array(nq), np.concatenate(circuits), offsets, circuits


@pytest.mark.parametrize("precision,tol", [("df64", 1e-12), ("fp64", 1e-12), ("complex64", 5e-5)])
@pytest.mark.parametrize("tile", [5, 0])
def test_batch_matches_oracle(precision, tol, tile):
    nq, ops, off, circuits = random_batch(30, 2, 14, 80, seed=31)
    b = llgpu.Batch(nq, ops, off, precision, tile)
    b.run()
    for i, (n, c) in enumerate(zip(nq, circuits)):
        assert np.max(np.abs(b.state(i) - oracle.run_ops(int(n), c))) <= tol, i
    b.run()  # runs again from |0..0>
    assert np.max(np.abs(b.state(3) - oracle.run_ops(int(nq[3]), circuits[3]))) <= tol
    b.close()


def test_fidelity_of_complex64_batch():
    nq, ops, off, _ = random_batch(20, 4, 15, 120, seed=5)
    b128 = llgpu.Batch(nq, ops, off, "df64")
    b64 = llgpu.Batch(nq, ops, off, "complex64")
    b128.run()
    b64.run()
    f = b64.fidelity(b128)
    for i in range(len(nq)):
        s1, s2 = b64.state(i), b128.state(i)
        want = abs(np.vdot(s1, s2)) ** 2 / (np.vdot(s1, s1).real * np.vdot(s2, s2).real)
        assert abs(f[i, 0] - want) <= 1e-12
    assert np.all(1 - f[:, 0] < 1e-8) and np.all(np.abs(f[:, 2] - 1) < 1e-12)


def test_bounded_wait_reports_timeout():
    # 2 circuits of 8 qubits with 5-qubit tiles: 8 tiles per pass, several passes
    nq, ops, off, _ = random_batch(2, 8, 8, 60, seed=2)
    b = llgpu.Batch(nq, ops, off, "df64", 5)
    assert b.info()["total_passes"] > 2
    b.run()
    # work items are ordered by pass round: item 16 is a pass-1 tile of circuit 0
    assert llgpu.lib().llg_batch_debug_block_item(b._h, 16) == llgpu.LLG_OK
    with pytest.raises(llgpu.LLGError, match="waited past its limit"):
        b.run(spin_limit=20000)
    b.close()
    b2 = llgpu.Batch(nq, ops, off, "df64", 5)  # the context is still usable
    b2.run()
    b2.close()


def test_full_config5_batch():
    """512 circuits, n uniform in 10..22, 200 gates each, in IEEE complex128, double-float and
    complex64: every circuit of up to 18 qubits against the oracle (the oracle runs them on every
    host core), the rest of the complex128 batch against the double-float one, and complex64 against
    complex128 per circuit."""
    import concurrent.futures as cf
    import multiprocessing as mp

    nq, ops, off = workloads.mixed_batch(512, 10, 22, 200)
    b128 = llgpu.Batch(nq, ops, off, "complex128")
    bdf = llgpu.Batch(nq, ops, off, "df64")
    b64 = llgpu.Batch(nq, ops, off, "complex64")
    for b in (b128, bdf, b64):
        b.run()
    f = b64.fidelity(b128)
    assert np.all(np.abs(f[:, 2] - 1) < 1e-11)
    assert np.all(1 - f[:, 0] < 1e-8)
    fd = bdf.fidelity(b128)
    assert np.all(1 - fd[:, 0] < 1e-13)
    small = [i for i in range(512) if nq[i] <= 18]
    assert len(small) > 250
    oracle.set_threads(1)
    # oracle runs in worker processes started with spawn (the GPU context stays in this process)
    with cf.ProcessPoolExecutor(max_workers=min(16, mp.cpu_count()), mp_context=mp.get_context("spawn")) as ex:
        wants = list(ex.map(_oracle_circuit, [(int(nq[i]), ops[off[i]:off[i + 1]]) for i in small], chunksize=8))
    for i, want in zip(small, wants):
        assert np.max(np.abs(b128.state(i) - want)) <= 1e-12, i
        assert np.max(np.abs(bdf.state(i) - want)) <= 1e-12, i
    oracle.set_threads(oracle.max_threads())
    for b in (b128, bdf, b64):
        b.close()


def _oracle_circuit(args):
    import oracle as orc

    orc.set_threads(1)
    n, o = args
    return orc.run_ops(n, o)
