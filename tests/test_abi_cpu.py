"""The C ABI boundary without a GPU: the library loads, exports every symbol include/*.h
declares, fails loudly (no CPU fallback) when no device exists, validates arguments with the
reference's error contract, and its fusion planner computes the same state as the oracle."""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np
import pytest

import llgpu
import oracle
import workloads
from conftest import REPO, split
from llgpu import OP_CNOT, OP_CZ, OP_DTYPE, OP_H, OP_MCZ, OP_RX, OP_RY, OP_RZ, OP_U2, OP_X, make_ops
from planexec import execute, unregister


def header_symbols():
    names = set()
    inc = os.path.join(REPO, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"^\s*(?:const\s+)?[\w\*]+[\s\*]+(llg_\w+)\s*\(", src, flags=re.M))
    return sorted(names)


def test_library_exports_every_declared_symbol(built):
    L = ctypes.CDLL(llgpu.LIB_PATH)
    names = header_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_no_gpu_means_loud_failure(built):
    if llgpu.device_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(llgpu.LLGError, match="cuda|CUDA|driver"):
        llgpu.State(4)
    import quantum_sim_v3

    with pytest.raises(RuntimeError):
        quantum_sim_v3.StateVector(4)


def test_plan_export_validates_like_the_reference(built):
    bad = [(OP_H, -1), (OP_X, 3), (OP_RX, 0, 0, float("nan")), (OP_RY, 0, 0, float("inf")), (OP_RZ, 5, 0, 0.1),
           (OP_CNOT, 1, 1), (OP_CNOT, 0, 3), (OP_MCZ, 0, 0, 0.0, 0), (OP_MCZ, 0, 0, 0.0, 0b10001), (OP_CZ, 2, 2)]
    for rec in bad:
        with pytest.raises(ValueError):
            llgpu.plan_export(3, make_ops([rec]), 3)


def random_ops(n, depth, rng):
    recs = []
    for _ in range(depth):
        k = rng.integers(10)
        q = int(rng.integers(n))
        if k == 0:
            recs.append((OP_H, q))
        elif k == 1:
            recs.append((OP_X, q))
        elif k in (2, 3, 4):
            recs.append(((OP_RX, OP_RY, OP_RZ)[k - 2], q, 0, float(rng.uniform(-3.2, 3.2))))
        elif k in (5, 6):
            a, b = rng.choice(n, 2, replace=False)
            recs.append(((OP_CNOT, OP_CZ)[k - 5], int(a), int(b)))
        elif k == 7:
            mask = int(rng.integers(1, 1 << n))
            recs.append((OP_MCZ, 0, 0, 0.0, mask))
        else:
            u, _ = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))
            recs.append((OP_U2, q, 0, 0.0, None, u.reshape(4)))
    return make_ops(recs)


@pytest.mark.parametrize("zyz", [False, True])
@pytest.mark.parametrize("n,tile", [(6, 5), (8, 5), (9, 6), (10, 7), (11, 5)])
def test_planned_passes_reproduce_the_oracle(built, n, tile, zyz):
    rng = np.random.default_rng(100 + n)
    ops = random_ops(n, 300, rng)
    passes, xops = llgpu.plan_export(n, ops, tile, zyz=zyz)
    if n > tile:
        assert len(passes) > 1
    got = execute(oracle.zero_state(n), n, passes, xops)
    want = oracle.run_ops(n, ops)
    assert np.max(np.abs(got - want)) < 1e-12


@pytest.mark.parametrize("zyz", [False, True])
def test_plan_of_layered_circuit(built, golden, zyz):
    g = golden("config2_layered")
    for n, ops in zip(g["n"], split(g["ops"], g["offsets"])):
        n = int(n)
        passes, xops = llgpu.plan_export(n, ops, 5, zyz=zyz)
        got = execute(oracle.zero_state(n), n, passes, xops)
        assert np.max(np.abs(got - oracle.run_ops(n, ops))) < 1e-12
        # fewer passes than gates: runs of rotations share a pass
        assert len(passes) < len(ops) / 4


def test_plan_of_random_2024_circuits(built, golden):
    g = golden("random_2024")
    for n, ops in zip(g["n"], split(g["ops"], g["offsets"])):
        n = int(n)
        passes, xops = llgpu.plan_export(n, ops, 3)
        got = execute(oracle.zero_state(n), n, passes, xops)
        assert np.max(np.abs(got - oracle.run_ops(n, ops))) < 1e-12


@pytest.mark.parametrize("n,tile", [(6, 5), (9, 6), (12, 9), (14, 13)])
def test_two_qubit_blocks_reproduce_the_oracle(built, n, tile):
    # complex64 tile passes merge each local CNOT with its neighbouring one-qubit ops into a 4x4
    # block (kind 20): the plan's product is unchanged
    rng = np.random.default_rng(500 + n)
    for ops in (random_ops(n, 300, rng), workloads.layered_rotations(n, 6, seed=n)):
        passes, xops, tab = llgpu.plan_export(n, ops, tile, fuse2=True)
        p0, x0 = llgpu.plan_export(n, ops, tile)
        blocks, cblocks = int(np.sum(xops["kind"] == 20)), int(np.sum(xops["kind"] == 21))
        assert blocks > 0 and len(xops) < len(x0)
        assert tab.size == 16 * blocks + 8 * cblocks
        got = execute(oracle.zero_state(n), n, passes, xops, tab)
        assert np.max(np.abs(got - oracle.run_ops(n, ops))) < 1e-12
    with pytest.raises(ValueError):
        llgpu.plan_export(n, ops, tile, fuse2=True, zyz=True)


def test_two_qubit_blocks_on_the_layered_circuit(built):
    # 30 qubits, 13-qubit tiles: most one-qubit ops move into the blocks of the brickwork's CNOTs
    ops = workloads.layered_rotations(30, 20)
    p0, x0 = llgpu.plan_export(30, ops, 13)
    passes, xops, tab = llgpu.plan_export(30, ops, 13, fuse2=True)
    assert len(passes) == len(p0)
    assert len(xops) < 0.6 * len(x0)


@pytest.mark.parametrize("tile", [9, 11, 13])
def test_register_programs_reproduce_the_oracle(built, tile):
    n = 16
    ops = workloads.layered_rotations(n, 6, seed=3)
    passes, xops = llgpu.plan_export(n, ops, tile, zyz=True, regs=True)
    assert int(np.sum(xops["kind"] == 19)) > 0
    got = execute(oracle.zero_state(n), n, passes, unregister(passes, xops))
    assert np.max(np.abs(got - oracle.run_ops(n, ops))) < 1e-12


def test_zyz_plan_carries_the_global_phase_in_one_u2(built):
    # fused rotations become ZYZ ops; exactly one generic 2x2 remains and carries the phases
    n = 12
    ops = workloads.layered_rotations(n, layers=6)
    passes, xops = llgpu.plan_export(n, ops, 8, zyz=True)
    kinds = np.bincount(xops["kind"], minlength=16)
    # rotations as RY diag(1, g) over their dropped cos / sin factor (kinds 14, 15), output phases
    # carried; one full RY (kind 12) absorbs the flush's dropped factors
    assert kinds[0] == 1 and kinds[14] + kinds[15] > 50 and kinds[12] == 1
    assert kinds[5] == 0  # every RZ folded into carried phases
    phased = (xops["kind"] == 6) & ((xops["flags"] & 8) != 0)
    assert phased.sum() > 10  # carried target phases pushed through CNOTs
    assert 0 < kinds[13] <= n  # the phases still carried at the end, one op per qubit at most
    got = execute(oracle.zero_state(n), n, passes, xops)
    assert np.max(np.abs(got - oracle.run_ops(n, ops))) < 1e-12


def test_zyz_keeps_non_unitary_gates_generic(built):
    rng = np.random.default_rng(7)
    recs = []
    for k in range(40):
        g = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
        if k % 2:
            g, _ = np.linalg.qr(g)  # unitary
        recs.append((OP_U2, int(rng.integers(6)), 0, 0.0, None, g.reshape(4)))
        recs.append((OP_CNOT, k % 6, (k + 1) % 6, 0.0))
    ops = make_ops(recs)
    passes, xops = llgpu.plan_export(6, ops, 5, zyz=True)
    kinds = np.bincount(xops["kind"], minlength=16)
    assert kinds[0] >= 10 and kinds[12] + kinds[14] + kinds[15] >= 5  # non-unitary products stay generic
    got = execute(oracle.zero_state(6), 6, passes, xops)
    want = oracle.run_ops(6, ops)
    assert np.max(np.abs(got - want)) <= 1e-12 * max(1.0, np.max(np.abs(want)))


def _flush_scales(passes, xops):
    """The smallest running product of the factors dropped by kind 14/15 ops since the last full
    rotation (kind 12), over the whole flush (the product carries across passes), and the product
    left at the end of the flush."""
    sig, low = 1.0, 1.0
    for p in passes:
        for x in xops[p["op_begin"]:p["op_begin"] + p["nops"]]:
            k = int(x["kind"])
            if k in (14, 15):
                sig /= np.sqrt(1.0 + x["c"][2] ** 2)
                low = min(low, sig)
            elif k == 12:
                sig = 1.0
    return low, sig


@pytest.mark.parametrize("df64,floor", [(False, 2.0 ** -300), (True, 2.0 ** -40)])
def test_tangent_rotations_renormalise_per_flush(built, df64, floor):
    # 600 rotations on 8 qubits: the dropped factors (|f| >= 1/sqrt 2 each) shrink the running
    # scale; full rotations absorb it before the precision's floor (2^-40 for double-float, 2^-300
    # for IEEE double) and once at the end of the flush, whatever the pass boundaries
    n = 8
    ops = workloads.layered_rotations(n, layers=75)
    for tile in (8, 5):
        passes, xops = llgpu.plan_export(n, ops, tile, zyz=True, df64=df64)
        if tile == 8:
            assert len(passes) == 1
        kinds = np.bincount(xops["kind"], minlength=16)
        ntan = kinds[14] + kinds[15]
        # one full rotation at the end, plus one per ~60 or more tangent rotations for double-float
        assert 0 < kinds[12] <= 1 + (ntan // 60 if df64 else 0)
        low, end = _flush_scales(passes, xops)
        assert low >= floor / np.sqrt(2.0) and end == 1.0
        got = execute(oracle.zero_state(n), n, passes, xops)
        assert np.max(np.abs(got - oracle.run_ops(n, ops))) < 1e-12
    if df64:
        return
    # angles near 0 and pi/2 (tangent and cotangent forms, |coefficient| <= 1), and exactly pi
    rng = np.random.default_rng(5)
    recs = []
    for k in range(200):
        q = int(rng.integers(4))
        ang = [0.0, np.pi, -np.pi, np.pi / 2, 1e-9, np.pi - 1e-9, float(rng.uniform(-7, 7))][k % 7]
        recs += [(OP_RY, q, 0, ang), (OP_RZ, q, 0, float(rng.uniform(-3, 3))), (OP_CNOT, q, (q + 1) % 4)]
    ops = make_ops(recs)
    passes, xops = llgpu.plan_export(4, ops, 4, zyz=True)
    t = xops["c"][:, 2][np.isin(xops["kind"], (14, 15))]
    assert t.size and np.all(np.abs(t) <= 1.0)
    got = execute(oracle.zero_state(4), 4, passes, xops)
    assert np.max(np.abs(got - oracle.run_ops(4, ops))) < 1e-12


def test_carried_phases_through_every_gate_kind(built):
    # RZ and X on qubits carrying phases, CNOTs with carried phases on control and target,
    # H / RX / RY after a carried phase, CZ / MCZ in between, non-local qubits: the plan with
    # carried phases reproduces the oracle
    rng = np.random.default_rng(23)
    n = 9
    recs = []
    for _ in range(300):
        k = rng.integers(9)
        q = int(rng.integers(n))
        a, b = (int(x) for x in rng.choice(n, 2, replace=False))
        ang = float(rng.uniform(-3, 3))
        recs.append([(OP_RZ, q, 0, ang), (OP_X, q), (OP_H, q), (OP_RX, q, 0, ang), (OP_RY, q, 0, ang),
                     (OP_CNOT, a, b), (OP_CZ, a, b), (OP_MCZ, 0, 0, 0.0, int(rng.integers(1, 1 << n))),
                     (OP_U2, q, 0, 0.0, None, np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))[0].reshape(4))][k])
    ops = make_ops(recs)
    for tile in (4, 6, 9):
        passes, xops = llgpu.plan_export(n, ops, tile, zyz=True)
        got = execute(oracle.zero_state(n), n, passes, xops)
        assert np.max(np.abs(got - oracle.run_ops(n, ops))) < 1e-12, tile


def test_thirty_qubit_plan_is_compact(built):
    ops = workloads.layered_rotations(30, layers=20)
    passes, xops = llgpu.plan_export(30, ops, 12)
    # every pass holds the 4 low qubits plus at most 8 more
    assert all(bin(int(p["local_mask"])).count("1") == 12 for p in passes)
    assert all(int(p["local_mask"]) & 0xF == 0xF for p in passes)
    assert len(passes) < 60


def _plan_exec(n, ops, tile, tables):
    r = llgpu.plan_export(n, ops, tile, zyz=True, tables=tables)
    return r, execute(oracle.zero_state(n), n, r[0], r[1], r[2] if tables else None)


@pytest.mark.parametrize("n,tile", [(6, 5), (9, 6), (10, 7), (11, 5)])
def test_phase_table_plans_reproduce_the_oracle(built, n, tile):
    # random circuits over every gate kind (non-unitary 2x2s, MCZ masks, CNOTs with non-local
    # controls): gathering diagonal factors into phase tables keeps the plan's product
    rng = np.random.default_rng(300 + n)
    ops = random_ops(n, 300, rng)
    (passes, xops, tab), got = _plan_exec(n, ops, tile, True)
    want = oracle.run_ops(n, ops)
    assert np.max(np.abs(got - want)) <= 1e-12 * max(1.0, np.max(np.abs(want)))
    # every table op points at a whole table of 2^t unit-modulus entries
    for p in passes:
        for x in xops[p["op_begin"]:p["op_begin"] + p["nops"]]:
            if int(x["kind"]) == 18:
                ent = tab[int(x["mask"]):int(x["mask"]) + (1 << int(p["t"]))]
                assert ent.size == 1 << int(p["t"]) and np.allclose(np.abs(ent), 1.0, atol=1e-14)


def test_phase_tables_on_the_layered_circuit(built, golden):
    g = golden("config2_layered")
    for n, ops in zip(g["n"], split(g["ops"], g["offsets"])):
        n = int(n)
        for tile in (5, 8):
            (passes, xops, tab), got = _plan_exec(n, ops, tile, True)
            assert np.max(np.abs(got - oracle.run_ops(n, ops))) < 1e-12


def _fp64_mults_per_pair(xops):
    # FP64 multiply-adds per amplitude pair of each executor kind (phased CNOT: a quarter of the
    # amplitudes times a complex constant)
    cost = {0: 16, 1: 8, 2: 8, 3: 8, 5: 8, 11: 16, 12: 12, 13: 4, 14: 8, 15: 8, 16: 4, 17: 4, 18: 8}
    c = sum(cost.get(int(k), 0) for k in xops["kind"])
    return c + 2 * int(np.sum((xops["kind"] == 6) & ((xops["flags"] & 8) != 0)))


def test_phase_tables_halve_the_rotation_arithmetic(built):
    # the 30-qubit headline recipe with 12-qubit tiles: rotations lose their complex input-phase
    # product (8 -> 4 multiply-adds per pair) and phased CNOTs their controlled phase; the tables
    # that take them over cost less than what they replace
    n = 30
    ops = workloads.layered_rotations(n, layers=20)
    plain = llgpu.plan_export(n, ops, 12, zyz=True)
    passes, xops, tab = llgpu.plan_export(n, ops, 12, zyz=True, tables=True)
    assert len(passes) == len(plain[0])
    kinds = np.bincount(xops["kind"], minlength=19)
    assert kinds[16] + kinds[17] > 500 and kinds[18] > 0
    assert _fp64_mults_per_pair(xops) < 0.7 * _fp64_mults_per_pair(plain[1])
    assert tab.size == kinds[18] << 12


def _ising_diagonal(n, zz, z):
    # the reference's ising_diagonal (python/algorithms.py:139-152), restated in numpy
    idx = np.arange(1 << n, dtype=np.int64)
    s = [1.0 - 2.0 * ((idx >> q) & 1) for q in range(n)]
    d = np.zeros(idx.size)
    for i, j, c in zz:
        d += c * s[i] * s[j]
    for i, h in z:
        d += h * s[i]
    return d


@pytest.mark.parametrize("n", [1, 5, 12, 13, 17])
def test_general_observable_decomposition(built, n):
    # any number of Z / ZZ terms with any coefficients (all-to-all couplings, fields, repeated
    # pairs): the chunked decomposition the GPU kernel uses gives ising_diagonal's values
    rng = np.random.default_rng(40 + n)
    zz = [(i, j, float(rng.normal())) for i in range(n) for j in range(i + 1, n)]
    zz += [(j, i, 0.5) for i, j, _ in zz[:3]]  # the same pair twice, in either order
    z = [(i, float(rng.normal())) for i in range(n)]
    a, b, c = llgpu.ising_terms(n, zz, z)
    got = llgpu.diag_export(n, a, b, c)
    want = _ising_diagonal(n, zz, z)
    assert np.max(np.abs(got - want)) <= 1e-12 * max(1.0, np.max(np.abs(want)))


def test_general_observable_rejects_bad_terms(built):
    for a, b, c in (([0], [0], [1.0]), ([3], [-1], [1.0]), ([0], [1], [float("nan")]), ([-1], [0], [1.0])):
        with pytest.raises(ValueError):
            llgpu.diag_export(3, a, b, c)


def test_algorithms_module_without_a_gpu(built):
    import quantum_sim_algorithms as alg

    g = alg.Graph(4, [(0, 1, 1.0), (1, 2, 2.0)])
    g.add_edge(2, 3, 0.5)
    assert alg.QAOA.cut_value(g, 0b0101) == 3.5 and len(g.edges) == 3
    if llgpu.device_count() == 0:
        with pytest.raises(RuntimeError):
            alg.make_gpu_backend(3)  # no CPU fallback


def test_stream_lowering_reproduces_the_oracle(built):
    # IEEE complex128 per-gate flushes: scale-free RX / RY / H, RZ as diag(1, e^it) on the |1> half,
    # the carried factor and phase absorbed once (into a generic 2x2 when there is one)
    rng = np.random.default_rng(77)
    for n, with_u2 in ((6, True), (7, False), (9, False), (10, True)):
        ops = random_ops(n, 300, rng)
        if not with_u2:
            ops = ops[ops["kind"] != OP_U2]
        passes, xops = llgpu.plan_export(n, ops, n, stream=True)
        assert len(passes) == 1 and len(xops) >= len(ops)
        kinds = np.bincount(xops["kind"], minlength=27)
        assert kinds[22] + kinds[23] + kinds[16] + kinds[17] + kinds[24] > 0 and kinds[13] > 0
        # unitary 2x2s as phase-rotation-phase without their factor (kinds 25 / 26)
        assert (kinds[25] + kinds[26] > 0) == with_u2
        # full forms: at most one real op (or the unitary form it absorbs into) and one
        # whole-state diagonal take the carried factor and phase
        full = int(kinds[0] + kinds[1] + kinds[2] + kinds[3] + kinds[5] + kinds[11])
        assert full <= 2
        got = execute(oracle.zero_state(n), n, passes, xops)
        assert np.max(np.abs(got - oracle.run_ops(n, ops))) < 1e-12
    # a flush of unitary 2x2s alone: four scale-free forms, the last one the generic 2x2 that
    # takes the carried factor and phase; a non-unitary 2x2 takes them for free
    for recs in ([(OP_U2, q, 0, 0.0, None, np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))[0].reshape(4))
                  for q in (0, 1, 2, 3, 4)],
                 [(OP_U2, 2, 0, 0.0, None, np.array([1.0, 0.5, 0.25j, 2.0]))] +
                 [(OP_RY, q, 0, 0.3 + q) for q in range(5)] + [(OP_RZ, 1, 0, 0.7)]):
        ops = make_ops(recs)
        passes, xops = llgpu.plan_export(5, ops, 5, stream=True)
        kinds = np.bincount(xops["kind"], minlength=27)
        got = execute(oracle.zero_state(5), 5, passes, xops)
        assert np.max(np.abs(got - oracle.run_ops(5, ops))) < 1e-12
        assert kinds[0] == 1 and kinds[1] + kinds[2] + kinds[3] + kinds[5] + kinds[11] == 0


def test_stream_lowering_phase_on_qubit_0_takes_the_global_phase(built):
    # five RZs: the one on qubit 0 (whose half-state pass moves every sector anyway) becomes the
    # whole-state diagonal, the others stay half-state phases
    n = 8
    rng = np.random.default_rng(5)
    psi0 = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi0 /= np.linalg.norm(psi0)
    for targets in ((0, 3, 5, 6, 7), (4, 0, 7), (3, 5, 7)):
        ops = make_ops([(OP_RZ, q, 0, 0.3 + 0.4 * q) for q in targets])
        passes, xops = llgpu.plan_export(n, ops, n, stream=True)
        kinds = xops["kind"].tolist()
        diag = [int(xops["q0"][i]) for i, k in enumerate(kinds) if k == 5]  # EX_DIAG
        assert kinds.count(13) == len(targets) - 1 and diag == [0 if 0 in targets else targets[-1]]
        got = execute(psi0, n, passes, xops)
        assert np.max(np.abs(got - oracle.run_ops(n, ops, psi0.copy()))) < 1e-12


def test_stream_lowering_absorbs_before_the_floor(built):
    # 700 rotations at |cos| = |sin| = 2^-1/2 shrink the carried factor to 2^-350: it is absorbed
    # before 2^-300 and once at the end
    n = 3
    recs = [((OP_RX, OP_RY)[k % 2], k % n, 0, np.pi / 2 + (1e-3 if k % 3 else -1e-3)) for k in range(700)]
    ops = make_ops(recs)
    passes, xops = llgpu.plan_export(n, ops, n, stream=True)
    kinds = np.bincount(xops["kind"], minlength=25)
    assert kinds[1] + kinds[2] == 2  # one mid-flush absorption, one at the end
    got = execute(oracle.zero_state(n), n, passes, xops)
    assert np.max(np.abs(got - oracle.run_ops(n, ops))) < 1e-12
    with pytest.raises(ValueError):
        llgpu.plan_export(n, ops, n, stream=True, zyz=True)
