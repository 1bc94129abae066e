"""GPU parity: the CUDA engine against the oracle and the reference's own outputs (golden
fixtures), through the C ABI (llgpu) and the drop-in pybind11 modules.

Tolerances: complex128 (double-float) and fp64 states <= 1e-12 max |amplitude difference|, the
spec bar; complex64 states <= 5e-5 (fp32 rounding over a few hundred gates)."""
from __future__ import annotations

import numpy as np
import pytest

import llgpu
import oracle
import workloads
from conftest import split, split_states
from llgpu import OP_CNOT, OP_CZ, OP_H, OP_MCZ, OP_RX, OP_RY, OP_RZ, OP_U2, OP_X, make_ops

pytestmark = pytest.mark.gpu

TOL = {"df64": 1e-12, "fp64": 1e-12, "complex64": 5e-5}
PRECISIONS = ["df64", "fp64", "complex64"]


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    assert llgpu.device_count() > 0, "no CUDA device visible"


def run_gpu(n, ops, precision="df64", fusion="tile", tile=0, init=None):
    st = llgpu.State(n, precision) if init is None else llgpu.State(precision=precision, amps=init)
    st.set_fusion(fusion, tile)
    st.apply_ops(ops)
    out = st.state()
    st.close()
    return out


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("fusion", ["tile", "none"])
def test_random_2024_circuits(golden, precision, fusion):
    g = golden("random_2024")
    worst = 0.0
    for n, ops, ref in zip(g["n"], split(g["ops"], g["offsets"]), split_states(g["ref_states"], g["state_offsets"])):
        got = run_gpu(int(n), ops, precision, fusion)
        worst = max(worst, float(np.max(np.abs(got - ref))))
    assert worst <= TOL[precision], worst


@pytest.mark.parametrize("tile", [5, 8, 12])
def test_config2_layered_fixture(golden, tile):
    g = golden("config2_layered")
    for n, ops, ref in zip(g["n"], split(g["ops"], g["offsets"]), split_states(g["states"], g["state_offsets"])):
        got = run_gpu(int(n), ops, "df64", "tile", tile)
        assert np.max(np.abs(got - ref)) <= 1e-12


def test_config1_through_drop_in(golden):
    import quantum_sim_v3

    g = golden("config1_h_cnot")
    for n, ops, ref in zip(g["n"], split(g["ops"], g["offsets"]), split_states(g["states"], g["state_offsets"])):
        sv = quantum_sim_v3.StateVector(int(n))
        for op in ops:
            if op["kind"] == OP_H:
                sv.h(int(op["q0"]))
            else:
                sv.cnot(int(op["q0"]), int(op["q1"]))
        got = np.array(sv.get_numpy_view(), copy=True)
        assert np.max(np.abs(got - ref)) <= 1e-12


def test_v3_and_v2_gate_semantics(golden):
    import quantum_sim_v2
    import quantum_sim_v3

    g = golden("v3_gates")
    n = int(g["n"])
    for label, mod, meth in (("v3_cache", quantum_sim_v3, "apply_gate_cache_optimized"),
                             ("v3_standard", quantum_sim_v3, "apply_gate_standard"),
                             ("v2", quantum_sim_v2, "apply_gate")):
        buf = g["init"].copy()
        sv = mod.StateVector(buf)
        for t, gate in zip(g["targets"], g["gates"]):
            if t >= n and label != "v3_cache":
                continue  # the reference's mask-scan variants corrupt memory there
            getattr(sv, meth)(int(t), [complex(x) for x in gate])  # list of 4, as the reference takes
        view = sv.get_numpy_view()
        assert view.base is sv
        # the fixture's gates are random non-unitary matrices (amplitudes grow to ~1e6), so the
        # 1e-12 bar is applied relative to the state's scale
        scale = max(1.0, float(np.max(np.abs(g[label]))))
        assert np.max(np.abs(view - g[label])) <= 1e-12 * scale
        assert np.max(np.abs(buf - g[label])) <= 1e-12 * scale  # caller's array updated at the sync point
    # |0..0> constructor
    sv = quantum_sim_v3.StateVector(5)
    h = 1 / np.sqrt(2)
    sv.apply_gate_cache_optimized(0, [h, h, h, -h])
    sv.apply_gate_cache_optimized(4, np.array([0, 1, 1, 0], dtype=complex))  # numpy gates accepted too
    assert np.max(np.abs(sv.get_numpy_view() - g["ctor5_view"])) <= 1e-15
    assert sv.get_num_qubits() == 5 and sv.get_size() == 32


def test_drop_in_error_contract():
    import quantum_sim_v3

    sv = quantum_sim_v3.StateVector(3)
    for call in (lambda: sv.h(-1), lambda: sv.x(3), lambda: sv.rx(0, float("nan")), lambda: sv.ry(0, float("inf")),
                 lambda: sv.rz(5, 0.1), lambda: sv.cnot(1, 1), lambda: sv.cnot(0, 3), lambda: sv.mcz([]),
                 lambda: sv.mcz([0, 0]), lambda: sv.mcz([0, 4]), lambda: sv.cz(1, 1),
                 lambda: sv.apply_gate_cache_optimized(-1, [1, 0, 0, 1])):
        with pytest.raises(ValueError):
            call()
    assert sv.get_num_qubits() == 3
    sv.apply_gate_cache_optimized(7, [0, 1, 1, 0])  # target >= n: a no-op, as in the reference
    v = sv.get_numpy_view()
    assert v[0] == 1 and np.all(v[1:] == 0)
    with pytest.raises(RuntimeError, match="power of 2"):
        quantum_sim_v3.StateVector(np.zeros(6, dtype=np.complex128))
    with pytest.raises(TypeError):
        quantum_sim_v3.StateVector(np.zeros(8, dtype=np.float64))


def test_closed_forms_on_gpu():
    import quantum_sim_v3 as q

    r = 1 / np.sqrt(2)
    for precision in PRECISIONS:
        tol = 1e-14 if precision != "complex64" else 1e-6
        sv = q.StateVector(4, precision)
        sv.x(2)
        assert sv.probabilities()[4] > 1 - tol
        sv = q.StateVector(2, precision)
        sv.h(0)
        sv.cnot(0, 1)
        p = sv.probabilities()
        assert abs(p[0] - 0.5) < tol and abs(p[3] - 0.5) < tol
        sv = q.StateVector(3, precision)
        sv.x(2)
        sv.cnot(2, 0)
        assert sv.probabilities()[5] > 1 - tol
        sv = q.StateVector(1, precision)
        sv.rx(0, np.pi)
        assert abs(sv.get_numpy_view()[1] - (-1j)) < tol
        sv = q.StateVector(1, precision)
        sv.h(0)
        sv.rz(0, 0.7)
        s = sv.get_numpy_view()
        assert abs(s[0] - r * np.exp(-0.35j)) < tol and abs(s[1] - r * np.exp(0.35j)) < tol
        sv = q.StateVector(3, precision)
        for k in range(3):
            sv.h(k)
        sv.mcz([0, 1, 2])
        m = sv.get_numpy_view()
        assert abs(m[7] + r ** 3) < tol and np.all(np.abs(m[:7] - r ** 3) < tol)


def test_grover_on_gpu(golden):
    import quantum_sim_v3

    from test_oracle_golden import grover_ops

    g = golden("grover")
    for key, n in (("n8_m85", 8), ("n10_i10", 10), ("n12_i10", 12)):
        sv = quantum_sim_v3.StateVector(n)
        sv.apply_ops(grover_ops(n, g[key + "_marked"].tolist(), int(g[key + "_iterations"])))
        assert np.max(np.abs(sv.probabilities() - g[key + "_probs"])) <= 1e-12
    assert abs(quantum_sim_v3.StateVector(8).probabilities()[0] - 1.0) == 0.0


@pytest.mark.parametrize("precision", PRECISIONS)
def test_readouts_match_oracle(precision):
    rng = np.random.default_rng(3)
    for n in (7, 12, 16):
        psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        psi /= np.linalg.norm(psi)
        st = llgpu.State(precision=precision, amps=psi)
        tol = 1e-12 if precision != "complex64" else 1e-6
        assert np.max(np.abs(st.probabilities() - oracle.probabilities(psi, n))) <= tol
        assert abs(st.norm2() - 1.0) <= tol
        a, b, c = llgpu.ring_zz_terms(n)
        a = a + [0, 3]
        b = b + [-1, -1]
        c = c + [0.5, -0.25]
        assert abs(st.expect_zz(a, b, c) - oracle.expect_zz(psi, n, a, b, c)) <= 20 * tol
        st.close()


@pytest.mark.parametrize("precision", PRECISIONS)
def test_pinned_and_pageable_readback_agree(precision):
    """A pinned destination is written by the conversion kernel directly; pageable memory goes
    through 256 MiB staging chunks (two chunks at 25 qubits).  Both give the same bits."""
    import ctypes

    rng = np.random.default_rng(12)
    for n in (5, 14, 25):
        psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        psi /= np.linalg.norm(psi)
        st = llgpu.State(precision=precision, amps=psi)
        st.apply_ops(make_ops([(OP_H, 0), (OP_RX, n - 1, 0, 0.3), (OP_CNOT, 0, n - 1)]))
        pageable = st.state()
        buf = llgpu.lib().llg_host_alloc(16 << n)
        assert buf
        try:
            llgpu.check(llgpu.lib().llg_copy_to_host(st._h, buf))
            pinned = np.frombuffer((ctypes.c_double * (2 << n)).from_address(buf), dtype=np.float64).view(np.complex128).copy()
        finally:
            llgpu.lib().llg_host_free(buf)
        assert np.array_equal(pinned, pageable)
        st.close()


@pytest.mark.parametrize("precision", PRECISIONS)
def test_readback_fused_into_last_pass(precision):
    """get_numpy_view with gates still queued: the last tile pass writes the pinned mirror as it
    stores its tiles.  Same bits as flushing first and converting afterwards."""
    import quantum_sim_v3

    n = 14
    ops = workloads.layered_rotations(n, 3)
    a = quantum_sim_v3.StateVector(n, precision)
    a.set_fusion("tile", 10)
    a.apply_ops(ops)
    fused = a.get_numpy_view().copy()
    b = quantum_sim_v3.StateVector(n, precision)
    b.set_fusion("tile", 10)
    b.apply_ops(ops)
    b.flush()
    flushed = b.get_numpy_view().copy()
    assert np.array_equal(fused, flushed)
    tol = 1e-12 if precision != "complex64" else 1e-5
    assert np.max(np.abs(fused - oracle.run_ops(n, ops))) <= tol
    assert np.array_equal(a.get_numpy_view(), fused)  # nothing queued: the plain conversion
    # the mirror stays in step with gates applied after a fused readback
    a.apply_ops(ops)
    b.apply_ops(ops)
    b.flush()
    assert np.array_equal(a.get_numpy_view(), b.get_numpy_view())


def test_alias_entry_points_match():
    """llg_wrap_host / llg_apply_1q / llg_apply_block / llg_expect_diag_zz are the primary entry
    points under other names; llg_apply_1q also rejects a target outside the register."""
    import ctypes

    L = llgpu.lib()
    n = 9
    rng = np.random.default_rng(31)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    amps = np.ascontiguousarray(psi.view(np.float64))
    g = np.array([[np.cos(0.4), -1j * np.sin(0.4)], [-1j * np.sin(0.4), np.cos(0.4)]]).reshape(-1)
    gd = np.ascontiguousarray(g.view(np.float64))
    m = np.linalg.qr(rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8)))[0]
    md = np.ascontiguousarray(m.reshape(-1).view(np.float64))
    qs = (ctypes.c_int * 3)(1, 4, 7)
    a, b, c = llgpu.ring_zz_terms(n)
    ta, tb, tc = (ctypes.c_int * len(a))(*a), (ctypes.c_int * len(b))(*b), (ctypes.c_double * len(c))(*c)
    out = []
    for names in (("llg_create_from_host", "llg_apply_gate", "llg_apply_matrix", "llg_expect_zz"),
                  ("llg_wrap_host", "llg_apply_1q", "llg_apply_block", "llg_expect_diag_zz")):
        h = ctypes.c_void_p()
        llgpu.check(getattr(L, names[0])(amps.ctypes.data, 1 << n, 1, ctypes.byref(h)))
        llgpu.check(getattr(L, names[1])(h, 3, gd.ctypes.data))
        llgpu.check(getattr(L, names[2])(h, 3, qs, md.ctypes.data))
        e = ctypes.c_double()
        llgpu.check(getattr(L, names[3])(h, len(a), ta, tb, tc, ctypes.byref(e)))
        st = np.zeros(2 << n)
        llgpu.check(L.llg_copy_to_host(h, st.ctypes.data))
        if names[1] == "llg_apply_1q":
            assert L.llg_apply_1q(h, n, gd.ctypes.data) == llgpu.LLG_EINVAL
            assert L.llg_apply_1q(h, -1, gd.ctypes.data) == llgpu.LLG_EINVAL
        else:
            assert L.llg_apply_gate(h, n, gd.ctypes.data) == 0  # v3: a target >= n is a no-op
        llgpu.check(L.llg_destroy(h))
        out.append((st, e.value))
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1] == out[1][1]
    # and both are the gate, then the block (qubits[0] the low bit of its index), then the energy
    t = psi.reshape([2] * n)  # axis j is qubit n - 1 - j
    t = np.moveaxis(np.tensordot(g.reshape(2, 2), t, axes=([1], [n - 1 - 3])), 0, n - 1 - 3)
    ax = [n - 1 - 7, n - 1 - 4, n - 1 - 1]
    u = np.moveaxis(t, ax, [0, 1, 2]).reshape(8, -1)
    t = np.moveaxis((m @ u).reshape([2, 2, 2] + [2] * (n - 3)), [0, 1, 2], ax)
    want = t.reshape(-1)
    assert np.max(np.abs(out[0][0].view(np.complex128) - want)) <= 1e-12
    idx = np.arange(1 << n)
    z = lambda q: 1 - 2 * ((idx >> q) & 1)
    diag = sum(ck * z(ak) * (z(bk) if bk >= 0 else 1) for ak, bk, ck in zip(a, b, c))
    assert abs(out[0][1] - float(np.sum(np.abs(want) ** 2 * diag))) <= 1e-11


@pytest.mark.parametrize("precision", ["df64", "fp64"])
def test_every_gate_kind_both_paths(precision):
    rng = np.random.default_rng(8)
    n = 13
    recs = []
    for _ in range(400):
        k = rng.integers(9)
        q = int(rng.integers(n))
        if k == 0:
            recs.append((OP_H, q))
        elif k == 1:
            recs.append((OP_X, q))
        elif k < 5:
            recs.append(((OP_RX, OP_RY, OP_RZ)[k - 2], q, 0, float(rng.uniform(0, 2 * np.pi))))
        elif k < 7:
            a, b = rng.choice(n, 2, replace=False)
            recs.append(((OP_CNOT, OP_CZ)[k - 5], int(a), int(b)))
        elif k == 7:
            recs.append((OP_MCZ, 0, 0, 0.0, int(rng.integers(1, 1 << n))))
        else:
            u, _ = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))
            recs.append((OP_U2, q, 0, 0.0, None, u.reshape(4)))
    ops = make_ops(recs)
    want = oracle.run_ops(n, ops)
    for fusion, tile in (("none", 0), ("tile", 5), ("tile", 9), ("tile", 12)):
        got = run_gpu(n, ops, precision, fusion, tile)
        assert np.max(np.abs(got - want)) <= 1e-12, (fusion, tile)


@pytest.mark.parametrize("precision", ["complex128", "df64"])
def test_config2_recipe_at_24_qubits_vs_oracle(precision):
    # the headline circuit's recipe (20 layers of RX/RY/RZ + CNOT brickwork) at 24 qubits against
    # the CPU restatement, gate by gate, through the fused plan (carried phases, phase tables) in
    # IEEE FP64 and in double-float; the error is also bounded relative to the largest amplitude
    n = 24
    ops = workloads.layered_rotations(n, layers=20)
    want = oracle.run_ops(n, ops)
    st = llgpu.State(n, precision)
    st.apply_ops(ops)
    d = np.max(np.abs(st.state() - want))
    assert d <= 1e-12
    assert d / np.max(np.abs(want)) <= (1e-13 if precision == "complex128" else 1e-11)
    st.close()


def test_config2_at_30_qubits_fused_vs_unfused_fp64():
    # the 30-qubit headline circuit (16 GiB per state): the fused IEEE FP64 plan and the fused
    # double-float plan, each against one IEEE FP64 sweep per gate, compared on the device
    n = 30
    ops = workloads.layered_rotations(n, layers=20)
    ref = llgpu.State(n, "complex128")
    ref.set_fusion("none")
    ref.apply_ops(ops)
    for precision, tol in (("complex128", 1e-13), ("df64", 1e-12)):
        a = llgpu.State(n, precision)
        a.apply_ops(ops)
        fid, dmax = a.compare(ref)
        assert dmax <= tol and abs(1.0 - fid) <= tol, (precision, dmax, fid)
        a.close()
    ref.close()


def test_compare_contract():
    a, b, c = llgpu.State(4), llgpu.State(4, "complex64"), llgpu.State(5)
    a.h(0)
    fid, d = a.compare(b)
    assert abs(fid - 0.5) < 1e-12 and abs(d - 2 ** -0.5) < 1e-7
    with pytest.raises(ValueError):
        a.compare(c)
    for s in (a, b, c):
        s.close()


def test_twenty_qubit_layered_vs_oracle():
    n = 20
    ops = workloads.layered_rotations(n, layers=4, seed=12)
    want = oracle.run_ops(n, ops)
    for fusion in ("tile", "none"):
        got = run_gpu(n, ops, "df64", fusion)
        assert np.max(np.abs(got - want)) <= 1e-12
    # complex64: the direction to 1e-9 in fidelity; the norm drifts at the level of fp32 rounding
    # of the gates' coefficients (a slightly non-unitary matrix applied to every amplitude)
    got = run_gpu(n, ops, "complex64", "tile")
    norm = np.vdot(got, got).real
    fid = abs(np.vdot(want, got)) ** 2 / norm
    assert 1 - fid < 1e-9 and abs(norm - 1) < 1e-5


def _sk_terms(n, seed):
    # Sherrington-Kirkpatrick couplings J_ij ~ N(0, 1/n) on every pair plus random fields: more
    # terms and distinct coefficients than the class-counting kernel takes
    rng = np.random.default_rng(seed)
    zz = [(i, j, float(rng.normal() / np.sqrt(n))) for i in range(n) for j in range(i + 1, n)]
    z = [(i, float(rng.normal())) for i in range(n)]
    return llgpu.ising_terms(n, zz, z)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_sk_energy_matches_oracle(precision):
    # a 20-qubit SK-model energy (190 couplings + 20 fields) through llg_expect_zz's general
    # kernel, and the same diagonal as a full 2^n vector through llg_expect_diagonal (host and
    # device copies), against the oracle's term-by-term sum
    n = 20
    a, b, c = _sk_terms(n, 5)
    ops = workloads.layered_rotations(n, layers=2, seed=9)
    psi = oracle.run_ops(n, ops)
    want = oracle.expect_zz(psi, n, a, b, c)
    st = llgpu.State(precision=precision, amps=psi)
    tol = 1e-11 if precision != "complex64" else 1e-5
    assert abs(st.expect_zz(a, b, c) - want) <= tol
    assert abs(st.expect_zz(a, b, c) - want) <= tol  # the cached device layout
    d = llgpu.diag_export(n, a, b, c)
    assert abs(st.expect_diagonal(d) - want) <= tol
    torch = pytest.importorskip("torch")
    assert abs(st.expect_diagonal(torch.from_numpy(d).cuda()) - want) <= tol
    # a small observable still takes the class-counting kernel, after the large one
    ra, rb, rc = llgpu.ring_zz_terms(n)
    assert abs(st.expect_zz(ra, rb, rc) - oracle.expect_zz(psi, n, ra, rb, rc)) <= tol
    st.close()


def test_apply_fused_gate_list():
    # GateFuser.fuse_circuit output fed to StateVector.apply_fused (python/gate_fusion.py:15-37,
    # benchmarks/benchmark_fusion.py:36-50): the fused list gives the unfused circuit's state
    import quantum_sim_v3
    from gate_fusion import GATES, GateFuser

    rng = np.random.default_rng(44)
    n = 12
    gates = []
    for _ in range(400):
        q = int(rng.integers(n))
        if rng.uniform() < 0.5:
            gates.append((q, GATES[["X", "H", "S", "T"][int(rng.integers(4))]]))
        else:
            u = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))[0]
            gates.append((q, list(u.reshape(4))))
    fused = GateFuser.fuse_circuit(gates)
    assert len(fused) < len(gates)
    want = oracle.zero_state(n)
    for q, g in gates:
        oracle.apply_gate_v3(want, n, q, g)
    for precision in ("complex128", "df64"):
        sv = quantum_sim_v3.StateVector(n, precision)
        sv.apply_fused(fused)
        assert np.max(np.abs(sv.get_numpy_view() - want)) <= 1e-12, precision


@pytest.mark.parametrize("tile", [9, 11, 13])
def test_register_tiled_passes(golden, tile):
    # complex64 register-tiled passes (16 amplitudes per thread, shared memory only between
    # layouts) against the oracle: every gate kind, non-local CNOT controls and MCZ masks, the
    # layered recipe, and the readback fused into the last pass
    import quantum_sim_v3

    rng = np.random.default_rng(70 + tile)
    n = 15
    recs = []
    for _ in range(300):
        k = rng.integers(9)
        q = int(rng.integers(n))
        if k == 0:
            recs.append((OP_H, q))
        elif k == 1:
            recs.append((OP_X, q))
        elif k < 5:
            recs.append(((OP_RX, OP_RY, OP_RZ)[k - 2], q, 0, float(rng.uniform(0, 2 * np.pi))))
        elif k < 7:
            a, b = rng.choice(n, 2, replace=False)
            recs.append(((OP_CNOT, OP_CZ)[k - 5], int(a), int(b)))
        elif k == 7:
            recs.append((OP_MCZ, 0, 0, 0.0, int(rng.integers(1, 1 << n))))
        else:
            u, _ = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))
            recs.append((OP_U2, q, 0, 0.0, None, u.reshape(4)))
    for ops in (make_ops(recs), workloads.layered_rotations(n, layers=6, seed=tile)):
        want = oracle.run_ops(n, ops)
        got = run_gpu(n, ops, "complex64", "reg", tile)
        assert np.max(np.abs(got - want)) <= 5e-5
        sv = quantum_sim_v3.StateVector(n, "complex64")
        sv.set_fusion("reg", tile)
        sv.apply_ops(ops)
        view = sv.get_numpy_view().copy()  # gates queued: the last pass also writes the host mirror
        assert np.max(np.abs(view - want)) <= 5e-5
    with pytest.raises(ValueError):
        llgpu.State(12, "df64").set_fusion("reg", 12)
