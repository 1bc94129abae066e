"""Adjoint-method gradients on the GPU, checked against the reference's parameter-shift rule
(fixtures from the reference build, the CPU oracle and the GPU parameter-shift path), central
finite differences, checkpointed reverse sweeps and the torch.autograd.Function.

Tolerances: gradients <= 1e-10 against parameter shift (complex128 and fp64); central finite
differences with h = 1e-6 only to 1e-7 (their own rounding error eps*|E|/h is ~1e-9);
complex64 gradients to 5e-5."""
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


@pytest.mark.parametrize("precision", ["df64", "fp64"])
def test_hea_gradients_match_reference_parameter_shift(golden, precision):
    g = golden("hea_param_shift")
    n = int(g["n"])
    adj = llgpu.Adjoint(n, g["ops"], g["params"].shape[1], llgpu.ring_zz_terms(n), max_batch=4, precision=precision)
    e, gr = adj.run(g["params"])
    assert np.max(np.abs(e - g["energies"])) <= 1e-10
    assert np.max(np.abs(gr - g["grads"])) <= 1e-10
    e2, gr2 = adj.param_shift(g["params"])
    assert np.max(np.abs(gr2 - g["grads"])) <= 1e-10
    adj.close()


def test_vqe_ansatz_gradients_match_reference(golden):
    from test_oracle_golden import vqe_ops

    g = golden("vqe_param_shift")
    for n, layers in ((4, 2), (6, 3)):
        key = f"n{n}_l{layers}"
        theta = g[key + "_theta"]
        ops = vqe_ops(n, layers, theta)
        adj = llgpu.Adjoint(n, ops, theta.size, llgpu.ring_zz_terms(n), max_batch=1)
        e, gr = adj.run(theta[None, :])
        assert abs(e[0] - g[key + "_energy"]) <= 1e-10
        assert np.max(np.abs(gr[0] - g[key + "_grad"])) <= 1e-10
        adj.close()


def mixed_param_circuit(n, depth, nparams, rng):
    """Random circuit with parametrised RX/RY/RZ (shared parameters included) and fixed gates of
    every kind, so the reverse sweep sees local, non-local and fused ops."""
    recs = []
    for _ in range(depth):
        k = rng.integers(11)
        q = int(rng.integers(n))
        if k < 3:
            recs.append(((OP_RX, OP_RY, OP_RZ)[k], q, 0, 0.0, None, None, int(rng.integers(nparams))))
        elif k == 3:
            recs.append((OP_H, q))
        elif k == 4:
            recs.append((OP_X, q))
        elif k == 5:
            recs.append((OP_RZ, q, 0, float(rng.uniform(0, 6))))
        elif k in (6, 7):
            a, b = rng.choice(n, 2, replace=False)
            recs.append(((OP_CNOT, OP_CZ)[k - 6], int(a), int(b)))
        elif k == 8:
            recs.append((OP_MCZ, 0, 0, 0.0, int(rng.integers(1, 1 << n))))
        elif k == 9:
            recs.append((OP_RY, q, 0, float(rng.uniform(0, 6))))
        else:
            u, _ = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))
            recs.append((OP_U2, q, 0, 0.0, None, u.reshape(4)))
    return make_ops(recs)


def test_mixed_circuit_adjoint_vs_oracle_and_gpu_parameter_shift():
    rng = np.random.default_rng(12)
    n, nparams = 14, 24
    ops = mixed_param_circuit(n, 160, nparams, rng)
    obs = ([0, 3, 5, 13, 2], [1, 9, -1, 0, -1], [1.0, 0.5, -0.75, 1.0, 0.25])
    params = rng.uniform(0, 2 * np.pi, size=(3, nparams))
    adj = llgpu.Adjoint(n, ops, nparams, obs, max_batch=8)
    info = adj.info()
    assert info["forward_passes"] > 1  # 14 qubits > 11-qubit tiles: several passes, non-local ops
    e, gr = adj.run(params)
    e_ps, g_ps = adj.param_shift(params)
    assert np.max(np.abs(e - e_ps)) <= 1e-12
    assert np.max(np.abs(gr - g_ps)) <= 1e-10
    for b in range(2):
        e_o, g_o = oracle.param_shift(n, ops, params[b], *obs)
        assert abs(e[b] - e_o) <= 1e-10
        assert np.max(np.abs(gr[b] - g_o)) <= 1e-10
    adj.close()


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_long_rotation_pass_rescales(precision):
    """720 parametrised RX / RY in one tile pass, angles near pi/2 and 3pi/2 (both tangent and
    cotangent forms, either sign): the IEEE complex128 kernels' running factor of dropped cosines
    falls below 2^-300 and the tiles are rescaled in place, in the forward and the reverse sweep."""
    rng = np.random.default_rng(31)
    n, nrot = 5, 720
    recs = []
    for k in range(nrot):
        recs.append(((OP_RX, OP_RY)[k % 2], int(rng.integers(n)), 0, 0.0, None, None, k))
        if k % 9 == 8:
            a, b = rng.choice(n, 2, replace=False)
            recs.append(((OP_CNOT, OP_CZ)[k % 2], int(a), int(b)))
    ops = make_ops(recs)
    params = np.where(rng.random((2, nrot)) < 0.5, np.pi / 2, -1.5 * np.pi) + rng.uniform(-0.1, 0.1, (2, nrot))
    obs = ([0, 1, 2], [1, -1, 4], [1.0, -0.5, 0.75])
    adj = llgpu.Adjoint(n, ops, nrot, obs, max_batch=2, precision=precision)
    assert adj.info()["forward_passes"] == 1
    e, gr = adj.run(params)
    for b in range(2):
        e_o, g_o = oracle.param_shift(n, ops, params[b], *obs)
        assert abs(e[b] - e_o) <= 1e-10
        assert np.max(np.abs(gr[b] - g_o)) <= 1e-10
    adj.close()


def test_checkpointed_reverse_sweep_agrees():
    rng = np.random.default_rng(4)
    n = 16
    ops = workloads.hea_ansatz(n, 6)
    nparams = 6 * 2 * n
    params = rng.uniform(0, 2 * np.pi, size=(4, nparams))
    adj = llgpu.Adjoint(n, ops, nparams, llgpu.ring_zz_terms(n), max_batch=4)
    assert adj.info()["forward_passes"] >= 4
    e0, g0 = adj.run(params, checkpoint_every=0)
    for c in (1, 2, 3):
        e1, g1 = adj.run(params, checkpoint_every=c)
        assert np.max(np.abs(e1 - e0)) <= 1e-13
        assert np.max(np.abs(g1 - g0)) <= 1e-12
    adj.close()


def test_central_finite_differences():
    rng = np.random.default_rng(9)
    n = 10
    ops = workloads.hea_ansatz(n, 3)
    nparams = 3 * 2 * n
    theta = rng.uniform(0, 2 * np.pi, size=nparams)
    adj = llgpu.Adjoint(n, ops, nparams, llgpu.ring_zz_terms(n), max_batch=2 * nparams + 1)
    _, g = adj.run(theta[None, :])
    h = 1e-6
    rows = np.repeat(theta[None, :], 2 * nparams, axis=0)
    for k in range(nparams):
        rows[2 * k, k] += h
        rows[2 * k + 1, k] -= h
    e, _ = adj.run(rows, grads=False)
    fd = (e[0::2] - e[1::2]) / (2 * h)
    assert np.max(np.abs(fd - g[0])) <= 1e-7
    adj.close()


def test_complex64_gradients():
    rng = np.random.default_rng(2)
    n = 12
    ops = workloads.hea_ansatz(n, 4)
    nparams = 4 * 2 * n
    params = rng.uniform(0, 2 * np.pi, size=(2, nparams))
    ref = llgpu.Adjoint(n, ops, nparams, llgpu.ring_zz_terms(n), max_batch=2)
    c64 = llgpu.Adjoint(n, ops, nparams, llgpu.ring_zz_terms(n), max_batch=2, precision="complex64")
    _, g_ref = ref.run(params)
    _, g_64 = c64.run(params)
    assert np.max(np.abs(g_64 - g_ref)) <= 5e-5


def test_torch_autograd_function():
    torch = pytest.importorskip("torch")
    import adjoint

    n = 12
    ops = workloads.hea_ansatz(n, 3)
    nparams = 3 * 2 * n
    circ = adjoint.AdjointCircuit(n, ops, nparams, llgpu.ring_zz_terms(n), max_batch=8)
    theta = torch.rand(5, nparams, dtype=torch.float64, device="cuda") * 6.28
    theta.requires_grad_(True)
    w = torch.arange(1, 6, dtype=torch.float64, device="cuda")
    energy = circ(theta)
    (energy * w).sum().backward()
    e_np, g_np = circ.handle.run(theta.detach().cpu().numpy())
    assert np.max(np.abs(energy.detach().cpu().numpy() - e_np)) <= 1e-13
    assert np.max(np.abs(theta.grad.cpu().numpy() - w.cpu().numpy()[:, None] * g_np)) <= 1e-12
    with torch.no_grad():
        e_only = circ(theta)
    assert torch.allclose(e_only, energy.detach(), atol=1e-13, rtol=0)


def test_config3_full_size():
    """20 qubits, 10 layers of RY/RZ + CZ ring, 400 parameters, batch of 64 parameter sets."""
    n, layers, batch = 20, 10, 64
    ops = workloads.hea_ansatz(n, layers)
    nparams = layers * 2 * n
    params = workloads.hea_params(n, layers, batch)
    adj = llgpu.Adjoint(n, ops, nparams, llgpu.ring_zz_terms(n), max_batch=batch)
    e, g = adj.run(params)
    e_ps, g_ps = adj.param_shift(params[:1])
    assert np.max(np.abs(g[0] - g_ps[0])) <= 1e-10
    assert abs(e[0] - e_ps[0]) <= 1e-12
    # CPU oracle: the energy of set 1 and two parameter-shift components
    psi = oracle.run_ops(n, workloads.bind_params(ops, params[1]))
    assert abs(oracle.expect_zz(psi, n, *llgpu.ring_zz_terms(n)) - e[1]) <= 1e-10
    for k in (0, 217):
        vals = []
        for sh in (np.pi / 2, -np.pi / 2):
            p = params[1].copy()
            p[k] += sh
            s = oracle.run_ops(n, workloads.bind_params(ops, p))
            vals.append(oracle.expect_zz(s, n, *llgpu.ring_zz_terms(n)))
        assert abs(0.5 * (vals[0] - vals[1]) - g[1, k]) <= 1e-10
    adj.close()


@pytest.mark.parametrize("precision", ["complex128", "df64"])
def test_sk_model_energy_and_gradients(precision):
    # a 20-qubit SK-model observable (190 all-to-all couplings, 20 fields: beyond the class-counting
    # kernel) on a one-layer RY/RZ + CZ-ring ansatz (40 parameters): energies and adjoint gradients
    # against the oracle (the reference's ising_diagonal restated, energy = probabilities . diag,
    # the parameter-shift rule on selected parameters) and every gradient against the GPU's
    # parameter shift
    n, layers = 20, 1
    rng = np.random.default_rng(21)
    zz = [(i, j, float(rng.normal() / np.sqrt(n))) for i in range(n) for j in range(i + 1, n)]
    z = [(i, float(rng.normal())) for i in range(n)]
    obs = llgpu.ising_terms(n, zz, z)
    ops = workloads.hea_ansatz(n, layers)
    nparams = 2 * n * layers
    params = rng.uniform(0, 2 * np.pi, size=(2, nparams))
    adj = llgpu.Adjoint(n, ops, nparams, obs, max_batch=2, precision=precision)
    e, g = adj.run(params)
    _, g_ps = adj.param_shift(params)
    adj.close()
    assert np.max(np.abs(g - g_ps)) <= 1e-10
    idx = np.arange(1 << n, dtype=np.int64)
    s = [1.0 - 2.0 * ((idx >> q) & 1) for q in range(n)]
    diag = np.zeros(idx.size)
    for i, j, cpl in zz:
        diag += cpl * s[i] * s[j]
    for i, h in z:
        diag += h * s[i]

    def energy(theta):
        o = ops.copy()
        sel = o["param"] >= 0
        o["theta"][sel] = theta[o["param"][sel]]
        return float(np.dot(oracle.probabilities(oracle.run_ops(n, o), n), diag))

    assert abs(e[0] - energy(params[0])) <= 1e-10
    for k in (0, 7, 19, 20, 33, 39):
        tp, tm = params[0].copy(), params[0].copy()
        tp[k] += np.pi / 2
        tm[k] -= np.pi / 2
        assert abs(g[0, k] - 0.5 * (energy(tp) - energy(tm))) <= 1e-10, k
