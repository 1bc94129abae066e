"""The algorithms module on the GPU backend (quantum_sim_algorithms.make_gpu_backend): Grover,
QAOA and VQE give the reference's outputs -- fixtures written by running the reference's own
Algorithms.h on ll::StateVectorBackend (tests/golden/gen_golden.py).

Tolerances: probabilities <= 1e-12; VQE energies <= 1e-10 and parameters <= 1e-9 after the whole
gradient descent (parameter-shift gradients on the GPU, the reference's mt19937_64 start)."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

import llgpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def alg(built):
    assert llgpu.device_count() > 0
    import quantum_sim_algorithms

    return quantum_sim_algorithms


def test_grover_matches_reference(alg, golden):
    g = golden("grover")
    be = alg.make_gpu_backend(1)
    for key, n, iters in (("n8_m85", 8, -1), ("n10_i10", 10, 10), ("n12_i10", 12, 10)):
        r = alg.Grover.run(be, n, [int(m) for m in g[key + "_marked"]], iters)
        assert r.iterations == int(g[key + "_iterations"]) and r.marked_index == int(g[key + "_marked_index"])
        assert np.max(np.abs(r.probabilities - g[key + "_probs"])) <= 1e-12
    assert abs(alg.Grover.run(be, 8, [85]).probabilities[85] - 0.99994704) < 5e-9  # README.md:509


@pytest.mark.parametrize("precision", ["complex128", "df64"])
def test_qaoa_matches_reference(alg, golden, precision):
    from gen_golden import algorithm_cases

    g = golden("algorithms")
    qaoa, _ = algorithm_cases()
    be = alg.make_gpu_backend(1, precision)
    for label, (n, edges), gammas, betas in qaoa:
        r = alg.QAOA.run(be, alg.Graph(n, edges), gammas, betas)
        assert np.max(np.abs(r.probabilities - g[f"qaoa_{label}_probs"])) <= 1e-12, label
        assert r.best_cut == pytest.approx(float(g[f"qaoa_{label}_best_cut"]), abs=1e-12)
        assert be.n_qubits() == n


def test_vqe_optimize_matches_reference(alg, golden):
    from gen_golden import algorithm_cases

    g = golden("algorithms")
    _, vqe_cases = algorithm_cases()
    for label, n, layers, seed, iters, lr, zz, z in vqe_cases:
        a, b, c = llgpu.ising_terms(n, zz, z)
        be = alg.make_gpu_backend(n)
        vqe = alg.VQE(n, layers, seed)

        def energy(params):  # the energy evaluated on the device
            vqe.prepare(be, list(params))
            return be.expect_zz(a, b, c)

        r = vqe.optimize(be, energy, iters, lr)
        assert r.iterations == int(g[f"vqe_{label}_iterations"])
        assert abs(r.energy - float(g[f"vqe_{label}_energy"])) <= 1e-10
        assert np.max(np.abs(r.params - g[f"vqe_{label}_params"])) <= 1e-9
        # optimize leaves the best state prepared, as the reference does
        assert np.max(np.abs(be.probabilities() - g[f"vqe_{label}_probs"])) <= 1e-12


def test_vqe_energy_from_a_full_diagonal(alg, golden):
    # run_vqe(hamiltonian_diag=...) style: the energy is probabilities . diag; on the GPU backend
    # the diagonal (host array or device tensor) is read by the device, not the probabilities
    from gen_golden import algorithm_cases

    g = golden("algorithms")
    _, vqe_cases = algorithm_cases()
    label, n, layers, seed, iters, lr, zz, z = vqe_cases[1]
    diag = llgpu.diag_export(n, *llgpu.ising_terms(n, zz, z))
    torch = pytest.importorskip("torch")
    for d in (diag, torch.from_numpy(diag).cuda()):
        be = alg.make_gpu_backend(n)
        vqe = alg.VQE(n, layers, seed)
        r = vqe.optimize(be, lambda p: (vqe.prepare(be, list(p)), be.expect_diagonal(d))[1], iters, lr)
        assert abs(r.energy - float(g[f"vqe_{label}_energy"])) <= 1e-10
        host = float(np.dot(be.probabilities(), diag))
        assert abs(host - r.energy) <= 1e-12


def test_algorithm_error_contract(alg):
    be = alg.make_gpu_backend(2)
    with pytest.raises(ValueError):
        alg.Grover.run(be, 3, [])
    with pytest.raises(ValueError):
        alg.Grover.run(be, 3, [8])
    with pytest.raises(ValueError):
        alg.QAOA.run(be, alg.Graph(3, [(0, 0, 1.0)]), [0.1], [0.2])
    with pytest.raises(ValueError):
        alg.QAOA.run(be, alg.Graph(3, [(0, 1, 1.0)]), [0.1], [])
    with pytest.raises(ValueError):
        alg.VQE(0, 1)
    v = alg.VQE(3, 1)
    with pytest.raises(ValueError):
        v.prepare(be, [0.1])
    with pytest.raises(RuntimeError):
        v.optimize(be, lambda p: float("nan"), 2, 0.1)
