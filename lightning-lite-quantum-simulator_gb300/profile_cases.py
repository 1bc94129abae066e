"""Small workloads, one kernel family each, for ncu captures (the commands that made the summaries
under profiles/ name this script).  Each case runs its kernel a few times on a state larger than
the 129 MB L2 but of a few GB at most, so a capture of one to three launches ends in seconds.

    python profile_cases.py <case> [<case> ...]       cases: see CASES
"""
from __future__ import annotations

import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

import llgpu  # noqa: E402
import workloads  # noqa: E402


def tile_f64():
    """IEEE complex128 tile passes with phase tables: the 30-qubit recipe's circuit at 26 qubits
    (1 GiB), 12-qubit tiles and 256 threads (the tuner's choice at 30 qubits)."""
    n = 26
    st = llgpu.State(n, "complex128")
    st.set_fusion("tile", 12)
    st.set_tile_threads(256)
    st.apply_ops(workloads.layered_rotations(n, 4))
    st.sync()
    st.close()


def tile_reg_c64():
    """complex64 register-tiled passes, 27 qubits (1 GiB), 13-qubit tiles."""
    n = 27
    st = llgpu.State(n, "complex64")
    st.set_fusion("reg", 13)
    st.apply_ops(workloads.layered_rotations(n, 4))
    st.sync()
    st.close()


def tile_c64():
    """complex64 shared-memory tile passes, 27 qubits, 13-qubit tiles (the register kernel's baseline)."""
    n = 27
    st = llgpu.State(n, "complex64")
    st.set_fusion("tile", 13)
    st.apply_ops(workloads.layered_rotations(n, 4))
    st.sync()
    st.close()


def streaming():
    """Per-gate streaming kernels on a 27-qubit complex128 state (2 GiB): CNOT (control 3, target
    20), CZ / MCZ (3, 20), RY on qubit 13."""
    n = 27
    st = llgpu.State(n, "complex128")
    st.set_fusion("none")
    st.apply_ops(llgpu.make_ops([(llgpu.OP_CNOT, 3, 20)] * 3 + [(llgpu.OP_CZ, 3, 20)] * 3 +
                                [(llgpu.OP_RY, 13, 0, 0.4)] * 3))
    st.sync()
    st.close()


def reductions():
    """Observable reductions on a 27-qubit complex128 state: the class-counting kernel (ring ZZ,
    27 terms) and the chunked kernel (all-to-all couplings, 351 terms + 27 fields)."""
    n = 27
    st = llgpu.State(n, "complex128")
    st.apply_ops(workloads.layered_rotations(n, 1))
    a, b, c = llgpu.ring_zz_terms(n)
    rng = np.random.default_rng(3)
    zz = [(i, j, float(rng.normal())) for i in range(n) for j in range(i + 1, n)]
    z = [(i, float(rng.normal())) for i in range(n)]
    sa, sb, sc = llgpu.ising_terms(n, zz, z)
    for _ in range(3):
        st.expect_zz(a, b, c)
        st.expect_zz(sa, sb, sc)
    st.close()


def readback():
    """The host readback of a 26-qubit complex128 state into pinned memory (the conversion /
    copy kernel writing the mapped host buffer)."""
    import quantum_sim_v3

    n = 26
    sv = quantum_sim_v3.StateVector(n)
    sv.h(0)
    for _ in range(3):
        sv.get_numpy_view()
        sv.h(1)
        sv.flush()


def tsolve():
    """The dense trajectory solver at dim 1024 (10 qubits), 256 trajectories of 20 steps."""
    rng = np.random.default_rng(11)
    d = 1024
    a = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    h = (a + a.conj().T) / (4 * np.sqrt(d))
    s = llgpu.TrajectorySolver(10)
    s.set_hamiltonian(h)
    sm = np.array([[0, 1], [0, 0]], dtype=complex)
    s.add_lindblad(np.kron(np.eye(d // 2), sm), 0.4)
    psi0 = rng.normal(size=d) + 1j * rng.normal(size=d)
    s.states(psi0, 0.4, 0.02, 256, "PROJECTOR", seed=5)
    s.close()


def block_tc():
    """A dense 5-qubit block on a 26-qubit double-float state (1 GiB) on the tensor cores: a random
    32x32 unitary on qubits (0, 7, 13, 22, 25), applied three times after a layer of H."""
    n = 26
    st = llgpu.State(n, "df64")
    st.apply_ops(llgpu.make_ops([(llgpu.OP_H, q) for q in range(n)]))
    rng = np.random.default_rng(17)
    m = np.linalg.qr(rng.normal(size=(32, 32)) + 1j * rng.normal(size=(32, 32)))[0]
    for _ in range(3):
        st.apply_matrix([0, 7, 13, 22, 25], m)
    st.sync()
    st.close()


def block_tc_f64():
    """A dense 4-qubit block on a 26-qubit IEEE complex128 state (1 GiB) on the tensor cores (eight
    exact slices): a random 16x16 unitary on qubits (0, 7, 13, 25), three times after a layer of H."""
    n = 26
    st = llgpu.State(n, "complex128")
    st.apply_ops(llgpu.make_ops([(llgpu.OP_H, q) for q in range(n)]))
    rng = np.random.default_rng(19)
    m = np.linalg.qr(rng.normal(size=(16, 16)) + 1j * rng.normal(size=(16, 16)))[0]
    for _ in range(3):
        st.apply_matrix([0, 7, 13, 25], m)
    st.sync()
    st.close()


def dm_sparse():
    """Noise channels on a 13-qubit IEEE complex128 density matrix (a 26-qubit state, 1 GiB) through
    the sparse block kernel: amplitude damping on qubits 0..2, then 2-qubit depolarizing on
    (3, 4), (5, 6)."""
    dm = llgpu.DensityMatrix(13, "complex128")
    dm.apply_ops(llgpu.make_ops([(llgpu.OP_H, q) for q in range(13)]))
    ad, dp = llgpu.amplitude_damping(0.01), llgpu.depolarizing(0.01, 2)
    for q in range(3):
        dm.kraus(ad, [q])
    for q in (3, 5):
        dm.kraus(dp, [q, q + 1])
    dm.state.sync()
    dm.close()


def traj_f64():
    """IEEE complex128 noisy trajectories: 512 trajectories of the 14-qubit, 8-layer RX/RY +
    CNOT-chain circuit with amplitude damping and dephasing sites (one launch of the default
    configuration)."""
    ops = workloads.noisy_layers(14, 8)
    h = llgpu.Traj(14, ops, 0.01, 0.005, 512, "complex128")
    h.launch(2024, 512)
    h.launch(2024, 512)
    h.close()


def adjoint_f64():
    """IEEE complex128 adjoint gradients: the 20-qubit, 10-layer RY/RZ + CZ-ring ansatz, a batch of
    8 parameter sets (128 MiB per buffer)."""
    n, layers, batch = 20, 10, 8
    adj = llgpu.Adjoint(n, workloads.hea_ansatz(n, layers), 2 * n * layers, llgpu.ring_zz_terms(n), max_batch=batch,
                        precision="complex128")
    params = workloads.hea_params(n, layers, batch)
    adj.run(params)
    adj.run(params)
    adj.close()


CASES = {"tile_f64": tile_f64, "traj_f64": traj_f64, "adjoint_f64": adjoint_f64, "block_tc": block_tc, "block_tc_f64": block_tc_f64, "dm_sparse": dm_sparse, "tile_reg_c64": tile_reg_c64, "tile_c64": tile_c64, "streaming": streaming,
         "reductions": reductions, "readback": readback, "tsolve": tsolve}

if __name__ == "__main__":
    for name in sys.argv[1:]:
        CASES[name]()
    print("profile cases done:", " ".join(sys.argv[1:]))
