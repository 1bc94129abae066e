"""Writes the golden fixtures in this directory by running the REFERENCE's own code.

Runs only where the reference tree is present (found by oracle/build_oracle.py's
reference_root(); it is read in place, never copied):
  * oracle/_ref/libref.so -- ll::ReferenceBackend, ll::StateVectorBackend, ll::Grover,
    ll::VQE::prepare, ll::NoisyBackend and ll::ZNE compiled from the reference headers
    (oracle/build_oracle.py --ref);
  * oracle/_ref/quantum_sim_v3 / quantum_sim_v2 -- the reference pybind11 modules built from
    src/StateVectorOptimized.cpp and src/bindings_v2.cpp;
  * python/gate_fusion.py imported from the reference tree.
The .npz files it writes are committed; the tests read them on any machine.

    python tests/golden/gen_golden.py
"""
from __future__ import annotations

import ctypes
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "lightning-lite-quantum-simulator_gb300"))

import build_oracle  # noqa: E402

REF = build_oracle.reference_root()
import workloads  # noqa: E402
from llgpu import OP_DTYPE  # noqa: E402

PI = np.pi


def load_ref():
    paths = build_oracle.build_ref(REF)
    L = ctypes.CDLL(paths["libref.so"])
    vp, i, d, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_uint64
    L.ref_run_ops.argtypes = [i, i, vp, i, vp]
    L.ref_probabilities.argtypes = [i, i, vp, i, vp]
    L.ref_rng_new.restype = vp
    L.ref_rng_new.argtypes = [u64]
    L.ref_rng_free.argtypes = [vp]
    L.ref_random_circuit.argtypes = [vp, i, i, vp]
    L.ref_grover.argtypes = [i, vp, i, i, vp, ctypes.POINTER(i), ctypes.POINTER(i)]
    L.ref_vqe_prepare.argtypes = [i, i, vp, vp]
    L.ref_noisy_obs.argtypes = [i, vp, i, d, i, u64, i, i, vp, vp, vp, vp]
    L.ref_zne.argtypes = [i, vp, i, d, u64, vp, i, i, i, vp, vp, vp, vp]
    L.ref_qaoa.argtypes = [i, i, vp, vp, vp, i, vp, vp, vp, ctypes.POINTER(d)]
    L.ref_vqe_optimize.argtypes = [i, i, u64, i, d, i, vp, vp, vp, ctypes.POINTER(d), vp, ctypes.POINTER(i), vp]
    mods = {}
    for name in ("quantum_sim_v3", "quantum_sim_v2"):
        path = [p for k, p in paths.items() if k.startswith(name)][0]
        spec = importlib.util.spec_from_file_location(name, path)
        m = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(m)
        mods[name] = m
    return L, mods


def ref_state(L, backend: int, n: int, ops: np.ndarray) -> np.ndarray:
    out = np.zeros(1 << n, dtype=np.complex128)
    ops = np.ascontiguousarray(ops)
    rc = L.ref_run_ops(backend, n, ops.ctypes.data if ops.size else None, ops.size, out.ctypes.data)
    assert rc == 0, rc
    return out


def pack(circuits):
    """list of op arrays -> (concatenated ops, offsets)"""
    offs = np.zeros(len(circuits) + 1, dtype=np.int64)
    for k, c in enumerate(circuits):
        offs[k + 1] = offs[k] + len(c)
    ops = np.concatenate(circuits) if circuits else np.zeros(0, dtype=OP_DTYPE)
    return ops, offs


def gen_random_2024(L):
    # tests/test_backends.cpp:205-232: mt19937_64(2024), n = 1..6, 5 trials x 200 gates, then one
    # 500-gate circuit at n = 6, all from the same stream.
    rng = L.ref_rng_new(2024)
    circuits, ns, ref_states, sv_states = [], [], [], []
    for n in range(1, 7):
        for _ in range(5):
            ops = np.zeros(200, dtype=OP_DTYPE)
            L.ref_random_circuit(rng, n, 200, ops.ctypes.data)
            circuits.append(ops)
            ns.append(n)
    ops = np.zeros(500, dtype=OP_DTYPE)
    L.ref_random_circuit(rng, 6, 500, ops.ctypes.data)
    circuits.append(ops)
    ns.append(6)
    L.ref_rng_free(rng)
    for n, c in zip(ns, circuits):
        ref_states.append(ref_state(L, 0, n, c))
        sv_states.append(ref_state(L, 1, n, c))
    ops, offs = pack(circuits)
    states = np.concatenate(ref_states)
    soffs = np.concatenate([[0], np.cumsum([1 << n for n in ns])])
    np.savez_compressed(os.path.join(HERE, "random_2024.npz"), ops=ops, offsets=offs, n=np.array(ns),
                        ref_states=states, sv_states=np.concatenate(sv_states), state_offsets=soffs)


def gen_config1(L):
    circuits, ns, states = [], [], []
    for n in (4, 6, 8, 10, 12):
        ops = workloads.mixed_h_cnot(n, 1000, seed=1234)
        circuits.append(ops)
        ns.append(n)
        states.append(ref_state(L, 1, n, ops))
    ops, offs = pack(circuits)
    soffs = np.concatenate([[0], np.cumsum([1 << n for n in ns])])
    np.savez_compressed(os.path.join(HERE, "config1_h_cnot.npz"), ops=ops, offsets=offs, n=np.array(ns),
                        states=np.concatenate(states), state_offsets=soffs)


def gen_config2(L):
    circuits, ns, states = [], [], []
    for n in (6, 10, 12):
        ops = workloads.layered_rotations(n, layers=20, seed=2030)
        circuits.append(ops)
        ns.append(n)
        states.append(ref_state(L, 1, n, ops))
    ops, offs = pack(circuits)
    soffs = np.concatenate([[0], np.cumsum([1 << n for n in ns])])
    np.savez_compressed(os.path.join(HERE, "config2_layered.npz"), ops=ops, offsets=offs, n=np.array(ns),
                        states=np.concatenate(states), state_offsets=soffs)


def gen_v3(mods):
    # quantum_sim_v3 apply_gate_cache_optimized / apply_gate_standard and quantum_sim_v2 apply_gate
    # through the reference's own pybind11 API (gates passed as Python lists of 4 complex).
    rng = np.random.default_rng(77)
    n = 10
    init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    init /= np.linalg.norm(init)
    targets = rng.integers(0, n + 2, size=40)  # includes targets >= n (reference: no-op)
    gates = rng.normal(size=(40, 4)) + 1j * rng.normal(size=(40, 4))
    outs = {}
    for label, mod, meth in (("v3_cache", "quantum_sim_v3", "apply_gate_cache_optimized"),
                             ("v3_standard", "quantum_sim_v3", "apply_gate_standard"),
                             ("v2", "quantum_sim_v2", "apply_gate")):
        buf = init.copy()
        sv = mods[mod].StateVector(buf)
        for t, g in zip(targets, gates):
            # targets >= n: a no-op in apply_gate_cache_optimized (num_blocks = 0), but the mask-scan
            # variants write past the array (src/StateVectorOptimized.cpp:85-95,
            # src/bindings_v2.cpp:60-70), so they only get in-range targets
            if t >= n and meth != "apply_gate_cache_optimized":
                continue
            getattr(sv, meth)(int(t), [complex(x) for x in g])
        outs[label] = np.array(sv.get_numpy_view(), copy=True)
        assert np.array_equal(outs[label], buf)  # zero-copy: the caller's array was mutated
    # |0..0> constructor + view
    sv = mods["quantum_sim_v3"].StateVector(5)
    h = 1 / np.sqrt(2)
    sv.apply_gate_cache_optimized(0, [h, h, h, -h])
    sv.apply_gate_cache_optimized(4, [0, 1, 1, 0])
    ctor_view = np.array(sv.get_numpy_view(), copy=True)
    np.savez_compressed(os.path.join(HERE, "v3_gates.npz"), n=n, init=init, targets=targets, gates=gates,
                        ctor5_view=ctor_view, **outs)


def gen_fusion():
    spec = importlib.util.spec_from_file_location("ref_gate_fusion", os.path.join(REF, "python", "gate_fusion.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    G = m.GATES
    # benchmarks/benchmark_fusion.py:13-20 circuit shape, plus a mixed-target circuit
    circuit = []
    for _ in range(3):
        for q in range(6):
            for name in ("H", "X", "S", "T"):
                circuit.append((q, G[name]))
    rng = np.random.default_rng(5)
    names = list(G)
    mixed = [(int(rng.integers(3)), G[names[rng.integers(4)]]) for _ in range(60)]
    outs = {}
    for label, c in (("bench", circuit), ("mixed", mixed)):
        fused = m.GateFuser.fuse_circuit(c)
        outs[label + "_targets"] = np.array([t for t, _ in fused])
        outs[label + "_gates"] = np.array([np.asarray(g, dtype=np.complex128) for _, g in fused])
        outs[label + "_in_targets"] = np.array([t for t, _ in c])
        outs[label + "_in_gates"] = np.array([np.asarray(g, dtype=np.complex128) for _, g in c])
    np.savez_compressed(os.path.join(HERE, "gate_fusion.npz"), **outs)


def gen_grover(L):
    out = {}
    # README.md:509: n = 8, marked 85 -> 12 iterations, P = 0.99994704
    for label, n, marked, iters in (("n8_m85", 8, [85], -1), ("n10_i10", 10, [(1 << 10) // 3], 10),
                                    ("n12_i10", 12, [(1 << 12) // 3], 10)):
        probs = np.zeros(1 << n)
        mi, it = ctypes.c_int(), ctypes.c_int()
        m = np.array(marked, dtype=np.int32)
        rc = L.ref_grover(n, m.ctypes.data, m.size, iters, probs.ctypes.data, ctypes.byref(mi), ctypes.byref(it))
        assert rc == 0
        out[label + "_probs"] = probs
        out[label + "_marked_index"] = mi.value
        out[label + "_iterations"] = it.value
        out[label + "_marked"] = m
    np.savez_compressed(os.path.join(HERE, "grover.npz"), **out)


def ring_energy(state, n):
    p = np.abs(state) ** 2
    idx = np.arange(1 << n)
    e = 0.0
    for i in range(n):
        j = (i + 1) % n
        z = 1 - 2 * (((idx >> i) ^ (idx >> j)) & 1)
        e += float(np.dot(p, z))
    return e


def gen_vqe(L):
    # VQE::prepare (src/Algorithms.h:240-252) energies and parameter-shift gradients
    # (src/Algorithms.h:277-292) for the ring ZZ observable.
    out = {}
    rng = np.random.default_rng(11)
    for n, layers in ((4, 2), (6, 3)):
        theta = rng.uniform(-np.pi, np.pi, size=n * layers)

        def energy(th):
            st = np.zeros(1 << n, dtype=np.complex128)
            rc = L.ref_vqe_prepare(n, layers, np.ascontiguousarray(th).ctypes.data, st.ctypes.data)
            assert rc == 0
            return ring_energy(st, n), st

        e0, st0 = energy(theta)
        grad = np.zeros_like(theta)
        for k in range(theta.size):
            tp, tm = theta.copy(), theta.copy()
            tp[k] += PI / 2
            tm[k] -= PI / 2
            grad[k] = 0.5 * (energy(tp)[0] - energy(tm)[0])
        key = f"n{n}_l{layers}"
        out[key + "_theta"] = theta
        out[key + "_state"] = st0
        out[key + "_energy"] = e0
        out[key + "_grad"] = grad
    np.savez_compressed(os.path.join(HERE, "vqe_param_shift.npz"), **out)


def gen_hea(L):
    # config-3 ansatz (RY, RZ, CZ ring) at small n on ll::StateVectorBackend; gradient by the
    # reference's parameter-shift rule applied to each rotation.
    n, layers = 6, 2
    ops = workloads.hea_ansatz(n, layers)
    params = workloads.hea_params(n, layers, batch=2, seed=31)
    out = {"ops": ops, "params": params, "n": n, "layers": layers}
    energies, grads = [], []
    for b in range(params.shape[0]):
        def energy(p):
            return ring_energy(ref_state(L, 1, n, workloads.bind_params(ops, p)), n)

        e = energy(params[b])
        g = np.zeros(params.shape[1])
        for k in range(params.shape[1]):
            pp, pm = params[b].copy(), params[b].copy()
            pp[k] += PI / 2
            pm[k] -= PI / 2
            g[k] = 0.5 * (energy(pp) - energy(pm))
        energies.append(e)
        grads.append(g)
    out["energies"] = np.array(energies)
    out["grads"] = np.array(grads)
    np.savez_compressed(os.path.join(HERE, "hea_param_shift.npz"), **out)


def noise_circuits():
    """Our own seeded circuits for the NoisyBackend / ZNE fixtures: every gate kind the noise
    sites distinguish (1-qubit gates, cnot, 2-qubit cz, 1- and 3-qubit mcz)."""
    from llgpu import OP_CNOT, OP_CZ, OP_H, OP_MCZ, OP_RX, OP_RY, OP_RZ, OP_X, make_ops

    rng = np.random.default_rng(6060)
    recs = []
    for _ in range(5):
        recs += [(OP_H, int(rng.integers(3))), (OP_RY, int(rng.integers(3)), 0, float(rng.uniform(-3, 3))),
                 (OP_CNOT, 0, 2), (OP_RZ, 2, 0, float(rng.uniform(-3, 3))), (OP_CZ, 1, 2),
                 (OP_MCZ, 0, 0, 0.0, 0b111), (OP_X, 1), (OP_RX, 0, 0, float(rng.uniform(-3, 3))),
                 (OP_CNOT, 1, 0), (OP_MCZ, 0, 0, 0.0, 0b100)]
    three = make_ops(recs)
    one = make_ops([(OP_RY, 0, 0, 0.9), (OP_RZ, 0, 0, -0.6), (OP_RX, 0, 0, 0.35)])
    bell = make_ops([(OP_H, 0), (OP_CNOT, 0, 1)])
    return three, one, bell


def gen_noise(L):
    three, one, bell = noise_circuits()
    terms3 = (np.array([0, 2], dtype=np.int32), np.array([1, -1], dtype=np.int32), np.array([1.0, 0.5]))
    z0 = (np.array([0], dtype=np.int32), np.array([-1], dtype=np.int32), np.array([1.0]))
    zz = (np.array([0], dtype=np.int32), np.array([1], dtype=np.int32), np.array([1.0]))
    out = {"three_ops": three, "one_ops": one, "bell_ops": bell}

    def obs(ops, n, p, scale, seed, ntraj, terms):
        a, b, c = terms
        v = np.zeros(ntraj)
        rc = L.ref_noisy_obs(n, ops.ctypes.data, ops.size, p, scale, seed, ntraj, a.size, a.ctypes.data,
                             b.ctypes.data, c.ctypes.data, v.ctypes.data)
        assert rc == 0, rc
        return v

    def zne(ops, n, p, seed, scales, ntraj, terms):
        a, b, c = terms
        s = np.array(scales, dtype=np.float64)
        o = np.zeros(3 + 3 * s.size)
        rc = L.ref_zne(n, ops.ctypes.data if ops.size else None, ops.size, p, seed, s.ctypes.data, s.size, ntraj,
                       a.size, a.ctypes.data, b.ctypes.data, c.ctypes.data, o.ctypes.data)
        return rc, o

    # per-trajectory observables on one NoisyBackend (one mt19937_64 stream)
    out["obs3_p05_s1"] = obs(three, 3, 0.05, 1, 2024, 200, terms3)
    out["obs3_p05_s3"] = obs(three, 3, 0.05, 3, 2024, 200, terms3)
    out["obs3_p0_s5"] = obs(three, 3, 0.0, 5, 1, 3, terms3)
    # ZNE::extrapolate
    cases = {"zne3": (three, 3, 0.03, 77, [1, 3, 5], 300, terms3), "zne1": (one, 1, 0.02, 2024, [1, 3], 2000, z0),
             "zne_bell": (bell, 2, 0.03, 99, [1, 3], 1000, zz), "zne_p0": (three, 3, 0.0, 5, [1, 3, 5], 7, terms3),
             "zne_single": (one, 1, 0.02, 3, [1, 3], 1, z0)}
    for name, (ops, n, p, seed, scales, ntraj, terms) in cases.items():
        rc, o = zne(ops, n, p, seed, scales, ntraj, terms)
        assert rc == 0, (name, rc)
        out[name] = o
    # the contract: bad scales are invalid_argument (1); a circuit without gates is runtime_error (3)
    out["zne_rc_bad_scale"] = np.array(zne(one, 1, 0.02, 1, [1, 4], 10, z0)[0])
    out["zne_rc_no_gates"] = np.array(zne(one[:0], 1, 0.02, 1, [1, 3], 10, z0)[0])
    np.savez_compressed(os.path.join(HERE, "noisy_zne.npz"), **out)


def algorithm_cases():
    """QAOA graphs and VQE problems for the algorithm fixtures (shared with the tests)."""
    rng = np.random.default_rng(77)
    ring4 = (4, [(0, 1, 1.0), (1, 2, 1.0), (2, 3, 1.0), (3, 0, 1.0)])
    w6 = (6, [(i, j, float(np.round(rng.uniform(0.2, 2.0), 3))) for i in range(6) for j in range(i + 1, 6)
              if rng.uniform() < 0.6])
    w10 = (10, [(i, (i + 1) % 10, 1.0) for i in range(10)] + [(i, (i + 3) % 10, 0.5) for i in range(0, 10, 2)])
    qaoa = [("ring4_p1", ring4, [0.4], [0.3]), ("w6_p2", w6, [0.3, 0.7], [0.5, 0.2]),
            ("w10_p3", w10, [0.2, 0.5, 0.8], [0.6, 0.4, 0.1])]
    sk5 = [(i, j, float(np.round(rng.normal() / np.sqrt(5), 4))) for i in range(5) for j in range(i + 1, 5)]
    vqe = [("ring4_l2", 4, 2, 1, 12, 0.1, [(i, (i + 1) % 4, 1.0) for i in range(4)], []),
           ("sk5_l2", 5, 2, 7, 10, 0.05, sk5, [(i, 0.3 * (i - 2)) for i in range(5)])]
    return qaoa, vqe


def gen_algorithms(L):
    # Algorithms.h's QAOA::run (src/Algorithms.h:156-191) and VQE::optimize (:255-307) on
    # ll::StateVectorBackend, for the drop-in algorithms module on the GPU backend
    out = {}
    qaoa, vqe = algorithm_cases()
    for label, (n, edges), gammas, betas in qaoa:
        ei = np.array([e[0] for e in edges], dtype=np.int32)
        ej = np.array([e[1] for e in edges], dtype=np.int32)
        w = np.array([e[2] for e in edges], dtype=np.float64)
        g = np.array(gammas, dtype=np.float64)
        b = np.array(betas, dtype=np.float64)
        probs = np.zeros(1 << n)
        cut = ctypes.c_double()
        rc = L.ref_qaoa(n, ei.size, ei.ctypes.data, ej.ctypes.data, w.ctypes.data, g.size, g.ctypes.data,
                        b.ctypes.data, probs.ctypes.data, ctypes.byref(cut))
        assert rc == 0
        out[f"qaoa_{label}_probs"] = probs
        out[f"qaoa_{label}_best_cut"] = cut.value
    for label, n, layers, seed, iters, lr, zz, z in vqe:
        a = np.array([t[0] for t in zz] + [t[0] for t in z], dtype=np.int32)
        bb = np.array([t[1] for t in zz] + [-1] * len(z), dtype=np.int32)
        c = np.array([t[2] for t in zz] + [t[1] for t in z], dtype=np.float64)
        params = np.zeros(n * layers)
        probs = np.zeros(1 << n)
        e, it = ctypes.c_double(), ctypes.c_int()
        rc = L.ref_vqe_optimize(n, layers, seed, iters, lr, a.size, a.ctypes.data, bb.ctypes.data, c.ctypes.data,
                                ctypes.byref(e), params.ctypes.data, ctypes.byref(it), probs.ctypes.data)
        assert rc == 0
        out[f"vqe_{label}_energy"] = e.value
        out[f"vqe_{label}_params"] = params
        out[f"vqe_{label}_iterations"] = it.value
        out[f"vqe_{label}_probs"] = probs
    np.savez_compressed(os.path.join(HERE, "algorithms.npz"), **out)


def main():
    L, mods = load_ref()
    gen_random_2024(L)
    gen_config1(L)
    gen_config2(L)
    gen_v3(mods)
    gen_fusion()
    gen_grover(L)
    gen_vqe(L)
    gen_hea(L)
    gen_noise(L)
    gen_algorithms(L)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
