"""Seeded synthetic workloads for the five benchmark configurations (all inputs synthetic; the
reference publishes no dataset for this path).

Every generator returns gate records in the llg_op layout (see llgpu.OP_DTYPE), so the same op
list drives the GPU engine, the CPU oracle and the reference build.

1. `mixed_h_cnot`    -- n qubits from |0..0>, `n_ops` ops: H on a uniform qubit with p = 0.5,
                        else CNOT on a uniform distinct (control, target) pair (the published
                        1000-op Lightning-Lite vs Qiskit workload, docs/RESULTS.md:13-25).
2. `layered_rotations` -- `layers` layers of RX, RY, RZ on every qubit (angles U[0, 2pi)) then a
                        CNOT brickwork (i, i+1), even offsets on even layers, odd on odd layers.
3. `hea_ansatz`      -- hardware-efficient ansatz: per layer RY(theta_q) on every qubit, RZ(phi_q)
                        on every qubit, CZ ring (q, q+1 mod n); parameters indexed layer-major.
4. `noisy_layers`    -- `layers` layers of RX, RY (U[0, 2pi)) on every qubit + CNOT chain
                        (0,1)..(n-2,n-1); the trajectory workload.
5. `mixed_batch`     -- `count` circuits with n ~ U{lo..hi}, `depth` gates each, type uniform over
                        {H, RX, RY, RZ, CNOT, CZ}, angles U[0, 2pi), uniform (distinct) qubits.
"""
from __future__ import annotations

import numpy as np

from llgpu import OP_CNOT, OP_CZ, OP_DTYPE, OP_H, OP_RX, OP_RY, OP_RZ

TWO_PI = 2.0 * np.pi


def _ops(n: int) -> np.ndarray:
    ops = np.zeros(n, dtype=OP_DTYPE)
    ops["param"] = -1
    return ops


def mixed_h_cnot(n: int, n_ops: int = 1000, seed: int = 1234) -> np.ndarray:
    rng = np.random.default_rng(seed)
    ops = _ops(n_ops)
    for i in range(n_ops):
        if rng.random() < 0.5 or n < 2:
            ops[i]["kind"] = OP_H
            ops[i]["q0"] = rng.integers(n)
        else:
            c, t = rng.choice(n, size=2, replace=False)
            ops[i]["kind"] = OP_CNOT
            ops[i]["q0"] = c
            ops[i]["q1"] = t
    return ops


def layered_rotations(n: int, layers: int = 20, seed: int = 2030) -> np.ndarray:
    rng = np.random.default_rng(seed)
    recs = []
    for layer in range(layers):
        for q in range(n):
            for kind in (OP_RX, OP_RY, OP_RZ):
                recs.append((kind, q, 0, rng.uniform(0.0, TWO_PI)))
        for i in range(layer % 2, n - 1, 2):
            recs.append((OP_CNOT, i, i + 1, 0.0))
    ops = _ops(len(recs))
    for i, (k, a, b, t) in enumerate(recs):
        ops[i]["kind"], ops[i]["q0"], ops[i]["q1"], ops[i]["theta"] = k, a, b, t
    return ops


def hea_ansatz(n: int, layers: int = 10) -> np.ndarray:
    """Structure only; thetas come from the parameter vector (param index on every rotation)."""
    recs = []
    for layer in range(layers):
        for q in range(n):
            recs.append((OP_RY, q, 0, layer * 2 * n + q))
        for q in range(n):
            recs.append((OP_RZ, q, 0, layer * 2 * n + n + q))
        for q in range(n):
            if n > 1 and not (n == 2 and q == 1):
                recs.append((OP_CZ, q, (q + 1) % n, -1))
    ops = _ops(len(recs))
    for i, (k, a, b, p) in enumerate(recs):
        ops[i]["kind"], ops[i]["q0"], ops[i]["q1"], ops[i]["param"] = k, a, b, p
    return ops


def hea_params(n: int, layers: int = 10, batch: int = 64, seed: int = 3030) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.uniform(0.0, TWO_PI, size=(batch, layers * 2 * n))


def bind_params(ops: np.ndarray, params: np.ndarray) -> np.ndarray:
    out = ops.copy()
    sel = out["param"] >= 0
    out["theta"][sel] = params[out["param"][sel]]
    return out


def noisy_layers(n: int = 14, layers: int = 8, seed: int = 4040) -> np.ndarray:
    rng = np.random.default_rng(seed)
    recs = []
    for _ in range(layers):
        for q in range(n):
            recs.append((OP_RX, q, 0, rng.uniform(0.0, TWO_PI)))
            recs.append((OP_RY, q, 0, rng.uniform(0.0, TWO_PI)))
        for i in range(n - 1):
            recs.append((OP_CNOT, i, i + 1, 0.0))
    ops = _ops(len(recs))
    for i, (k, a, b, t) in enumerate(recs):
        ops[i]["kind"], ops[i]["q0"], ops[i]["q1"], ops[i]["theta"] = k, a, b, t
    return ops


def mixed_batch(count: int = 512, lo: int = 10, hi: int = 22, depth: int = 200, seed: int = 5050):
    """Returns (n_qubits[count] int32, ops concatenated, offsets[count + 1] int64)."""
    rng = np.random.default_rng(seed)
    kinds = (OP_H, OP_RX, OP_RY, OP_RZ, OP_CNOT, OP_CZ)
    nq = rng.integers(lo, hi + 1, size=count).astype(np.int32)
    ops = _ops(count * depth)
    for c in range(count):
        n = int(nq[c])
        for g in range(depth):
            r = ops[c * depth + g]
            k = kinds[rng.integers(len(kinds))]
            r["kind"] = k
            if k in (OP_CNOT, OP_CZ):
                a, b = rng.choice(n, size=2, replace=False)
                r["q0"], r["q1"] = a, b
            else:
                r["q0"] = rng.integers(n)
                if k != OP_H:
                    r["theta"] = rng.uniform(0.0, TWO_PI)
    offsets = np.arange(count + 1, dtype=np.int64) * depth
    return nq, ops, offsets
