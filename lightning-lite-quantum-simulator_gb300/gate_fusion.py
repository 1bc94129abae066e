"""Gate fusion front end with the reference's API (python/gate_fusion.py).

``GateFuser.fuse_circuit`` merges runs of consecutive single-qubit gates on the same target into
one 2x2 matrix, the later gate multiplied on the left (g2 @ g1), exactly the reference rule
(python/gate_fusion.py:7-37); its output list of ``(target, [g00, g01, g10, g11])`` feeds
``StateVector.apply_gate_cache_optimized`` or ``StateVector.apply_fused``.

On the GPU engine this front-end fusion is optional: every StateVector queues its gates and, at
flush time, the native planner (csrc/llg_plan.cpp) fuses them much further -- any gates whose
qubits fit one shared-memory tile run in a single HBM pass.
"""
from __future__ import annotations

import numpy as np


class GateFuser:
    """Pre-processor that fuses sequential gates on the same qubit."""

    @staticmethod
    def multiply_gates(gate1, gate2):
        """2x2 product for `gate1` followed by `gate2`: returns flat(gate2 @ gate1) as a list."""
        a = np.asarray(gate1, dtype=np.complex128).reshape(2, 2)
        b = np.asarray(gate2, dtype=np.complex128).reshape(2, 2)
        return (b @ a).reshape(4).tolist()

    @staticmethod
    def fuse_circuit(gates):
        """gates: list of (target_qubit, gate_matrix); returns the fused list."""
        out = []
        for target, gate in gates:
            if out and out[-1][0] == target:
                out[-1] = (target, GateFuser.multiply_gates(out[-1][1], gate))
            else:
                out.append((target, gate))
        return out

    @staticmethod
    def analyze_circuit(gates):
        """Print before/after counts and return the fused list."""
        fused = GateFuser.fuse_circuit(gates)
        before, after = len(gates), len(fused)
        print(f"Original gates: {before}")
        print(f"After fusion: {after}")
        print(f"Reduction: {(1 - after / before) * 100:.1f}%")
        return fused


_r = 1.0 / np.sqrt(2.0)
GATES = {
    "X": [0j, 1 + 0j, 1 + 0j, 0j],
    "H": [_r + 0j, _r + 0j, _r + 0j, -_r + 0j],
    "S": [1 + 0j, 0j, 0j, 1j],
    "T": [1 + 0j, 0j, 0j, complex(np.exp(1j * np.pi / 4))],
}
