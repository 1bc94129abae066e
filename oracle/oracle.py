"""ctypes loader for the ORACLE (oracle/_build/liboracle.so) -- test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs may import
this module; it is the checker, never the thing shipped or measured as the GPU path.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        import build_oracle  # noqa: E402  (same directory)

        path = build_oracle.build_oracle()
        L = ctypes.CDLL(path)
        vp, i, d, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_uint64
        P = ctypes.POINTER
        sigs = {
            "orc_set_threads": (None, [i]),
            "orc_max_threads": (i, []),
            "orc_init_zero": (None, [vp, i]),
            "orc_apply_gate_v3": (None, [vp, i, i, vp]),
            "orc_apply_gate_standard": (None, [vp, i, i, vp]),
            "orc_run_ops": (i, [vp, i, vp, i]),
            "orc_apply_op": (i, [vp, i, vp]),
            "orc_probabilities": (None, [vp, i, vp]),
            "orc_apply_matrix": (i, [vp, i, i, vp, vp]),
            "orc_expect_zz": (d, [vp, i, i, vp, vp, vp]),
            "orc_norm2": (d, [vp, i]),
            "orc_philox4x32_10": (None, [vp, vp, vp]),
            "orc_uniform_pair": (None, [u64, u64, u64, P(d), P(d)]),
            "orc_traj_run": (i, [i, vp, i, d, d, u64, u64, u64, vp, vp, vp, ctypes.c_int64, P(d)]),
            "orc_density_z0": (i, [i, vp, i, d, d, P(d)]),
            "orc_param_shift": (i, [i, vp, i, vp, i, i, vp, vp, vp, P(d), vp]),
            "orc_mt64_first": (u64, [u64, i]),
            "orc_noisy_run": (i, [i, vp, i, d, i, i, u64, u64, u64, i, vp, vp, vp, vp, vp]),
            "orc_richardson_weights": (i, [vp, i, vp]),
            "orc_zne": (i, [i, vp, i, d, vp, i, i, i, u64, i, vp, vp, vp, vp]),
            "orc_kraus_trace_preserving": (i, [i, vp, i, d]),
            "orc_kraus_apply": (i, [vp, i, i, vp, i, vp]),
            "orc_dm_apply_op": (i, [vp, i, vp]),
            "orc_expm": (i, [vp, i, vp]),
            "orc_tsolver_run": (i, [i, i, ctypes.c_longlong, d, i, vp, vp, i, vp, vp, vp, u64, u64, u64, vp]),
            "orc_lindblad_exact": (i, [i, vp, i, vp, vp, vp, d, i, vp]),
        }
        for name, (res, args) in sigs.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


def set_threads(t: int) -> None:
    lib().orc_set_threads(int(t))


def max_threads() -> int:
    return lib().orc_max_threads()


def zero_state(n: int) -> np.ndarray:
    s = np.zeros(1 << n, dtype=np.complex128)
    s[0] = 1.0
    return s


def run_ops(n: int, ops: np.ndarray, state: np.ndarray | None = None) -> np.ndarray:
    psi = zero_state(n) if state is None else np.array(state, dtype=np.complex128, copy=True)
    ops = np.ascontiguousarray(ops)
    rc = lib().orc_run_ops(_p(psi), n, _p(ops) if ops.size else None, ops.size)
    if rc:
        raise ValueError(f"oracle rejected the op list (rc={rc})")
    return psi


def apply_gate_v3(psi: np.ndarray, n: int, target: int, gate) -> None:
    g = np.asarray(gate, dtype=np.complex128).reshape(4)
    buf = np.ascontiguousarray(np.stack([g.real, g.imag], axis=1).reshape(8))
    lib().orc_apply_gate_v3(_p(psi), n, target, _p(buf))


def apply_gate_standard(psi: np.ndarray, n: int, target: int, gate) -> None:
    g = np.asarray(gate, dtype=np.complex128).reshape(4)
    buf = np.ascontiguousarray(np.stack([g.real, g.imag], axis=1).reshape(8))
    lib().orc_apply_gate_standard(_p(psi), n, target, _p(buf))


def probabilities(psi: np.ndarray, n: int) -> np.ndarray:
    out = np.empty(1 << n, dtype=np.float64)
    lib().orc_probabilities(_p(psi), n, _p(out))
    return out


def apply_matrix(psi: np.ndarray, n: int, qubits, m: np.ndarray) -> None:
    qs = np.ascontiguousarray(qubits, dtype=np.int32)
    mm = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
    rc = lib().orc_apply_matrix(_p(psi), n, qs.size, _p(qs), _p(mm))
    if rc:
        raise ValueError("oracle apply_matrix rejected its arguments")


def expect_zz(psi: np.ndarray, n: int, a, b, coeff) -> float:
    aa = np.ascontiguousarray(a, dtype=np.int32)
    bb = np.ascontiguousarray(b, dtype=np.int32)
    cc = np.ascontiguousarray(coeff, dtype=np.float64)
    return lib().orc_expect_zz(_p(psi), n, aa.size, _p(aa), _p(bb), _p(cc))


def philox(ctr, key) -> np.ndarray:
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(_p(c), _p(k), _p(out))
    return out


def uniform_pair(seed: int, traj: int, site: int) -> tuple[float, float]:
    u1, u2 = ctypes.c_double(), ctypes.c_double()
    lib().orc_uniform_pair(seed, traj, site, ctypes.byref(u1), ctypes.byref(u2))
    return u1.value, u2.value


def traj_run(n: int, ops: np.ndarray, gamma: float, lam: float, seed: int, begin: int, end: int,
             log_sites: int = 0):
    """Returns (z0[end-begin], jumps[end-begin], log or None, min margin)."""
    cnt = end - begin
    z0 = np.zeros(cnt, dtype=np.float64)
    jumps = np.zeros(cnt, dtype=np.uint32)
    log = np.zeros((cnt, log_sites), dtype=np.uint8) if log_sites else None
    margin = ctypes.c_double()
    ops = np.ascontiguousarray(ops)
    rc = lib().orc_traj_run(n, _p(ops), ops.size, gamma, lam, seed, begin, end, _p(z0), _p(jumps),
                            _p(log) if log is not None else None, log_sites, ctypes.byref(margin))
    if rc:
        raise ValueError(f"oracle trajectory run failed (rc={rc})")
    return z0, jumps, log, margin.value


def density_z0(n: int, ops: np.ndarray, gamma: float, lam: float) -> float:
    out = ctypes.c_double()
    ops = np.ascontiguousarray(ops)
    rc = lib().orc_density_z0(n, _p(ops), ops.size, gamma, lam, ctypes.byref(out))
    if rc:
        raise ValueError("oracle density evolution failed")
    return out.value


def param_shift(n: int, ops: np.ndarray, params: np.ndarray, a, b, coeff):
    """(energy, gradient) by the parameter-shift rule on the oracle state vector."""
    ops = np.ascontiguousarray(ops)
    pr = np.ascontiguousarray(params, dtype=np.float64)
    aa = np.ascontiguousarray(a, dtype=np.int32)
    bb = np.ascontiguousarray(b, dtype=np.int32)
    cc = np.ascontiguousarray(coeff, dtype=np.float64)
    e = ctypes.c_double()
    g = np.zeros(pr.size, dtype=np.float64)
    rc = lib().orc_param_shift(n, _p(ops), ops.size, _p(pr), pr.size, aa.size, _p(aa), _p(bb), _p(cc),
                               ctypes.byref(e), _p(g))
    if rc:
        raise ValueError(f"oracle parameter shift failed (rc={rc})")
    return e.value, g


RNG_PHILOX, RNG_MT = 0, 1


def _terms(terms):
    """[(a, b, coeff), ...] (b = -1: Z_a alone) -> int32 / int32 / float64 arrays."""
    terms = list(terms) or [(0, -1, 1.0)]
    a = np.ascontiguousarray([t[0] for t in terms], dtype=np.int32)
    b = np.ascontiguousarray([t[1] for t in terms], dtype=np.int32)
    c = np.ascontiguousarray([t[2] for t in terms], dtype=np.float64)
    return a, b, c


def noisy_run(n: int, ops: np.ndarray, p: float, scale: int, seed: int, begin: int, end: int, terms=(),
              rng: int = RNG_PHILOX):
    """Observable per trajectory and non-identity Pauli count per trajectory of the folded
    depolarizing-noise circuit (NoisyBackend restatement)."""
    ops = np.ascontiguousarray(ops)
    a, b, c = _terms(terms)
    obs = np.zeros(end - begin)
    paulis = np.zeros(end - begin, dtype=np.uint32)
    rc = lib().orc_noisy_run(n, _p(ops), ops.size, p, scale, rng, seed, begin, end, a.size, _p(a), _p(b), _p(c),
                             _p(obs), _p(paulis))
    if rc:
        raise ValueError(f"oracle noisy run failed (rc={rc})")
    return obs, paulis


def richardson_weights(scales) -> np.ndarray:
    s = np.ascontiguousarray(scales, dtype=np.float64)
    w = np.zeros(s.size)
    if lib().orc_richardson_weights(_p(s), s.size, _p(w)):
        raise ValueError("bad scales")
    return w


def zne(n: int, ops: np.ndarray, p: float, scales, trajectories: int, seed: int, terms=(), rng: int = RNG_PHILOX):
    """ZNE::extrapolate restatement: dict(value, std_error, trajectories, values, std_errors,
    weights).  Raises ValueError (bad arguments) or RuntimeError (no gates)."""
    ops = np.ascontiguousarray(ops)
    s = np.ascontiguousarray(scales, dtype=np.float64)
    a, b, c = _terms(terms)
    ns = s.size
    out = np.zeros(4 * ns + 3)
    rc = lib().orc_zne(n, _p(ops) if ops.size else None, ops.size, p, _p(s), ns, trajectories, rng, seed, a.size,
                       _p(a), _p(b), _p(c), _p(out))
    if rc == 3:
        raise RuntimeError("circuit applied no gates")
    if rc:
        raise ValueError(f"oracle zne failed (rc={rc})")
    return {"value": out[0], "std_error": out[1], "trajectories": int(out[2]), "values": out[3:3 + ns],
            "std_errors": out[3 + ns:3 + 2 * ns], "weights": out[3 + 2 * ns:3 + 3 * ns]}


def dm_zero(n: int) -> np.ndarray:
    """|0..0><0..0| as a dim x dim complex matrix (row, col)."""
    rho = np.zeros((1 << n, 1 << n), dtype=np.complex128)
    rho[0, 0] = 1.0
    return rho


def _dm_buf(rho: np.ndarray) -> np.ndarray:
    # element (row, col) at row + col * dim: the column-major order of the matrix
    return np.ascontiguousarray(rho.T)


def kraus_apply(rho: np.ndarray, n: int, ops, targets) -> np.ndarray:
    """KrausChannel::apply restatement: sum_k K rho K^+ on `targets` (bit j of K's index is
    targets[j])."""
    buf = _dm_buf(rho)
    kk = np.ascontiguousarray(np.asarray(ops, dtype=np.complex128))
    tg = np.ascontiguousarray(targets, dtype=np.int32)
    rc = lib().orc_kraus_apply(_p(buf), n, kk.shape[0], _p(kk), tg.size, _p(tg))
    if rc:
        raise ValueError("oracle kraus_apply rejected its arguments")
    return np.ascontiguousarray(buf.T)


def kraus_trace_preserving(ops, tol: float = 1e-10) -> bool:
    kk = np.ascontiguousarray(np.asarray(ops, dtype=np.complex128))
    m = int(np.log2(kk.shape[1]))
    return bool(lib().orc_kraus_trace_preserving(kk.shape[0], _p(kk), m, tol))


def dm_apply_ops(rho: np.ndarray, n: int, ops: np.ndarray) -> np.ndarray:
    buf = _dm_buf(rho)
    for op in np.ascontiguousarray(ops):
        one = np.ascontiguousarray(np.array([op]))
        if lib().orc_dm_apply_op(_p(buf), n, _p(one)):
            raise ValueError("oracle dm_apply_op rejected an op")
    return np.ascontiguousarray(buf.T)


def expm(a: np.ndarray) -> np.ndarray:
    """exp(A): the reference's scaling and squaring with an 18-term Taylor series."""
    a = np.ascontiguousarray(np.asarray(a, dtype=np.complex128))
    out = np.zeros_like(a)
    if lib().orc_expm(_p(a), a.shape[0], _p(out)):
        raise MemoryError("oracle expm")
    return out


def pauli_like(l: np.ndarray):
    """(True, P, c) when L is Hermitian with L^2 = c 1, c > 1e-12 (src/TrajectorySolver.h:363-373)."""
    if np.linalg.norm(l - l.conj().T) > 1e-9 * max(1.0, np.linalg.norm(l)):
        return False, None, 0.0
    l2 = l @ l
    c = l2[0, 0].real
    if not c > 1e-12 or np.linalg.norm(l2 - c * np.eye(l.shape[0])) > 1e-9 * max(1.0, np.linalg.norm(l2)):
        return False, None, 0.0
    return True, l / np.sqrt(c), c


def tsolver_plan(h, channels, kind: int, duration: float, dt: float, h_fn=None) -> dict:
    """The reference's make_plan (src/TrajectorySolver.h:400-441): channels [(L, gamma), ...],
    kind 0 STANDARD, 1 PROJECTOR, 2 ANALOG."""
    d = (h_fn(0.0) if h_fn is not None else h).shape[0]
    if not channels:
        kind = 0
    steps = max(1, int(np.ceil(duration / dt - 1e-9)))
    hh = duration / steps
    ops = []
    for l, gamma in channels:
        pl, pm, c = pauli_like(np.asarray(l, dtype=complex))
        if kind == 1 and pl:
            ops.append(np.sqrt(gamma * c) * (np.eye(d) - pm))
        else:
            ops.append(np.sqrt(gamma) * np.asarray(l, dtype=complex))
    dop = [j.conj().T @ j for j in ops]
    hnh = np.zeros((d, d), dtype=complex)
    if kind != 2:
        for m in dop:
            hnh -= 0.5j * m
    plan = {"steps": steps, "h": hh, "kind": kind, "ops": ops, "ops_dop": dop, "constant": h_fn is None}
    if h_fn is None:
        plan["prop"] = expm(-1j * (h + hnh) * hh)
        plan["nodes"] = []
    else:
        n_nodes = 2 * steps + 1 if kind != 2 else steps
        plan["prop"] = None
        plan["nodes"] = [-1j * (h_fn(0.5 * hh * j if kind != 2 else hh * j) + hnh) for j in range(n_nodes)]
    return plan


def tsolver_run(plan: dict, psi0, seed: int, begin: int, end: int) -> np.ndarray:
    """Trajectory states [end - begin, dim] for a plan (tsolver_plan's or the engine's export)."""
    d = np.asarray(psi0).size
    p0 = np.ascontiguousarray(np.asarray(psi0, dtype=np.complex128) / np.linalg.norm(psi0))
    ops = np.ascontiguousarray(np.array(plan["ops"], dtype=np.complex128).reshape(-1, d, d)) if len(plan["ops"]) else \
        np.zeros((1, d, d), dtype=np.complex128)
    dop = np.ascontiguousarray(np.array(plan["ops_dop"], dtype=np.complex128).reshape(-1, d, d)) if len(plan["ops"]) else ops
    prop = np.ascontiguousarray(plan["prop"] if plan["prop"] is not None else np.eye(d), dtype=np.complex128)
    nodes = np.ascontiguousarray(np.array(plan["nodes"], dtype=np.complex128)) if len(plan["nodes"]) else prop
    out = np.zeros((end - begin, d), dtype=np.complex128)
    rc = lib().orc_tsolver_run(d, int(plan["kind"]), int(plan["steps"]), float(plan["h"]), int(bool(plan["constant"])),
                               _p(prop), _p(nodes), len(plan["ops"]), _p(ops), _p(dop), _p(p0), seed, begin, end,
                               _p(out))
    if rc:
        raise RuntimeError(f"oracle trajectory solver failed (rc={rc})")
    return out


def lindblad_exact(h, channels, rho0, duration: float, steps: int) -> np.ndarray:
    """RK4 on the Lindblad equation for constant H (the reference's own check)."""
    d = h.shape[0]
    hh = np.ascontiguousarray(h, dtype=np.complex128)
    ls = np.ascontiguousarray(np.array([c[0] for c in channels], dtype=np.complex128).reshape(-1, d, d))
    gs = np.ascontiguousarray([c[1] for c in channels], dtype=np.float64)
    r0 = np.ascontiguousarray(rho0, dtype=np.complex128)
    out = np.zeros_like(r0)
    lib().orc_lindblad_exact(d, _p(hh), len(channels), _p(ls), _p(gs), _p(r0), duration, steps, _p(out))
    return out


def fuse_gate_list(n: int, ops: np.ndarray):
    """The reference's own fused CPU path for an op list: runs of consecutive single-qubit gates
    on one target merged into one 2x2, the later gate on the left (GateFuser.fuse_circuit,
    python/gate_fusion.py:15-37, as benchmarks/benchmark_fusion.py:36-50 feeds it to
    apply_gate_cache_optimized); CNOT / CZ / MCZ records stay as they are and end a run.
    Returns a list of ("u2", target, 2x2 matrix) and ("op", record) items."""
    out = []
    for op in ops:
        k = int(op["kind"])
        if k in (0, 1, 2, 3, 4, 8):  # H, X, RX, RY, RZ, U2
            m = _op_matrix(op)
            q = int(op["q0"])
            if out and out[-1][0] == "u2" and out[-1][1] == q:
                out[-1] = ("u2", q, m @ out[-1][2])
            else:
                out.append(("u2", q, m))
        else:
            out.append(("op", op))
    return out


def _op_matrix(op) -> np.ndarray:
    k, t = int(op["kind"]), float(op["theta"])
    c, s = np.cos(0.5 * t), np.sin(0.5 * t)
    r = 1.0 / np.sqrt(2.0)
    if k == 0:
        return np.array([[r, r], [r, -r]], dtype=complex)
    if k == 1:
        return np.array([[0, 1], [1, 0]], dtype=complex)
    if k == 2:
        return np.array([[c, -1j * s], [-1j * s, c]])
    if k == 3:
        return np.array([[c, -s], [s, c]], dtype=complex)
    if k == 4:
        return np.diag([np.exp(-0.5j * t), np.exp(0.5j * t)])
    return np.asarray(op["m"], dtype=np.float64).view(np.complex128).reshape(2, 2)
