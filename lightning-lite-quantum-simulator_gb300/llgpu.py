"""ctypes binding of libllgpu.so's C ABI (include/llgpu.h).

This is the plain-C view of the engine: the same entry points a cgo/JNI/ctypes caller of the C
ABI binds.  The pybind11 modules ``quantum_sim_v3`` / ``quantum_sim_v2`` are the reference-
compatible Python API; this module exists for callers (and tests) that want the C ABI itself,
and for the batched forms (adjoint gradients, trajectories, mixed-size batches).

Loading fails loudly if the shared library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from typing import Iterable, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libllgpu.so")

# status codes / enums (include/llgpu.h)
LLG_OK, LLG_EINVAL, LLG_ERUNTIME, LLG_ENOMEM, LLG_ECUDA, LLG_ETIMEOUT = range(6)
LLG_F64, LLG_DF64, LLG_F32 = 0, 1, 2
LLG_FUSE_NONE, LLG_FUSE_TILE, LLG_FUSE_REG = 0, 1, 2
FUSE_MODES = {"none": LLG_FUSE_NONE, "tile": LLG_FUSE_TILE, "reg": LLG_FUSE_REG}
FUSE_NAMES = {v: k for k, v in FUSE_MODES.items()}
OP_H, OP_X, OP_RX, OP_RY, OP_RZ, OP_CNOT, OP_MCZ, OP_CZ, OP_U2 = range(9)

PROF_CLASSES = 4
PROF_NAMES = ("tile", "gate", "init", "readout")

# "complex128" is the reference's arithmetic: IEEE binary64 (LLG_F64).  "df64" keeps each real part as an
# fp32 pair (about 48 significant bits, faster on this GPU's FP32 pipe); "complex64" is FP32.
PRECISIONS = {"complex128": LLG_F64, "fp64": LLG_F64, "f64": LLG_F64, "df64": LLG_DF64, "complex64": LLG_F32}

# numpy view of llg_op (96 bytes)
OP_DTYPE = np.dtype([
    ("kind", np.int32), ("q0", np.int32), ("q1", np.int32), ("param", np.int32),
    ("mask", np.uint64), ("theta", np.float64), ("m", np.float64, (8,)),
])
assert OP_DTYPE.itemsize == 96

PASS_DTYPE = np.dtype([("local_mask", np.uint64), ("t", np.int32), ("low", np.int32),
                       ("op_begin", np.int32), ("nops", np.int32)])
XOP_DTYPE = np.dtype([("kind", np.int32), ("q0", np.int32), ("q1", np.int32), ("flags", np.int32),
                      ("mask", np.uint64), ("nl_mask", np.uint64), ("c", np.float64, (8,))])


class LLGError(RuntimeError):
    pass


TUNE_AUTO = -1
TUNE_DTYPE = np.dtype([("fuse_mode", np.int32), ("tile_qubits", np.int32), ("cta_threads", np.int32),
                       ("cluster", np.int32), ("candidates", np.int32), ("cached", np.int32),
                       ("best_ms", np.float64), ("default_ms", np.float64)])


def _tune_dict(r: np.ndarray) -> dict:
    return {k: (float(r[k][0]) if r.dtype[k].kind == "f" else int(r[k][0])) for k in r.dtype.names}


def tune_cache_clear() -> None:
    lib().llg_tune_cache_clear()


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is not built; run build_ext.py (there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        vp, i, d, u64, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_uint64, ctypes.c_size_t
        P = ctypes.POINTER
        sigs = {
            "llg_last_error": (ctypes.c_char_p, []),
            "llg_version": (ctypes.c_char_p, []),
            "llg_device_count": (i, []),
            "llg_create": (i, [i, i, P(vp)]),
            "llg_create_from_host": (i, [vp, sz, i, P(vp)]),
            "llg_destroy": (i, [vp]),
            "llg_reset": (i, [vp, i]),
            "llg_num_qubits": (i, [vp, P(i)]),
            "llg_size": (i, [vp, P(u64)]),
            "llg_get_precision": (i, [vp, P(i)]),
            "llg_set_fusion": (i, [vp, i, i]),
            "llg_apply_gate": (i, [vp, i, vp]),
            "llg_h": (i, [vp, i]),
            "llg_x": (i, [vp, i]),
            "llg_rx": (i, [vp, i, d]),
            "llg_ry": (i, [vp, i, d]),
            "llg_rz": (i, [vp, i, d]),
            "llg_cnot": (i, [vp, i, i]),
            "llg_cz": (i, [vp, i, i]),
            "llg_mcz": (i, [vp, vp, i]),
            "llg_apply_ops": (i, [vp, vp, i]),
            "llg_apply_matrix": (i, [vp, i, vp, vp]),
            "llg_wrap_host": (i, [vp, sz, i, P(vp)]),
            "llg_apply_1q": (i, [vp, i, vp]),
            "llg_apply_block": (i, [vp, i, vp, vp]),
            "llg_expect_diag_zz": (i, [vp, i, vp, vp, vp, P(d)]),
            "llg_flush": (i, [vp]),
            "llg_sync": (i, [vp]),
            "llg_copy_to_host": (i, [vp, vp]),
            "llg_copy_from_host": (i, [vp, vp]),
            "llg_probabilities": (i, [vp, vp]),
            "llg_norm2": (i, [vp, P(d)]),
            "llg_expect_zz": (i, [vp, i, vp, vp, vp, P(d)]),
            "llg_expect_diagonal": (i, [vp, vp, i, P(d)]),
            "llg_diag_export": (i, [i, i, vp, vp, vp, vp]),
            "llg_renormalize": (i, [vp]),
            "llg_host_alloc": (vp, [sz]),
            "llg_host_free": (None, [vp]),
            "llg_plan_export": (i, [i, vp, i, i, vp, i, P(i), vp, i, P(i)]),
            "llg_plan_export_ex": (i, [i, vp, i, i, i, vp, i, P(i), vp, i, P(i)]),
            "llg_plan_export_tables": (i, [i, vp, i, i, i, vp, ctypes.c_int64, P(ctypes.c_int64)]),
            "llg_profile": (i, [vp, i]),
            "llg_profile_read": (i, [vp, vp, vp, i]),
            "llg_kernel_launches": (ctypes.c_int64, []),
            "llg_fp64_fma_rate": (i, [i, P(d)]),
            "llg_get_stream": (i, [vp, P(vp)]),
            "llg_expect_zz_noalloc": (i, [vp, i, i, i, vp, vp, vp, vp, vp]),
            "llg_adjoint_create": (i, [i, vp, i, i, i, i, i, vp, vp, vp, P(vp)]),
            "llg_adjoint_destroy": (i, [vp]),
            "llg_adjoint_info": (i, [vp, P(i), P(i), P(i)]),
            "llg_adjoint_run": (i, [vp, vp, i, vp, vp, i]),
            "llg_param_shift_run": (i, [vp, vp, i, vp, vp]),
            "llg_adjoint_stream": (i, [vp, P(vp)]),
            "llg_adjoint_set_threads": (i, [vp, i]),
            "llg_traj_run": (i, [i, vp, i, d, d, u64, u64, u64, i, vp, vp, vp, ctypes.c_int64, P(d)]),
            "llg_batch_create": (i, [i, vp, vp, vp, i, i, P(vp)]),
            "llg_batch_destroy": (i, [vp]),
            "llg_batch_info": (i, [vp, P(ctypes.c_int64), P(ctypes.c_int64), P(i)]),
            "llg_batch_run": (i, [vp, ctypes.c_int64]),
            "llg_batch_debug_block_item": (i, [vp, ctypes.c_int64]),
            "llg_batch_copy_state": (i, [vp, i, vp]),
            "llg_batch_fidelity": (i, [vp, vp, vp]),
            "llg_batch_stream": (i, [vp, P(vp)]),
            "llg_batch_autotune": (i, [i, vp, vp, vp, i, vp]),
            "llg_batch_config": (i, [vp, P(i), P(i), P(i)]),
            "llg_set_tile_threads": (i, [vp, i]),
            "llg_compare": (i, [vp, vp, P(d), P(d)]),
            "llg_compare_ex": (i, [vp, vp, P(d), P(d), P(d)]),
            "llg_get_tuning": (i, [vp, P(i), P(i), P(i)]),
            "llg_autotune": (i, [vp, vp, i, i, vp]),
            "llg_tune_cache_clear": (None, []),
            "llg_traj_create": (i, [i, vp, i, d, d, i, u64, i, i, P(vp)]),
            "llg_traj_destroy": (i, [vp]),
            "llg_traj_launch": (i, [vp, u64, u64, u64, vp, vp, P(d)]),
            "llg_traj_autotune": (i, [vp, u64, vp]),
            "llg_traj_config": (i, [vp, P(i), P(i), P(i), P(ctypes.c_int64)]),
            "llg_traj_stream": (i, [vp, P(vp)]),
            "llg_noisy_create": (i, [i, vp, i, d, i, i, u64, i, vp, vp, vp, i, i, P(vp)]),
            "llg_dm_apply_op": (i, [vp, i, vp]),
            "llg_tsolver_create": (i, [i, P(vp)]),
            "llg_tsolver_destroy": (i, [vp]),
            "llg_tsolver_set_hamiltonian": (i, [vp, vp]),
            "llg_tsolver_set_hamiltonian_fn": (i, [vp, vp, vp]),
            "llg_tsolver_add_lindblad": (i, [vp, vp, d]),
            "llg_tsolver_clear_lindblad": (i, [vp]),
            "llg_tsolver_info": (i, [vp, P(i), P(i)]),
            "llg_tsolver_projector_applies": (i, [vp, i, P(i)]),
            "llg_tsolver_run": (i, [vp, vp, d, d, ctypes.c_int64, i, u64, vp, vp, vp, vp]),
            "llg_tsolver_plan_export": (i, [vp, P(ctypes.c_longlong), P(d), P(i), P(i), vp, vp, ctypes.c_int64, vp,
                                            vp, P(i), P(ctypes.c_int64)]),
            "llg_dm_apply_kraus": (i, [vp, i, i, vp, i, vp]),
            "llg_richardson_weights": (i, [vp, i, vp]),
            "llg_zne_run": (i, [i, vp, i, d, i, vp, i, ctypes.c_int64, u64, i, vp, vp, vp, vp]),
        }
        for name, (res, args) in sigs.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    return lib().llg_last_error().decode()


def check(rc: int) -> None:
    if rc == LLG_OK:
        return
    msg = last_error()
    if rc == LLG_EINVAL:
        raise ValueError(msg)
    if rc == LLG_ENOMEM:
        raise MemoryError(msg)
    raise LLGError(f"[{rc}] {msg}")


def device_count() -> int:
    return lib().llg_device_count()


def kernel_launches() -> int:
    return int(lib().llg_kernel_launches())


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


# ---------------------------------------------------------------------------------------------
# gate records
# ---------------------------------------------------------------------------------------------
def make_ops(records: Iterable[tuple]) -> np.ndarray:
    """Build an llg_op array from tuples (kind, q0, q1, theta[, mask[, m[, param]]])."""
    recs = list(records)
    ops = np.zeros(len(recs), dtype=OP_DTYPE)
    ops["param"] = -1
    for i, r in enumerate(recs):
        ops[i]["kind"] = r[0]
        ops[i]["q0"] = r[1]
        ops[i]["q1"] = r[2] if len(r) > 2 else 0
        ops[i]["theta"] = r[3] if len(r) > 3 else 0.0
        if len(r) > 4 and r[4] is not None:
            ops[i]["mask"] = r[4]
        if len(r) > 5 and r[5] is not None:
            g = np.asarray(r[5], dtype=np.complex128).reshape(4)
            ops[i]["m"] = np.stack([g.real, g.imag], axis=1).reshape(8)
        if len(r) > 6 and r[6] is not None:
            ops[i]["param"] = r[6]
    return ops


def ops_from_fused(fused: Sequence[tuple]) -> np.ndarray:
    """GateFuser output [(target, [g00, g01, g10, g11]), ...] -> U2 records."""
    return make_ops([(OP_U2, int(t), 0, 0.0, None, g) for t, g in fused])


# ---------------------------------------------------------------------------------------------
# State: thin object over llg_state*
# ---------------------------------------------------------------------------------------------
class State:
    def __init__(self, n: int | None = None, precision: str = "complex128", amps: np.ndarray | None = None):
        L = lib()
        self._h = ctypes.c_void_p()
        p = PRECISIONS[precision]
        if amps is not None:
            a = np.ascontiguousarray(amps, dtype=np.complex128)
            check(L.llg_create_from_host(_ptr(a), a.size, p, ctypes.byref(self._h)))
        else:
            check(L.llg_create(int(n), p, ctypes.byref(self._h)))

    def close(self) -> None:
        if self._h:
            lib().llg_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    @property
    def n(self) -> int:
        v = ctypes.c_int()
        check(lib().llg_num_qubits(self._h, ctypes.byref(v)))
        return v.value

    @property
    def size(self) -> int:
        v = ctypes.c_uint64()
        check(lib().llg_size(self._h, ctypes.byref(v)))
        return v.value

    def set_fusion(self, mode: str = "tile", tile_qubits: int = 0) -> None:
        """mode: "tile" (shared-memory tile passes), "reg" (register-tiled passes, complex64) or
        "none" (one streaming kernel per gate)."""
        if mode not in FUSE_MODES:
            raise ValueError("fusion mode must be 'tile', 'reg' or 'none'")
        check(lib().llg_set_fusion(self._h, FUSE_MODES[mode], tile_qubits))

    def set_tile_threads(self, threads: int) -> None:
        check(lib().llg_set_tile_threads(self._h, threads))

    def tuning(self) -> dict:
        m, t, th = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().llg_get_tuning(self._h, ctypes.byref(m), ctypes.byref(t), ctypes.byref(th)))
        return {"fuse_mode": FUSE_NAMES.get(m.value, "none"), "tile_qubits": t.value, "cta_threads": th.value}

    def autotune(self, ops: np.ndarray, sample_ops: int = 0) -> dict:
        """Time candidate (fusion mode, tile width, CTA threads) settings on a scratch state with
        ops[:sample_ops] and keep the fastest for this state."""
        ops = np.ascontiguousarray(ops, dtype=OP_DTYPE)
        r = np.zeros(1, dtype=TUNE_DTYPE)
        check(lib().llg_autotune(self._h, _ptr(ops) if ops.size else None, ops.size, sample_ops, _ptr(r)))
        return _tune_dict(r)

    def apply_gate(self, target: int, gate) -> None:
        g = np.asarray(gate, dtype=np.complex128).reshape(4)
        buf = np.ascontiguousarray(np.stack([g.real, g.imag], axis=1).reshape(8))
        check(lib().llg_apply_gate(self._h, target, _ptr(buf)))

    def h(self, q): check(lib().llg_h(self._h, q))
    def x(self, q): check(lib().llg_x(self._h, q))
    def rx(self, q, t): check(lib().llg_rx(self._h, q, t))
    def ry(self, q, t): check(lib().llg_ry(self._h, q, t))
    def rz(self, q, t): check(lib().llg_rz(self._h, q, t))
    def cnot(self, c, t): check(lib().llg_cnot(self._h, c, t))
    def cz(self, a, b): check(lib().llg_cz(self._h, a, b))

    def mcz(self, qubits: Sequence[int]) -> None:
        q = np.ascontiguousarray(qubits, dtype=np.int32)
        check(lib().llg_mcz(self._h, _ptr(q) if q.size else None, q.size))

    def apply_ops(self, ops: np.ndarray) -> None:
        ops = np.ascontiguousarray(ops, dtype=OP_DTYPE)
        check(lib().llg_apply_ops(self._h, _ptr(ops) if ops.size else None, ops.size))

    def apply_matrix(self, qubits: Sequence[int], m) -> None:
        """Dense 2^k x 2^k complex block on `qubits` (k <= 5); bit j of the block's row / column
        index is qubits[j]."""
        qs = np.ascontiguousarray(qubits, dtype=np.int32)
        mm = np.ascontiguousarray(np.asarray(m, dtype=np.complex128).reshape(-1))
        if mm.size != (1 << (2 * qs.size)):
            raise ValueError("apply_matrix: matrix must be 2^k x 2^k for k qubits")
        check(lib().llg_apply_matrix(self._h, qs.size, _ptr(qs), _ptr(mm)))

    def flush(self): check(lib().llg_flush(self._h))
    def sync(self): check(lib().llg_sync(self._h))

    def state(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.size, dtype=np.complex128)
        check(lib().llg_copy_to_host(self._h, _ptr(out)))
        return out

    def load(self, amps: np.ndarray) -> None:
        a = np.ascontiguousarray(amps, dtype=np.complex128)
        check(lib().llg_copy_from_host(self._h, _ptr(a)))

    def probabilities(self) -> np.ndarray:
        out = np.empty(self.size, dtype=np.float64)
        check(lib().llg_probabilities(self._h, _ptr(out)))
        return out

    def norm2(self) -> float:
        v = ctypes.c_double()
        check(lib().llg_norm2(self._h, ctypes.byref(v)))
        return v.value

    def compare(self, other: "State") -> tuple[float, float]:
        """(fidelity, max |amplitude difference|) against another state of the same size, on the
        device in double."""
        f, d = ctypes.c_double(), ctypes.c_double()
        check(lib().llg_compare(self._h, other._h, ctypes.byref(f), ctypes.byref(d)))
        return f.value, d.value

    def compare_ex(self, other: "State") -> tuple[float, float, float]:
        """compare() plus the largest |re| or |im| of `other`'s amplitudes (the scale of a relative
        error)."""
        f, d, m = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(lib().llg_compare_ex(self._h, other._h, ctypes.byref(f), ctypes.byref(d), ctypes.byref(m)))
        return f.value, d.value, m.value

    def expect_diagonal(self, diag) -> float:
        """sum_i |a_i|^2 diag[i] for a full diagonal: a numpy array of 2^n doubles (copied to the
        device) or a CUDA array with __cuda_array_interface__ (a torch tensor, read in place)."""
        cai = getattr(diag, "__cuda_array_interface__", None)
        v = ctypes.c_double()
        if cai is not None:
            if tuple(cai["shape"]) != (self.size,) or cai["typestr"] != "<f8" or cai.get("strides") not in (None, (8,)):
                raise ValueError("the diagonal must be a contiguous float64 vector of 2^n entries")
            check(lib().llg_expect_diagonal(self._h, ctypes.c_void_p(cai["data"][0]), 1, ctypes.byref(v)))
        else:
            d = np.ascontiguousarray(diag, dtype=np.float64)
            if d.shape != (self.size,):
                raise ValueError("the diagonal must have 2^n entries")
            check(lib().llg_expect_diagonal(self._h, _ptr(d), 0, ctypes.byref(v)))
        return v.value

    def expect_zz(self, a: Sequence[int], b: Sequence[int], coeff: Sequence[float]) -> float:
        aa = np.ascontiguousarray(a, dtype=np.int32)
        bb = np.ascontiguousarray(b, dtype=np.int32)
        cc = np.ascontiguousarray(coeff, dtype=np.float64)
        v = ctypes.c_double()
        check(lib().llg_expect_zz(self._h, aa.size, _ptr(aa), _ptr(bb), _ptr(cc), ctypes.byref(v)))
        return v.value

    def renormalize(self) -> None:
        check(lib().llg_renormalize(self._h))

    def reset(self, n: int) -> None:
        check(lib().llg_reset(self._h, n))

    def profile(self, on: bool = True) -> None:
        check(lib().llg_profile(self._h, 1 if on else 0))

    def profile_read(self, reset: bool = True):
        """{class: (milliseconds, launches)} for tile / gate / init / readout kernels."""
        ms = np.zeros(PROF_CLASSES, dtype=np.float64)
        n = np.zeros(PROF_CLASSES, dtype=np.int64)
        check(lib().llg_profile_read(self._h, _ptr(ms), _ptr(n), 1 if reset else 0))
        return {name: (float(ms[k]), int(n[k])) for k, name in enumerate(PROF_NAMES)}

    @property
    def stream(self) -> int:
        v = ctypes.c_void_p()
        check(lib().llg_get_stream(self._h, ctypes.byref(v)))
        return v.value or 0


# ---------------------------------------------------------------------------------------------
# planner introspection (host only)
# ---------------------------------------------------------------------------------------------
PLAN_ZYZ = 1
PLAN_TABLES = 2
PLAN_REGS = 4
PLAN_FUSE2 = 8
PLAN_DF64 = 16
PLAN_STREAM = 32


def plan_export(n: int, ops: np.ndarray, tile_qubits: int, zyz: bool = False, tables: bool = False,
                regs: bool = False, fuse2: bool = False, df64: bool = False, stream: bool = False):
    """Host-side plan of `ops` (passes, executor ops; coefficients as doubles).  zyz=True plans
    as the engine does for complex128 states (fused unitary 2x2s as carried-phase rotations);
    tables=True (with zyz) also gathers diagonal factors into phase tables, and the result gains a
    third item: the tables as a complex array (2^tile_qubits entries per table); fuse2=True plans the
    two-qubit blocks of complex64 tile passes (kind 20, 16 table entries each) and also returns the
    tables; df64=True plans as for a double-float state (IEEE complex128 otherwise); stream=True
    returns the per-gate lowering of an unfused IEEE complex128 flush as one whole-register pass."""
    ops = np.ascontiguousarray(ops, dtype=OP_DTYPE)
    flags = ((PLAN_ZYZ if zyz else 0) | (PLAN_TABLES if tables else 0) | (PLAN_REGS if regs else 0) |
             (PLAN_FUSE2 if fuse2 else 0) | (PLAN_DF64 if df64 else 0) | (PLAN_STREAM if stream else 0))
    npasses, nx = ctypes.c_int(), ctypes.c_int()
    check(lib().llg_plan_export_ex(n, _ptr(ops) if ops.size else None, ops.size, tile_qubits, flags, None, 0,
                                   ctypes.byref(npasses), None, 0, ctypes.byref(nx)))
    passes = np.zeros(npasses.value, dtype=PASS_DTYPE)
    xops = np.zeros(max(nx.value, 1), dtype=XOP_DTYPE)
    check(lib().llg_plan_export_ex(n, _ptr(ops) if ops.size else None, ops.size, tile_qubits, flags, _ptr(passes),
                                   passes.size, ctypes.byref(npasses), _ptr(xops), xops.size, ctypes.byref(nx)))
    if not (tables or fuse2):
        return passes, xops[: nx.value]
    nd = ctypes.c_int64()
    check(lib().llg_plan_export_tables(n, _ptr(ops) if ops.size else None, ops.size, tile_qubits, flags, None, 0,
                                       ctypes.byref(nd)))
    tab = np.zeros(max(nd.value, 2), dtype=np.float64)
    check(lib().llg_plan_export_tables(n, _ptr(ops) if ops.size else None, ops.size, tile_qubits, flags, _ptr(tab),
                                       tab.size, ctypes.byref(nd)))
    return passes, xops[: nx.value], tab[: nd.value].view(np.complex128)


def fp64_fma_rate(iters: int = 1 << 16) -> float:
    """FP64 fused multiply-adds per second of the current device (a timed throughput kernel)."""
    v = ctypes.c_double()
    check(lib().llg_fp64_fma_rate(iters, ctypes.byref(v)))
    return v.value


def diag_export(n: int, a, b, coeff) -> np.ndarray:
    """The observable's eigenvalue per basis index by the GPU kernel's chunked decomposition,
    computed on the host (tests)."""
    aa = np.ascontiguousarray(a, dtype=np.int32)
    bb = np.ascontiguousarray(b, dtype=np.int32)
    cc = np.ascontiguousarray(coeff, dtype=np.float64)
    out = np.empty(1 << n, dtype=np.float64)
    check(lib().llg_diag_export(n, aa.size, _ptr(aa), _ptr(bb), _ptr(cc), _ptr(out)))
    return out


def ising_terms(n: int, zz=(), z=()):
    """(a, b, coeff) lists of H = sum J_ij Z_i Z_j + sum h_i Z_i with the arguments of the
    reference's ising_diagonal (python/algorithms.py:139-152): zz a list of (i, j, J), z a list of
    (i, h).  llg_expect_zz evaluates them without the 2^n diagonal."""
    a, b, c = [], [], []
    for i, j, v in zz:
        a.append(int(i))
        b.append(int(j))
        c.append(float(v))
    for i, v in z:
        a.append(int(i))
        b.append(-1)
        c.append(float(v))
    for q in a + [x for x in b if x >= 0]:
        if not 0 <= q < n:
            raise ValueError(f"qubit {q} outside [0, {n})")
    return a, b, c


def ring_zz_terms(n: int):
    """Observable sum_i Z_i Z_{i+1 mod n} as (a, b, coeff) lists."""
    a = list(range(n))
    b = [(i + 1) % n for i in range(n)]
    return a, b, [1.0] * n



# ---------------------------------------------------------------------------------------------
# batched parametrised circuits (adjoint gradients, parameter shift)
# ---------------------------------------------------------------------------------------------
class Adjoint:
    """A planned parametrised circuit for batches of up to `max_batch` parameter sets.

    `ops` is an llg_op array whose RX/RY/RZ records carry `param` >= 0 for trainable angles;
    the observable is sum_k coeff[k] Z_a[k] Z_b[k] (b[k] < 0: single Z)."""

    def __init__(self, n: int, ops: np.ndarray, nparams: int, observable, max_batch: int = 64,
                 precision: str = "complex128"):
        a, b, c = observable
        aa = np.ascontiguousarray(a, dtype=np.int32)
        bb = np.ascontiguousarray(b, dtype=np.int32)
        cc = np.ascontiguousarray(c, dtype=np.float64)
        self._ops = np.ascontiguousarray(ops, dtype=OP_DTYPE)
        self.n, self.nparams, self.max_batch = n, nparams, max_batch
        self._h = ctypes.c_void_p()
        check(lib().llg_adjoint_create(n, _ptr(self._ops) if self._ops.size else None, self._ops.size, nparams,
                                       max_batch, PRECISIONS[precision], aa.size, _ptr(aa), _ptr(bb), _ptr(cc),
                                       ctypes.byref(self._h)))

    def close(self) -> None:
        if self._h:
            lib().llg_adjoint_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_threads(self, threads: int) -> None:
        check(lib().llg_adjoint_set_threads(self._h, threads))

    def info(self) -> dict:
        f, b_, n = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().llg_adjoint_info(self._h, ctypes.byref(f), ctypes.byref(b_), ctypes.byref(n)))
        return {"forward_passes": f.value, "backward_passes": b_.value, "param_ops": n.value}

    @property
    def stream(self) -> int:
        v = ctypes.c_void_p()
        check(lib().llg_adjoint_stream(self._h, ctypes.byref(v)))
        return v.value or 0

    def run(self, params: np.ndarray, grads: bool = True, checkpoint_every: int = 0):
        """(energies[batch], grads[batch, nparams] or None) for host parameter sets."""
        p = np.ascontiguousarray(np.atleast_2d(params), dtype=np.float64)
        batch = p.shape[0]
        e = np.zeros(batch)
        g = np.zeros((batch, self.nparams)) if grads else None
        check(lib().llg_adjoint_run(self._h, _ptr(p), batch, _ptr(e), _ptr(g) if grads else None, checkpoint_every))
        return e, g

    def run_device(self, params_ptr: int, batch: int, energies_ptr: int, grads_ptr: int | None,
                   checkpoint_every: int = 0) -> None:
        """Same, on device pointers (e.g. torch CUDA tensors' data_ptr())."""
        check(lib().llg_adjoint_run(self._h, params_ptr, batch, energies_ptr, grads_ptr, checkpoint_every))

    def param_shift(self, params: np.ndarray):
        p = np.ascontiguousarray(np.atleast_2d(params), dtype=np.float64)
        sets = p.shape[0]
        e = np.zeros(sets)
        g = np.zeros((sets, self.nparams))
        check(lib().llg_param_shift_run(self._h, _ptr(p), sets, _ptr(e), _ptr(g)))
        return e, g


# ---------------------------------------------------------------------------------------------
# batched noisy trajectories
# ---------------------------------------------------------------------------------------------
def noise_sites(ops: np.ndarray) -> int:
    """Number of touched-qubit noise sites of a circuit (each runs amplitude then phase damping)."""
    k = np.asarray(ops["kind"])
    two = np.isin(k, [OP_CNOT, OP_CZ]).sum()
    mcz = sum(bin(int(m)).count("1") for m in np.asarray(ops["mask"])[k == OP_MCZ])
    return int(len(ops) - two - (k == OP_MCZ).sum() + 2 * two + mcz)


def traj_run(n: int, ops: np.ndarray, gamma: float, lam: float, seed: int, n_traj: int, begin: int = 0,
             precision: str = "complex128", log: bool = False):
    """(z0[n_traj], jumps[n_traj], jump_log[n_traj, sites] or None, min margin)."""
    ops = np.ascontiguousarray(ops, dtype=OP_DTYPE)
    z0 = np.zeros(n_traj)
    jumps = np.zeros(n_traj, dtype=np.uint32)
    sites = noise_sites(ops)
    jl = np.zeros((n_traj, max(sites, 1)), dtype=np.uint8) if log else None
    margin = ctypes.c_double()
    check(lib().llg_traj_run(n, _ptr(ops) if ops.size else None, ops.size, gamma, lam, seed, begin, n_traj,
                             PRECISIONS[precision], _ptr(z0), _ptr(jumps), _ptr(jl) if log else None,
                             jl.shape[1] if log else 0, ctypes.byref(margin)))
    return z0, jumps, jl, margin.value


class Traj:
    """A trajectory circuit planned once; every launch replays its captured CUDA graph."""

    def __init__(self, n: int, ops: np.ndarray, gamma: float, lam: float, max_traj: int,
                 precision: str = "complex128", cluster: int = 0, cta_threads: int = 0):
        self._ops = np.ascontiguousarray(ops, dtype=OP_DTYPE)
        self._h = ctypes.c_void_p()
        self.max_traj = int(max_traj)
        check(lib().llg_traj_create(n, _ptr(self._ops) if self._ops.size else None, self._ops.size, gamma, lam,
                                    PRECISIONS[precision], self.max_traj, cluster, cta_threads, ctypes.byref(self._h)))

    def launch(self, seed: int, n_traj: int, begin: int = 0):
        """(z0[n_traj], jumps[n_traj], min margin)."""
        z0 = np.zeros(n_traj)
        jumps = np.zeros(n_traj, dtype=np.uint32)
        margin = ctypes.c_double()
        check(lib().llg_traj_launch(self._h, seed, begin, n_traj, _ptr(z0), _ptr(jumps), ctypes.byref(margin)))
        return z0, jumps, margin.value

    def autotune(self, sample_traj: int = 0) -> dict:
        r = np.zeros(1, dtype=TUNE_DTYPE)
        check(lib().llg_traj_autotune(self._h, sample_traj, _ptr(r)))
        return _tune_dict(r)

    def config(self) -> dict:
        c, t, g, s = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int64()
        check(lib().llg_traj_config(self._h, ctypes.byref(c), ctypes.byref(t), ctypes.byref(g), ctypes.byref(s)))
        return {"cluster": c.value, "cta_threads": t.value, "grid": g.value, "sites": s.value}

    @property
    def stream(self) -> int:
        v = ctypes.c_void_p()
        check(lib().llg_traj_stream(self._h, ctypes.byref(v)))
        return v.value or 0

    def close(self) -> None:
        if self._h:
            lib().llg_traj_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NoisyTraj(Traj):
    """Depolarizing-noise trajectories of a folded circuit (batched ll::NoisyBackend); launch()
    returns (observable[n_traj], non-identity Paulis[n_traj], margin)."""

    def __init__(self, n: int, ops: np.ndarray, p: float, scale: int, max_traj: int, terms=(),
                 precision: str = "complex128", cluster: int = 0, cta_threads: int = 0):
        self._ops = np.ascontiguousarray(ops, dtype=OP_DTYPE)
        self._h = ctypes.c_void_p()
        self.max_traj = int(max_traj)
        a, b, c = _obs_terms(terms)
        check(lib().llg_noisy_create(n, _ptr(self._ops) if self._ops.size else None, self._ops.size, p, scale,
                                     PRECISIONS[precision], self.max_traj, a.size, _ptr(a), _ptr(b), _ptr(c),
                                     cluster, cta_threads, ctypes.byref(self._h)))


def _obs_terms(terms):
    """[(a, b, coeff), ...] with b = -1 for a single Z -> three contiguous arrays."""
    terms = list(terms)
    a = np.ascontiguousarray([t[0] for t in terms], dtype=np.int32)
    b = np.ascontiguousarray([t[1] for t in terms], dtype=np.int32)
    c = np.ascontiguousarray([t[2] for t in terms], dtype=np.float64)
    return a, b, c


ZNE_DTYPE = np.dtype([("value", np.float64), ("std_error", np.float64), ("nscales", np.int32), ("pad", np.int32),
                      ("trajectories", np.int64), ("scales", np.float64, (8,)), ("values", np.float64, (8,)),
                      ("std_errors", np.float64, (8,)), ("weights", np.float64, (8,))])


def richardson_weights(scales) -> np.ndarray:
    s = np.ascontiguousarray(scales, dtype=np.float64)
    w = np.zeros(s.size)
    check(lib().llg_richardson_weights(_ptr(s), s.size, _ptr(w)))
    return w


def zne(n: int, ops: np.ndarray, p: float, scales=(1, 3, 5), trajectories: int = 1000, seed: int = 1, terms=(),
        precision: str = "complex128") -> dict:
    """ll::ZNE::extrapolate over the GPU noisy trajectories: value, std_error, per-scale values,
    standard errors and Richardson weights."""
    ops = np.ascontiguousarray(ops, dtype=OP_DTYPE)
    s = np.ascontiguousarray(scales, dtype=np.float64)
    a, b, c = _obs_terms(terms)
    r = np.zeros(1, dtype=ZNE_DTYPE)
    check(lib().llg_zne_run(n, _ptr(ops) if ops.size else None, ops.size, p, PRECISIONS[precision], _ptr(s), s.size,
                            trajectories, seed, a.size, _ptr(a), _ptr(b), _ptr(c), _ptr(r)))
    k = int(r["nscales"][0])
    return {"value": float(r["value"][0]), "std_error": float(r["std_error"][0]),
            "trajectories": int(r["trajectories"][0]), "scales": r["scales"][0][:k].copy(),
            "values": r["values"][0][:k].copy(), "std_errors": r["std_errors"][0][:k].copy(),
            "weights": r["weights"][0][:k].copy()}


# ---------------------------------------------------------------------------------------------
# density matrices (the reference's KrausChannel on a GPU-resident rho)
# ---------------------------------------------------------------------------------------------
_PAULI = [np.eye(2), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]), np.diag([1.0, -1.0])]


def amplitude_damping(gamma: float):
    """Kraus operators of src/Noise.cpp:274-285."""
    if not 0.0 <= gamma <= 1.0:
        raise ValueError("KrausChannel::amplitude_damping: gamma must be in [0, 1]")
    return [np.array([[1, 0], [0, np.sqrt(max(0.0, 1 - gamma))]], dtype=complex),
            np.array([[0, np.sqrt(gamma)], [0, 0]], dtype=complex)]


def phase_damping(lam: float):
    """Kraus operators of src/Noise.cpp:287-298."""
    if not 0.0 <= lam <= 1.0:
        raise ValueError("KrausChannel::phase_damping: lambda must be in [0, 1]")
    return [np.array([[1, 0], [0, np.sqrt(max(0.0, 1 - lam))]], dtype=complex),
            np.array([[0, 0], [0, np.sqrt(lam)]], dtype=complex)]


def depolarizing(p: float, m: int = 1):
    """DepolarizingChannel(p, m).to_kraus (src/Noise.cpp:309-333): sqrt(1-p) I and
    sqrt(p / (4^m - 1)) P for each non-identity Pauli string; digit j of the string code (base 4)
    acts on target j, the most significant target first in the Kronecker product."""
    if not 0.0 <= p <= 1.0 or m not in (1, 2):
        raise ValueError("DepolarizingChannel: p in [0, 1] and 1 or 2 qubits")
    ops = []
    for code in range(4 ** m):
        w = np.sqrt(1 - p) if code == 0 else np.sqrt(p / (4 ** m - 1))
        if w > 0:
            mat = np.eye(1)
            for j in range(m - 1, -1, -1):
                mat = np.kron(mat, _PAULI[(code >> (2 * j)) & 3])
            ops.append(w * mat)
    return ops


class DensityMatrix:
    """rho on n qubits held on the GPU as a 2n-qubit state (element (row, col) at amplitude
    row + col * 2^n).  Gates act as U rho U^+; kraus() applies the reference's
    KrausChannel::apply."""

    def __init__(self, n: int, precision: str = "complex128", rho: np.ndarray | None = None):
        self.n = int(n)
        if rho is None:
            self._st = State(2 * self.n, precision)
        else:
            rho = np.asarray(rho, dtype=np.complex128)
            if rho.shape != (1 << self.n, 1 << self.n):
                raise ValueError("rho must be 2^n x 2^n")
            self._st = State(precision=precision, amps=np.ascontiguousarray(rho.T).reshape(-1))

    def apply_ops(self, ops: np.ndarray) -> None:
        for op in np.ascontiguousarray(ops, dtype=OP_DTYPE):
            one = np.ascontiguousarray(np.array([op], dtype=OP_DTYPE))
            check(lib().llg_dm_apply_op(self._st.handle, self.n, _ptr(one)))

    def kraus(self, ops, targets: Sequence[int]) -> None:
        kk = np.ascontiguousarray(np.asarray(ops, dtype=np.complex128))
        tg = np.ascontiguousarray(targets, dtype=np.int32)
        if kk.ndim != 3 or kk.shape[1] != kk.shape[2] or kk.shape[1] != (1 << tg.size):
            raise ValueError("KrausChannel: operators must be 2^m x 2^m for m targets")
        check(lib().llg_dm_apply_kraus(self._st.handle, self.n, kk.shape[0], _ptr(kk), tg.size, _ptr(tg)))

    @property
    def state(self) -> "State":
        """The 2n-qubit state that holds rho (for sync, profiling and the other State calls)."""
        return self._st

    def rho(self) -> np.ndarray:
        dim = 1 << self.n
        return np.ascontiguousarray(self._st.state().reshape(dim, dim).T)

    def probabilities(self) -> np.ndarray:
        return np.real(np.diag(self.rho())).copy()

    def trace(self) -> complex:
        return complex(np.trace(self.rho()))

    def close(self) -> None:
        self._st.close()


# ---------------------------------------------------------------------------------------------
# dense trajectory solver (the reference's TrajectorySolver)
# ---------------------------------------------------------------------------------------------
UNRAVEL = {"STANDARD": 0, "PROJECTOR": 1, "ANALOG": 2}
_HFN = ctypes.CFUNCTYPE(None, ctypes.c_double, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p)


def _cmat(m, dim: int) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
    if a.shape != (dim, dim):
        raise ValueError(f"operator must be {dim} x {dim}")
    return a


class TrajectorySolver:
    """Lindblad trajectories with dense operators on n <= 10 qubits (src/TrajectorySolver.h),
    every call one persistent GPU launch over all trajectories."""

    def __init__(self, n_qubits: int):
        self._h = ctypes.c_void_p()
        check(lib().llg_tsolver_create(n_qubits, ctypes.byref(self._h)))
        self.n_qubits = int(n_qubits)
        self.dim = 1 << self.n_qubits
        self._fn = None

    def set_hamiltonian(self, h) -> None:
        """A dim x dim Hermitian matrix, or a function t -> matrix (sampled at the plan's nodes)."""
        if callable(h):
            dim = self.dim

            def cb(t, out, user):
                m = np.ascontiguousarray(np.asarray(h(t), dtype=np.complex128))
                if m.shape != (dim, dim):
                    m = np.full((dim, dim), np.nan, dtype=np.complex128)
                ctypes.memmove(out, m.ctypes.data, m.nbytes)

            fn = _HFN(cb)
            check(lib().llg_tsolver_set_hamiltonian_fn(self._h, ctypes.cast(fn, ctypes.c_void_p), None))
            self._fn = fn  # the callback lives as long as the solver uses it
        else:
            m = _cmat(h, self.dim)
            check(lib().llg_tsolver_set_hamiltonian(self._h, _ptr(m)))
            self._fn = None

    def add_lindblad(self, l, gamma: float) -> None:
        m = _cmat(l, self.dim)
        check(lib().llg_tsolver_add_lindblad(self._h, _ptr(m), float(gamma)))

    def clear_lindblad(self) -> None:
        check(lib().llg_tsolver_clear_lindblad(self._h))

    def n_channels(self) -> int:
        v = ctypes.c_int()
        check(lib().llg_tsolver_info(self._h, ctypes.byref(v), None))
        return v.value

    def projector_applies(self, i: int) -> bool:
        v = ctypes.c_int()
        check(lib().llg_tsolver_projector_applies(self._h, i, ctypes.byref(v)))
        return bool(v.value)

    def _run(self, psi0, duration, dt, n, kind, seed, states=False, rho=False, obs=None):
        p0 = np.ascontiguousarray(np.asarray(psi0, dtype=np.complex128).reshape(-1))
        if p0.size != self.dim:
            raise ValueError("psi0 must have length 2^n_qubits")
        st = np.zeros((n, self.dim), dtype=np.complex128) if states else None
        r = np.zeros((self.dim, self.dim), dtype=np.complex128) if rho else None
        o = _cmat(obs, self.dim) if obs is not None else None
        ov = np.zeros(n) if obs is not None else None
        check(lib().llg_tsolver_run(self._h, _ptr(p0), float(duration), float(dt), int(n), UNRAVEL[kind], int(seed),
                                    _ptr(st) if states else None, _ptr(r) if rho else None,
                                    _ptr(o) if o is not None else None, _ptr(ov) if ov is not None else None))
        return st, r, ov

    def run_one(self, psi0, duration: float, dt: float, seed: int, kind: str = "STANDARD") -> np.ndarray:
        st, _, _ = self._run(psi0, duration, dt, 1, kind, seed, states=True)
        return st[0]

    def evolve_ensemble(self, psi0, duration: float, dt: float, n_trajectories: int, kind: str = "STANDARD",
                        seed: int = 0) -> np.ndarray:
        _, r, _ = self._run(psi0, duration, dt, n_trajectories, kind, seed, rho=True)
        return r

    def states(self, psi0, duration: float, dt: float, n_trajectories: int, kind: str = "STANDARD",
               seed: int = 0) -> np.ndarray:
        st, _, _ = self._run(psi0, duration, dt, n_trajectories, kind, seed, states=True)
        return st

    def estimate_observable(self, psi0, duration: float, dt: float, n_trajectories: int, kind: str, obs,
                            seed: int = 0) -> dict:
        """Mean and standard error of obs(psi_T); obs is a Hermitian matrix (evaluated on the GPU)
        or a function of the state vector (evaluated on the host over the returned states)."""
        if callable(obs):
            st, _, _ = self._run(psi0, duration, dt, n_trajectories, kind, seed, states=True)
            v = np.array([float(obs(x)) for x in st])
        else:
            _, _, v = self._run(psi0, duration, dt, n_trajectories, kind, seed, obs=obs)
        n = v.size
        mean = float(v.sum() / n)
        se = float(np.sqrt(np.sum((v - mean) ** 2) / (n - 1) / n)) if n > 1 else 0.0
        return {"mean": mean, "std_error": se, "n": n}

    def plan(self) -> dict:
        steps, h, const, kind = ctypes.c_longlong(), ctypes.c_double(), ctypes.c_int(), ctypes.c_int()
        nops, nnodes = ctypes.c_int(), ctypes.c_int64()
        check(lib().llg_tsolver_plan_export(self._h, ctypes.byref(steps), ctypes.byref(h), ctypes.byref(const),
                                            ctypes.byref(kind), None, None, 0, None, None, ctypes.byref(nops),
                                            ctypes.byref(nnodes)))
        d = self.dim
        prop = np.zeros((d, d), dtype=np.complex128)
        nodes = np.zeros((max(nnodes.value, 1), d, d), dtype=np.complex128)
        ops = np.zeros((max(nops.value, 1), d, d), dtype=np.complex128)
        dop = np.zeros_like(ops)
        check(lib().llg_tsolver_plan_export(self._h, None, None, None, None, _ptr(prop), _ptr(nodes), nodes.shape[0],
                                            _ptr(ops), _ptr(dop), ctypes.byref(nops), ctypes.byref(nnodes)))
        return {"steps": steps.value, "h": h.value, "constant": bool(const.value), "kind": kind.value, "prop": prop,
                "nodes": nodes[:nnodes.value], "ops": ops[:nops.value], "ops_dop": dop[:nops.value]}

    def close(self) -> None:
        if self._h:
            lib().llg_tsolver_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------------------------
# mixed-size batches
# ---------------------------------------------------------------------------------------------
def batch_autotune(n_qubits, ops: np.ndarray, offsets, precision: str = "complex128") -> dict:
    nq = np.ascontiguousarray(n_qubits, dtype=np.int32)
    ops = np.ascontiguousarray(ops, dtype=OP_DTYPE)
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    r = np.zeros(1, dtype=TUNE_DTYPE)
    check(lib().llg_batch_autotune(nq.size, _ptr(nq), _ptr(ops) if ops.size else None, _ptr(off),
                                   PRECISIONS[precision], _ptr(r)))
    return _tune_dict(r)


class Batch:
    """Circuits of uneven sizes run together in one persistent launch."""

    def __init__(self, n_qubits, ops: np.ndarray, offsets, precision: str = "complex128", tile_qubits: int = 0):
        self.nq = np.ascontiguousarray(n_qubits, dtype=np.int32)
        self._ops = np.ascontiguousarray(ops, dtype=OP_DTYPE)
        self._off = np.ascontiguousarray(offsets, dtype=np.int64)
        self._h = ctypes.c_void_p()
        check(lib().llg_batch_create(self.nq.size, _ptr(self.nq), _ptr(self._ops) if self._ops.size else None,
                                     _ptr(self._off), PRECISIONS[precision], tile_qubits, ctypes.byref(self._h)))

    def close(self) -> None:
        if self._h:
            lib().llg_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> dict:
        w, a, p = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        check(lib().llg_batch_info(self._h, ctypes.byref(w), ctypes.byref(a), ctypes.byref(p)))
        t, g, th = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().llg_batch_config(self._h, ctypes.byref(t), ctypes.byref(g), ctypes.byref(th)))
        return {"work_items": w.value, "total_amps": a.value, "total_passes": p.value, "tile_qubits": t.value,
                "grid": g.value, "cta_threads": th.value}

    def run(self, spin_limit: int = 0) -> None:
        check(lib().llg_batch_run(self._h, spin_limit))

    def state(self, index: int) -> np.ndarray:
        out = np.empty(1 << int(self.nq[index]), dtype=np.complex128)
        check(lib().llg_batch_copy_state(self._h, index, _ptr(out)))
        return out

    def fidelity(self, other: "Batch") -> np.ndarray:
        out = np.zeros((self.nq.size, 3))
        check(lib().llg_batch_fidelity(self._h, other._h, _ptr(out)))
        return out

    @property
    def stream(self) -> int:
        v = ctypes.c_void_p()
        check(lib().llg_batch_stream(self._h, ctypes.byref(v)))
        return v.value or 0
