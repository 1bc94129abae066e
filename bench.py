#!/usr/bin/env python
"""Benchmark: 30-qubit complex128 layered circuit on one GB300 (the headline workload).

Workload (seeded, synthetic): a 30-qubit state from |0..0> (16 GiB of complex128), 20 layers of
RX, RY, RZ on every qubit (angles U[0, 2pi)) plus a CNOT brickwork on (i, i+1) with alternating
offsets -- 1800 rotations + 290 CNOTs = 2090 gates.  One step = reset the state and run the whole
circuit through the engine: fused shared-memory tile passes with carried phases and phase tables,
complex128 in IEEE binary64 (the reference's arithmetic).

Printed as one JSON line:
  value        gates/s over the whole job (logical, pre-fusion gates), device-timed with CUDA
               events on the engine's stream, inputs resident in HBM;
  e2e          the same metric through the drop-in API (quantum_sim_v3.StateVector) with the
               final amplitudes read back to host memory (get_numpy_view) every step;
  roofline     the dominant kernel (the tile pass): algorithmic bytes per launch (32 B x 2^30
               amplitudes: one read and one write of the state) / its mean launch time, measured
               with CUDA events around every launch inside the timed region;
  fp64_roofline the bound that applies to IEEE complex128 on this GPU: the plan's algorithmic FP64
               multiply-adds per step over the tile passes' time, against the FP64 FMA rate
               measured live by a throughput kernel;
  cpu_baseline the reference's CPU algorithms on the machine's host cores (the oracle's restatement,
               checked bit-exact against the reference build): the per-gate ll::StateVectorBackend
               path and the fused path (GateFuser.fuse_circuit + apply_gate_cache_optimized), each
               timed per gate kind on the 30-qubit state and combined over the circuit's gate mix;
  variants     the same circuit in double-float ("df64") and complex64, each with its rate, e2e,
               rooflines and its error against the IEEE FP64 state (max |d amp|, relative to the
               largest amplitude, and 1 - fidelity).
`--impl reference` times the CPU implementation alone as the reference arm.

Beside the headline the line carries, each with its own workload description and, where the
oracle can run a sample of it, a CPU baseline: per-gate and dense-block sweeps against HBM
(`gate_sweeps`), adjoint gradients against parameter shift (`adjoint`), noisy trajectories
(`trajectories`), mixed circuit batches (`mixed_batch`), zero-noise extrapolation (`zne`), the
12-qubit published workload (`config1_12q`), the dense trajectory solver (`trajectory_solver`) and
density-matrix channels (`density_matrix`); `summary` at the end repeats their key figures.
`--no-sweeps`, `--no-adjoint`, `--no-forms`, `--no-variants` skip them.

Multi-GPU: the path does not shard (one state per GPU); with torchrun each rank runs an
independent replica and `value` sums them ("replicas only", weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "lightning-lite-quantum-simulator_gb300")
ORACLE = os.path.join(REPO, "oracle")
for _p in (PKG, ORACLE):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "30q gates/s"
FALLBACK_HBM_GBS = 6800.0
E2E_STEPS_MAX = 5  # the e2e loop and the variants run at most this many steps


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--layers", type=int, default=20)
    ap.add_argument("--precision", default="complex128",
                    help="complex128 (IEEE FP64, the reference's arithmetic), df64 or complex64")
    ap.add_argument("--tile", type=int, default=-1,
                    help="tile width in qubits; -1 (default): the autotuner picks width and CTA threads")
    ap.add_argument("--cta-threads", type=int, default=0, help="tile-kernel CTA threads with an explicit --tile")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-variants", action="store_true", help="skip the df64 / complex64 variants of the headline")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint-gradient measurement")
    ap.add_argument("--no-forms", action="store_true", help="skip the trajectory and mixed-batch measurements")
    ap.add_argument("--no-sweeps", action="store_true", help="skip the per-gate sweep roofline measurement")
    return ap.parse_args()


def dist_env():
    import replicas

    return replicas.rank_env()


def peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


# --------------------------------------------------------------------------------------------
# CPU side: the reference's algorithms (oracle restatements), timed per gate kind
# --------------------------------------------------------------------------------------------
def circuit_mix(n: int, ops: np.ndarray) -> dict:
    """Gate counts of the per-gate path (rotations, CNOTs) and of the reference's fused path
    (fused 2x2s after GateFuser.fuse_circuit, CNOTs)."""
    import oracle

    kinds = ops["kind"]
    fused = oracle.fuse_gate_list(n, ops)
    return {"gates": int(len(ops)), "rotations": int(np.sum(np.isin(kinds, (2, 3, 4)))),
            "cnots": int(np.sum(kinds == 5)), "fused_2x2": sum(1 for f in fused if f[0] == "u2")}


def cpu_gate_times(n: int, threads: int, reps: int, kinds=("rx", "ry", "rz", "cnot", "u2")) -> dict:
    """Best-of-`reps` seconds per gate of each kind on an n-qubit state with `threads` OpenMP
    threads (after one untimed application of each): RX/RY/RZ/CNOT by the reference's per-gate
    ll::StateVectorBackend algorithm (src/StateVectorBackend.h:61-135), U2 by
    apply_gate_cache_optimized (src/StateVectorOptimized.cpp:56-78), as the oracle restates them.
    Targets spread over the register: rotations on qubits 0, n/2, n-1; CNOTs on (0, 1) and
    (n-2, n-1), the brickwork's pairs."""
    import ctypes

    import oracle

    L = oracle.lib()
    oracle.set_threads(threads)
    psi = oracle.zero_state(n)
    p = psi.ctypes.data
    u = np.linalg.qr(np.array([[0.6 + 0.1j, 0.3 - 0.2j], [-0.3 - 0.2j, 0.6 - 0.1j]]))[0].reshape(4)
    gbuf = np.ascontiguousarray(np.stack([u.real, u.imag], axis=1).reshape(8))
    L.orc_rx.argtypes = L.orc_ry.argtypes = L.orc_rz.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                                  ctypes.c_double]
    L.orc_cnot.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    qs = (0, n // 2, n - 1)
    calls = {"rx": [lambda q=q: L.orc_rx(p, n, q, 0.7) for q in qs],
             "ry": [lambda q=q: L.orc_ry(p, n, q, 1.1) for q in qs],
             "rz": [lambda q=q: L.orc_rz(p, n, q, 0.4) for q in qs],
             "cnot": [lambda: L.orc_cnot(p, n, 0, 1), lambda: L.orc_cnot(p, n, n - 2, n - 1)],
             "u2": [lambda q=q: L.orc_apply_gate_v3(p, n, q, gbuf.ctypes.data) for q in qs]}
    out = {}
    for k in kinds:
        for f in calls[k]:
            f()  # untimed
        best = float("inf")
        for _ in range(reps):
            t0 = time.perf_counter()
            for f in calls[k]:
                f()
            best = min(best, (time.perf_counter() - t0) / len(calls[k]))
        out[k] = best
    del psi
    return out


def cpu_rates(mix: dict, t: dict) -> dict:
    """Whole-circuit gates/s of the reference's per-gate path and of its fused path, from the
    per-kind times and the circuit's gate mix."""
    t_rot = (t["rx"] + t["ry"] + t["rz"]) / 3.0
    per_gate = mix["gates"] / (mix["rotations"] * t_rot + mix["cnots"] * t["cnot"])
    fused = mix["gates"] / (mix["fused_2x2"] * t["u2"] + mix["cnots"] * t["cnot"])
    return {"per_gate": per_gate, "fused": fused}


def cpu_baseline(n: int, ops: np.ndarray, reps: int = 5, one_thread: bool = True) -> dict:
    """Both reference CPU paths on every host core (best of `reps`) and on one thread (best of 1);
    `value` is the faster all-core figure."""
    mix = circuit_mix(n, ops)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    t_all = cpu_gate_times(n, cores, reps)
    r_all = cpu_rates(mix, t_all)
    out = {"value": max(r_all.values()), "unit": "gates/s", "cores": cores, "kind": "port",
           "path": "fused" if r_all["fused"] >= r_all["per_gate"] else "per_gate",
           "per_gate_gates_per_s": r_all["per_gate"], "fused_gates_per_s": r_all["fused"],
           "seconds_per_gate": t_all, "circuit_mix": mix}
    if one_thread:
        t_one = cpu_gate_times(n, 1, 1)
        r_one = cpu_rates(mix, t_one)
        out.update({"one_thread_per_gate_gates_per_s": r_one["per_gate"], "one_thread_fused_gates_per_s": r_one["fused"],
                    "one_thread_seconds_per_gate": t_one})
    out["sample"] = (f"each gate kind timed on the {n}-qubit state (RX/RY/RZ/U2 on qubits 0, {n // 2}, {n - 1}; CNOT "
                     f"on (0, 1), ({n - 2}, {n - 1})), best of {reps} on {cores} threads"
                     f"{' and best of 1 on 1 thread' if one_thread else ''} after one untimed application; "
                     f"combined over the circuit's {mix['rotations']} rotations + {mix['cnots']} CNOTs (per-gate "
                     f"ll::StateVectorBackend path) and {mix['fused_2x2']} fused 2x2s + {mix['cnots']} CNOTs "
                     f"(GateFuser.fuse_circuit + apply_gate_cache_optimized); oracle restatements; "
                     f"{time.perf_counter() - t0:.0f} s of CPU time")
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return
    import workloads

    ops = workloads.layered_rotations(args.qubits, args.layers)
    mix = circuit_mix(args.qubits, ops)
    cores = os.cpu_count() or 1
    # warm-up steps, then K timed steps: each step times one application of every gate kind on
    # every host core (a bounded sample of the circuit) and rates the whole circuit from it
    for _ in range(max(1, args.warmup)):
        cpu_gate_times(args.qubits, cores, 1)
    rates, times = [], []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        r = cpu_rates(mix, cpu_gate_times(args.qubits, cores, 1))
        times.append(time.perf_counter() - t0)
        rates.append(max(r.values()))
    rate = statistics.median(rates)
    sample = (f"per step: each gate kind applied once on the {args.qubits}-qubit state with {cores} threads, the "
              f"faster of the per-gate (ll::StateVectorBackend) and fused (GateFuser + apply_gate_cache_optimized) "
              f"paths combined over the circuit's gate mix; median of {len(rates)} steps after "
              f"{max(1, args.warmup)} warm-up")
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "gates/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(1, args.warmup), "ms_per_step": 1e3 * statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.qubits}-qubit complex128 layered circuit ({args.layers} layers), "
                               f"CPU sample per step", "qubits": args.qubits, "layers": args.layers},
        "cpu_baseline": {"value": rate, "unit": "gates/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": "gates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------------------------
# GPU side
# --------------------------------------------------------------------------------------------
# FP32 lane instructions per amplitude pair of each executor op kind (0 U2, 1 RX, 2 RY, 3 H, 4 X,
# 5 DIAG, 6 CNOT, 7 MCZ, 11 ZYZ, 12 ZY, 13 carried-phase flush, 14/15 tangent rotations with an input
# phase, 16/17 tangent rotations whose phase a table applied, 18 phase table), counted from the
# double-float routines of the kernels.  Results are stored without the closing Fast2Sum: a 4-term
# double-float dot product (df_lin4_raw) is 40 instructions, a 2-term one (df_lin2_raw) 16, an
# x + a*y update (df_fma_raw) 12.  A U2 pair needs four 4-term products; RX/RY/H four 2-term ones;
# a diagonal two 2-term ones per amplitude; a ZYZ eight; a ZY six; a flush two per pair; a tangent
# rotation two 2-term products and four updates, or the four updates alone after a table; a table
# a complex product per amplitude.  A CNOT carrying a pushed phase multiplies a quarter of the
# amplitudes.  CNOT, MCZ and X otherwise move or negate data without arithmetic.
FP32_INST_PER_PAIR = {"df64": {0: 160, 1: 64, 2: 64, 3: 64, 4: 0, 5: 64, 6: 0, 7: 0, 11: 128, 12: 96, 13: 32, 14: 80,
                               15: 80, 16: 48, 17: 48, 18: 64},
                      "complex64": {0: 16, 1: 8, 2: 8, 3: 8, 4: 0, 5: 8, 6: 0, 7: 0, 11: 16, 12: 12, 13: 4, 14: 8, 15: 8,
                                    16: 4, 17: 4, 18: 8, 20: 32, 21: 16}}
PHASED_CNOT_PER_PAIR = {"df64": 16, "complex64": 2}  # a complex multiply on a quarter of the amplitudes
# FP64 multiply-adds (DFMA or DMUL) per amplitude pair of each kind in IEEE complex128: a complex
# product is four, a real 2x2 row two, a generic complex 2x2 row eight
FP64_FMA_PER_PAIR = {0: 16, 1: 8, 2: 8, 3: 8, 4: 0, 5: 8, 6: 0, 7: 0, 11: 16, 12: 12, 13: 4, 14: 8, 15: 8, 16: 4, 17: 4,
                     18: 8}
FP64_PHASED_CNOT_PER_PAIR = 2
SMS, FP32_LANES_PER_SM = 152, 128
TILE_POLICY = {"df64": "PolDF64", "complex64": "PolF32", "complex128": "PolF64", "fp64": "PolF64"}
ELEM_BYTES = {"complex64": 8}


def is_f64(precision: str) -> bool:
    return precision in ("complex128", "fp64", "f64")


def plan_for(precision: str, n: int, ops, tile_q: int, regs: bool = False):
    """The plan the engine runs: carried phases and phase tables for 16-byte precisions, two-qubit
    blocks for complex64 shared-memory tiles, register programs for register-tiled passes."""
    import llgpu

    if regs:
        p, x = llgpu.plan_export(n, ops, tile_q, zyz=True, regs=True)
        return p, x, 0
    if precision == "complex64":
        p, x, tab = llgpu.plan_export(n, ops, tile_q, fuse2=True)
        return p, x, int(tab.nbytes)
    p, x, tab = llgpu.plan_export(n, ops, tile_q, zyz=True, tables=True, df64=precision == "df64")
    return p, x, int(tab.nbytes)


def compute_roofline(precision, n, xops, tile_ms_step, sm_mhz):
    """FP32-issue roofline of the tile passes (double-float and complex64): algorithmic FP32 lane
    instructions per step over the measured tile-pass time, against 152 SMs x 128 lanes x the
    sampled SM clock."""
    table = FP32_INST_PER_PAIR.get(precision)
    if table is None or not tile_ms_step or not len(xops):
        return None
    per_pair = sum(table.get(int(k), 0) for k in xops["kind"])
    per_pair += PHASED_CNOT_PER_PAIR.get(precision, 0) * int(np.sum((xops["kind"] == 6) & ((xops["flags"] & 8) != 0)))
    inst = per_pair * float(1 << (n - 1))
    achieved = inst / (tile_ms_step / 1e3) / 1e12
    mhz = sm_mhz or 2070.0
    peak = SMS * FP32_LANES_PER_SM * mhz * 1e6 / 1e12
    return {"bound": "fp32_issue", "achieved": achieved, "peak": peak, "unit": "Tinst/s", "frac": achieved / peak,
            "fp32_inst_per_step": inst, "peak_basis": f"{SMS} SMs x {FP32_LANES_PER_SM} FP32 lanes x {mhz:.0f} MHz"}


def fp64_roofline(n, xops, tile_ms_step, fma_rate):
    """FP64 roofline of the IEEE complex128 tile passes: the plan's FP64 multiply-adds per step
    (FP64_FMA_PER_PAIR x 2^(n-1) pairs per op) over the tile passes' time, against the FP64 FMA
    rate measured by the throughput kernel."""
    if not tile_ms_step or not len(xops) or not fma_rate:
        return None
    per_pair = sum(FP64_FMA_PER_PAIR.get(int(k), 0) for k in xops["kind"])
    per_pair += FP64_PHASED_CNOT_PER_PAIR * int(np.sum((xops["kind"] == 6) & ((xops["flags"] & 8) != 0)))
    fma = per_pair * float(1 << (n - 1))
    achieved = fma / (tile_ms_step / 1e3)
    return {"bound": "fp64_fma", "achieved": achieved / 1e12, "peak": fma_rate / 1e12, "unit": "TFMA/s",
            "frac": achieved / fma_rate, "fp64_fma_per_step": fma, "tflops_fp64": 2 * achieved / 1e12,
            "peak_basis": "FP64 FMA throughput kernel (llg_fp64_fma_rate), measured in this run"}


def profile_traffic(precision: str, n: int):
    """DRAM bytes per tile-pass launch from the committed ncu summary of this precision's tile
    pass, if present (scaled to a full launch there)."""
    name = {"df64": "k_tile_df64_30q.md", "complex128": "k_tile_f64_30q.md"}.get(precision)
    path = os.path.join(REPO, "profiles", name) if name else None
    if n != 30 or not path or not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if line.startswith("traffic_bytes_per_launch:"):
                try:
                    return float(line.split(":", 1)[1].strip())
                except ValueError:
                    return None
    return None


def measure_circuit(args, torch, precision, n, ops, steps, warmup, world, sampler_gpu=None, keep=False):
    """Timed steps of the layered circuit at `precision`: reset, apply, flush per step, CUDA events
    on the engine's stream, per-launch events for the tile passes.  Returns a dict (and the state
    when keep=True)."""
    import llgpu
    import replicas

    ngates = len(ops)
    st = llgpu.State(n, precision)
    tune = None
    if args.tile < 0:
        # autotuner: two layers of the circuit on a scratch state, outside the timed region
        tune = st.autotune(ops, sample_ops=4 * len(ops) // max(1, args.layers))
    else:
        st.set_fusion("tile", args.tile)
        st.set_tile_threads(args.cta_threads)
    tuning = st.tuning()
    tile_q = tuning["tile_qubits"]
    passes, xops, table_bytes = plan_for(precision, n, ops, tile_q, tuning["fuse_mode"] == "reg")
    if tuning["fuse_mode"] == "none":
        passes = np.zeros(ngates)  # one streaming pass per gate
    state_bytes = ELEM_BYTES.get(precision, 16) * (1 << n)
    stream = torch.cuda.ExternalStream(st.stream)
    for _ in range(warmup):
        st.reset(n)
        st.apply_ops(ops)
        st.flush()
    st.sync()
    st.profile(True)
    st.profile_read(reset=True)
    launches0 = llgpu.kernel_launches()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)

    def timed():
        if world > 1:
            torch.distributed.barrier()
        st.sync()
        ev0.record(stream)
        for _ in range(steps):
            st.reset(n)
            st.apply_ops(ops)
            st.flush()
        ev1.record(stream)
        st.sync()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    clocks = None
    if sampler_gpu is not None:
        with ClockSampler(sampler_gpu) as clk:
            timed()
        clocks = clk.summary()
    else:
        timed()
    launches = llgpu.kernel_launches() - launches0
    elapsed_ms = ev0.elapsed_time(ev1)
    prof = st.profile_read(reset=True)
    st.profile(False)
    value, slowest_s = replicas.job_rate(ngates * steps, elapsed_ms / 1e3, torch.distributed if world > 1 else None,
                                         device="cuda")
    elapsed_ms = slowest_s * 1e3
    tile_ms, tile_n = prof["tile"] if prof["tile"][1] else prof["gate"]
    peak, peak_kind = peaks()
    per_launch_s = (tile_ms / tile_n) / 1e3 if tile_n else float("nan")
    achieved = state_bytes * 2 / per_launch_s / 1e9 if tile_n else None
    res = {
        "value": value, "unit": "gates/s", "steps": steps, "warmup": warmup, "ms_per_step": elapsed_ms / steps,
        "gpu_launches": launches, "tile_passes": int(len(passes)), "tile_qubits": tile_q, "fusion": tuning,
        "phase_table_bytes": table_bytes,
        "autotune": tune, "state_bytes": state_bytes, "clocks": clocks,
        "sweeps_per_s": len(passes) * steps * world / (elapsed_ms / 1e3),
        "hbm_gbs_algorithmic": len(passes) * 2 * state_bytes * steps * world / (elapsed_ms / 1e3) / 1e9,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": profile_traffic(precision, n),
                     "kernel": (f"k_tile_reg<{TILE_POLICY.get(precision, precision)}> (register-tiled pass)"
                                if tuning["fuse_mode"] == "reg" else f"k_tile<{TILE_POLICY.get(precision, precision)}> (tile pass)"),
                     "launches": tile_n,
                     "mean_launch_ms": tile_ms / tile_n if tile_n else None, "peak_source": f"{peak_kind} hbm_gbs"},
        "kernel_ms_per_step": {k: v[0] / steps for k, v in prof.items()},
        "_xops": xops if tuning["fuse_mode"] != "none" else np.zeros(0, dtype=xops.dtype),
        "_tile_ms_step": prof["tile"][0] / steps,
    }
    if keep:
        return res, st
    st.close()
    return res


def finish_rooflines(res, precision, n, fma_rate):
    xops, tile_ms_step = res.pop("_xops"), res.pop("_tile_ms_step")
    sm = (res.get("clocks") or {}).get("sm_mhz")
    if is_f64(precision):
        res["fp64_roofline"] = fp64_roofline(n, xops, tile_ms_step, fma_rate)
    else:
        res["compute_roofline"] = compute_roofline(precision, n, xops, tile_ms_step, sm)
    return res


def run_ours(args, rank, world, local):
    import __graft_entry__

    __graft_entry__.build()
    import llgpu
    import workloads

    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        import torch

    n = args.qubits
    ops = workloads.layered_rotations(n, args.layers)
    ngates = len(ops)
    fma_rate = llgpu.fp64_fma_rate()
    head, st = measure_circuit(args, torch, args.precision, n, ops, args.steps, args.warmup, world,
                               sampler_gpu=local, keep=True)
    head = finish_rooflines(head, args.precision, n, fma_rate)
    clocks = head.pop("clocks")
    elem = ELEM_BYTES.get(args.precision, 16)
    _, xops_e2e, tables_e2e = plan_for(args.precision, n, ops, head["tile_qubits"], head["fusion"]["fuse_mode"] == "reg")

    # the same circuit in the other precisions, each compared with this (FP64) final state
    variants = None
    if not args.no_variants and is_f64(args.precision):
        variants = {}
        for prec in ("df64", "complex64"):
            vsteps = max(1, min(args.steps, E2E_STEPS_MAX))
            v, vst = measure_circuit(args, torch, prec, n, ops, vsteps, 2, world, keep=True)
            v = finish_rooflines(v, prec, n, fma_rate)
            v.pop("clocks", None)
            fid, dmax, amax = vst.compare_ex(st)
            v["vs_fp64"] = {"max_abs_diff": dmax, "one_minus_fidelity": 1.0 - fid, "max_abs_amp": amax,
                            "max_abs_diff_rel_to_max_amp": (dmax / amax) if amax else None}
            vst.close()
            if not args.no_e2e:
                _, vx, vtab = plan_for(prec, n, ops, v["tile_qubits"], v["fusion"]["fuse_mode"] == "reg")
                v["e2e"] = run_e2e(args, prec, ops, vx, vtab, n, ELEM_BYTES.get(prec, 16), world, torch)
            variants[prec] = v
    st.close()

    # end to end through the drop-in module: op records in, final amplitudes out, every step
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, args.precision, ops, xops_e2e, tables_e2e, n, elem, world, torch)

    sweeps = None
    if not args.no_sweeps:
        sweeps = run_sweep_bench(args, torch, fma_rate)

    adj = None
    if not args.no_adjoint:
        adj = run_adjoint_bench(args, torch)
    traj = batch = zne = config1 = tsolver = dmat = None
    cpu_ok = rank == 0 and world == 1 and not args.no_cpu_baseline
    if not args.no_forms:
        traj = run_traj_bench(args, torch, cpu=cpu_ok)
        batch = run_batch_bench(args, torch, cpu=cpu_ok)
        zne = run_zne_bench(args, torch, cpu=cpu_ok)
        config1 = run_config1_bench(args, torch, cpu=cpu_ok)
        tsolver = run_tsolver_bench(args, torch, cpu=cpu_ok)
        dmat = run_dm_bench(args, torch, cpu=cpu_ok)

    cpu = cpu_baseline(n, ops) if cpu_ok else None

    if rank != 0:
        return
    dtype = {"complex128": "f64", "fp64": "f64", "f64": "f64", "df64": "df64", "complex64": "c64"}.get(args.precision,
                                                                                                     args.precision)
    line = {
        "metric": METRIC, "value": head["value"], "unit": "gates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": dtype,
        "data": "synthetic (seeded layered circuit)",
        "config": {"workload": f"{n}-qubit complex128 layered circuit: {args.layers} layers of RX/RY/RZ on every "
                               f"qubit + CNOT brickwork, {ngates} gates, fused into {head['tile_passes']} shared-memory "
                               f"tile passes of {head['tile_qubits']} qubits", "qubits": n, "layers": args.layers,
                   "gates": ngates, "tile_passes": head["tile_passes"], "tile_qubits": head["tile_qubits"],
                   "precision": args.precision,
                   "arithmetic": "IEEE binary64 (FP64 pipe)" if is_f64(args.precision) else args.precision,
                   "fusion": head["fusion"], "autotune": head["autotune"],
                   "l2": f"inputs larger than L2 ({head['state_bytes'] / 2**30:g} GiB state), no flush needed"},
        "sweeps_per_s": head["sweeps_per_s"], "hbm_gbs_algorithmic": head["hbm_gbs_algorithmic"],
        "roofline": head["roofline"],
        "fp64_roofline": head.get("fp64_roofline"),
        "compute_roofline": head.get("compute_roofline"),
        "kernel_ms_per_step": head["kernel_ms_per_step"],
        "gpu_launches": head["gpu_launches"],
        "clocks": clocks,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "variants": variants,
        "gate_sweeps": sweeps,
        "adjoint": adj,
        "trajectories": traj,
        "mixed_batch": batch,
        "zne": zne,
        "config1_12q": config1,
        "trajectory_solver": tsolver,
        "density_matrix": dmat,
    }
    line["summary"] = summarize(line)
    print(json.dumps(line), flush=True)


def summarize(line: dict) -> dict:
    """The key figure of every measured form, repeated at the end of the line."""
    def get(d, *path):
        for p in path:
            if not isinstance(d, dict) or p not in d:
                return None
            d = d[p]
        return d

    return {
        "headline_gates_per_s": line["value"], "dtype": line["dtype"],
        "e2e_gates_per_s": get(line, "e2e", "value"),
        "fp64_roofline_frac": get(line, "fp64_roofline", "frac"), "hbm_roofline_frac": get(line, "roofline", "frac"),
        "cpu_gates_per_s": get(line, "cpu_baseline", "value"),
        "df64_gates_per_s": get(line, "variants", "df64", "value"),
        "df64_one_minus_fidelity": get(line, "variants", "df64", "vs_fp64", "one_minus_fidelity"),
        "complex64_gates_per_s": get(line, "variants", "complex64", "value"),
        "complex64_one_minus_fidelity": get(line, "variants", "complex64", "vs_fp64", "one_minus_fidelity"),
        "adjoint_grads_per_s": get(line, "adjoint", "grads_per_s"),
        "adjoint_speedup_vs_param_shift": get(line, "adjoint", "speedup_vs_param_shift"),
        "adjoint_df64_grads_per_s": get(line, "adjoint", "df64", "grads_per_s"),
        "trajectories_per_s_c128": get(line, "trajectories", "c128", "traj_per_s"),
        "trajectories_per_s_df64": get(line, "trajectories", "df64", "traj_per_s"),
        "trajectories_per_s_c64": get(line, "trajectories", "c64", "traj_per_s"),
        "mixed_batch_circuits_per_s_c128": get(line, "mixed_batch", "c128", "circuits_per_s"),
        "mixed_batch_circuits_per_s_df64": get(line, "mixed_batch", "df64", "circuits_per_s"),
        "mixed_batch_circuits_per_s_c64": get(line, "mixed_batch", "c64", "circuits_per_s"),
        "zne_traj_per_s": get(line, "zne", "traj_per_s"),
        "complex128_gate_sweep_hbm_frac": {k: round(v["frac"], 3) for k, v in (get(line, "gate_sweeps", "complex128") or {}).items()
                                           if isinstance(v, dict) and "frac" in v and not k.startswith("block")} or None,
        "complex128_dense_block_ms": {k: round(v["ms_per_sweep"], 2) for k, v in (get(line, "gate_sweeps", "complex128") or {}).items()
                                      if k.startswith("block")} or None,
        "block5_tensor_core_hbm_frac": get(line, "gate_sweeps", "df64", "block5", "frac"),
        "dm_depolarizing_2q_df64_hbm_frac": get(line, "density_matrix", "df64_n13", "depolarizing_2q", "frac_of_hbm"),
    }


def run_adjoint_bench(args, torch):
    """Adjoint gradients of the 20-qubit, 10-layer RY/RZ + CZ-ring ansatz (400 parameters,
    observable sum_i Z_i Z_{i+1} periodic) for a batch of 64 parameter sets, against the
    parameter-shift rule evaluated on the same GPU (batched shifted circuits) for one set; in IEEE
    complex128 (the headline) and in double-float (`df64`)."""
    out = adjoint_once(args, torch, args.precision)
    if is_f64(args.precision):
        out["df64"] = adjoint_once(args, torch, "df64")
        # the double-float gradients against the IEEE FP64 ones, relative to the largest gradient
        g64, gdf = out.pop("_grads"), out["df64"].pop("_grads")
        scale = float(np.max(np.abs(g64)))
        out["df64"]["vs_fp64"] = {"max_abs_grad_diff": float(np.max(np.abs(gdf - g64))),
                                  "max_abs_grad_diff_rel_to_max_grad": float(np.max(np.abs(gdf - g64))) / scale
                                  if scale else None}
    out.pop("_grads", None)
    return out


def adjoint_once(args, torch, precision):
    import llgpu
    import workloads

    n, layers, batch = 20, 10, 64
    ops = workloads.hea_ansatz(n, layers)
    nparams = layers * 2 * n
    params = workloads.hea_params(n, layers, batch)
    adj = llgpu.Adjoint(n, ops, nparams, llgpu.ring_zz_terms(n), max_batch=batch, precision=precision)
    stream = torch.cuda.ExternalStream(adj.stream)
    for _ in range(2):
        adj.run(params)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(1, args.steps)
    ev0.record(stream)
    for _ in range(reps):
        e, g = adj.run(params)
    ev1.record(stream)
    ev1.synchronize()
    t_adj = ev0.elapsed_time(ev1) / 1e3 / reps
    adj.param_shift(params[:1])  # warm-up
    ev0.record(stream)
    e_ps, g_ps = adj.param_shift(params[:1])
    ev1.record(stream)
    ev1.synchronize()
    t_ps = ev0.elapsed_time(ev1) / 1e3
    info = adj.info()
    adj.close()
    grads_adj = batch * nparams / t_adj
    grads_ps = nparams / t_ps
    return {"workload": f"{n}-qubit hardware-efficient ansatz, {layers} layers RY/RZ + CZ ring, {nparams} "
                        f"parameters, batch {batch}, observable sum Z_i Z_i+1",
            "grads_per_s": grads_adj, "param_shift_grads_per_s": grads_ps, "speedup_vs_param_shift": grads_adj / grads_ps,
            "adjoint_s_per_batch": t_adj, "param_shift_s_per_set": t_ps,
            "max_abs_grad_diff_vs_param_shift": float(np.max(np.abs(g[0] - g_ps[0]))),
            "forward_passes": info["forward_passes"], "backward_passes": info["backward_passes"],
            "precision": precision, "_grads": np.array(g)}


def run_sweep_bench(args, torch, fma_rate=None):
    """Per-gate streaming sweeps on the 30-qubit state (the reference's one-pass-per-gate method):
    each gate kind on several target qubits, timed per launch with CUDA events on the engine's
    stream.  Algorithmic bytes per sweep: 32 B x 2^n for 1-qubit gates (read + write every
    amplitude), 16 B x 2^n for CNOT (the control = 1 half), 8 B x 2^n for CZ (one quarter)."""
    import llgpu
    from llgpu import OP_CNOT, OP_CZ, OP_H, OP_RX, OP_RY, OP_RZ, OP_U2, make_ops

    n = args.qubits
    peak, peak_kind = peaks()
    u = np.array([[0.6 + 0.1j, 0.3 - 0.2j], [-0.3 - 0.2j, 0.6 - 0.1j]], dtype=complex)
    u, _ = np.linalg.qr(u)
    targets = [0, 5, 13, 22, n - 1]
    kinds = {"RX": [(OP_RX, q, 0, 0.7) for q in targets], "RY": [(OP_RY, q, 0, 1.1) for q in targets],
             "RZ": [(OP_RZ, q, 0, 0.4) for q in targets], "H": [(OP_H, q) for q in targets],
             "U2": [(OP_U2, q, 0, 0.0, None, u.reshape(4)) for q in targets],
             "CNOT": [(OP_CNOT, 0, n - 1), (OP_CNOT, n - 1, 0), (OP_CNOT, 12, 13), (OP_CNOT, 3, 20)],
             "CZ": [(OP_CZ, 0, n - 1), (OP_CZ, 12, 13), (OP_CZ, 3, 20)]}
    bytes_per = {"CNOT": 16, "CZ": 8}
    out = {"qubits": n, "peak_gbs": peak, "peak_source": f"{peak_kind} hbm_gbs",
           "bytes_basis": "amplitudes each launch reads and writes (32 B x 2^n for a pair pass, 16 B x 2^n for "
                          "the IEEE complex128 RZ, which rewrites only the |1> half, 16 / 8 B x 2^n for CNOT / CZ)"}
    for prec in ("complex128", "df64"):
        st = llgpu.State(n, prec)
        st.set_fusion("none")
        res = {}
        for name, recs in kinds.items():
            ops = make_ops(recs)
            if prec == "complex128" and name not in bytes_per:
                # IEEE complex128 flushes run the per-gate lowering that carries the gates' real
                # factors (and RZ's global phase) and absorbs them in one op of the flush: its
                # launches move the bytes of the ops it exports
                _, xs = llgpu.plan_export(n, ops, n, stream=True)
                sweep_bytes = sum(16 if int(k) == 13 else 32 for k in xs["kind"]) * (1 << n) / len(xs)
                flush_ops = {str(int(k)): int(c) for k, c in zip(*np.unique(xs["kind"], return_counts=True))}
            else:
                sweep_bytes = bytes_per.get(name, 32) * (1 << n)
                flush_ops = None
            st.apply_ops(ops)  # warm-up
            st.sync()
            st.profile(True)
            st.profile_read(reset=True)
            for _ in range(2):
                st.apply_ops(ops)
            st.sync()
            ms, cnt = st.profile_read(reset=True)["gate"]
            st.profile(False)
            per = ms / cnt / 1e3
            gbs = sweep_bytes / per / 1e9
            res[name] = {"ms_per_sweep": per * 1e3, "gbs": gbs, "frac": gbs / peak}
            if flush_ops:
                res[name]["flush_ops_by_kind"] = flush_ops
            if name in bytes_per:
                # per (control, target): with qubit 0 among the touched bits, touched and untouched
                # amplitudes share every 32-byte sector, so DRAM moves twice the algorithmic bytes
                cases = []
                for rec in recs:
                    one = make_ops([rec])
                    st.profile(True)
                    st.profile_read(reset=True)
                    for _ in range(2):
                        st.apply_ops(one)
                    st.sync()
                    ms1, cnt1 = st.profile_read(reset=True)["gate"]
                    st.profile(False)
                    g1 = bytes_per[name] * (1 << n) / (ms1 / cnt1 / 1e3) / 1e9
                    cases.append({"qubits": [rec[1], rec[2]], "gbs": g1, "frac": g1 / peak})
                res[name]["cases"] = cases
        # dense k-qubit blocks (llg_apply_matrix): 32 B x 2^n per application and 8 x 4^k x 2^(n-k)
        # real FLOP of complex multiply-adds
        rng = np.random.default_rng(17)
        for k, qs in ((2, [0, n - 1]), (3, [0, 15, n - 1]), (4, [0, 11, 20, n - 1]), (5, [0, 7, 13, 22, n - 1])):
            m, _ = np.linalg.qr(rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k)))
            st.apply_matrix(qs, m)  # warm-up
            st.sync()
            st.profile(True)
            st.profile_read(reset=True)
            for _ in range(2):
                st.apply_matrix(qs, m)
            st.sync()
            ms, cnt = st.profile_read(reset=True)["gate"]
            st.profile(False)
            per = ms / cnt / 1e3
            gbs = 32 * (1 << n) / per / 1e9
            tflops = 8 * (4 ** k) * (1 << (n - k)) / per / 1e12
            res[f"block{k}"] = {"ms_per_sweep": per * 1e3, "gbs": gbs, "frac": gbs / peak, "tflops": tflops, "qubits": qs}
            if prec == "complex128" and fma_rate:
                # the dense FP64 forms are bound by the FP64 pipe: 2 FLOP per multiply-add
                res[f"block{k}"]["fp64_frac"] = tflops * 1e12 / (2 * fma_rate)
        st.close()
        out[prec] = res
    return out


def _timed(stream, torch, fn, reps=1):
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(reps):
        out = fn()
    ev1.record(stream)
    ev1.synchronize()
    return ev0.elapsed_time(ev1) / 1e3 / reps, out


def run_traj_bench(args, torch, cpu: bool):
    """4096 noisy trajectories of the 14-qubit, 8-layer RX/RY + CNOT-chain circuit with amplitude
    damping (0.01) then dephasing (0.005) after every gate on touched qubits; complex128 and
    complex64; the CPU figure runs the oracle's restatement of the same step on every core."""
    import llgpu
    import workloads

    n, ntraj, gamma, lam, seed = 14, 4096, 0.01, 0.005, 2024
    ops = workloads.noisy_layers(n, 8)
    out = {"workload": f"{ntraj} trajectories x {n} qubits, {len(ops)} gates, {llgpu.noise_sites(ops)} noise sites "
                       f"(amplitude damping {gamma} then dephasing {lam})"}
    for prec in ("complex128", "df64", "complex64"):
        # a handle planned once; the autotuner picks cluster split and CTA threads, and every
        # launch replays the captured CUDA graph (outputs copied to host inside the timing)
        h = llgpu.Traj(n, ops, gamma, lam, ntraj, prec)
        default_cfg = h.config()
        h.launch(seed, 256)
        t0 = time.perf_counter()
        h.launch(seed, ntraj)
        dt_default = time.perf_counter() - t0
        tune = h.autotune()
        h.launch(seed, 256)
        t0 = time.perf_counter()
        z, j, _ = h.launch(seed, ntraj)
        dt = time.perf_counter() - t0
        key = {"complex128": "c128", "df64": "df64", "complex64": "c64"}[prec]
        out[key] = {"traj_per_s": ntraj / dt, "seconds": dt, "mean_z0": float(z.mean()),
                    "std_error": float(z.std(ddof=1) / np.sqrt(ntraj)), "jumps_per_traj": float(j.mean()),
                    "config": h.config(), "default_config": default_cfg,
                    "default_traj_per_s": ntraj / dt_default, "autotune": tune, "_z": z}
        h.close()
    # every trajectory's <Z0> in double-float and complex64 against IEEE complex128 (same Philox
    # draws, so the same jumps unless a decision margin is below the arithmetic's error)
    z128 = out["c128"].pop("_z")
    for key in ("df64", "c64"):
        zk = out[key].pop("_z")
        out[key]["vs_fp64"] = {"max_abs_z0_diff": float(np.max(np.abs(zk - z128))),
                               "mean_z0_diff": float(abs(zk.mean() - z128.mean()))}
    if cpu:
        import oracle

        oracle.set_threads(os.cpu_count() or 1)
        sample = 64
        t0 = time.perf_counter()
        oracle.traj_run(n, ops, gamma, lam, seed, 0, sample)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": sample / dt, "unit": "traj/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": f"first {sample} trajectories, oracle restatement of the Kraus-jump step"}
    return out


def run_config1_bench(args, torch, cpu: bool):
    """The published 12-qubit workload: 1000 ops, H (p = 0.5) on a uniform qubit else CNOT on a
    uniform distinct pair, from |0..0>, amplitudes read back.  The autotuner picks the tile width
    (the 64 KiB state fits one tile, but 9- or 10-qubit tiles spread each pass over 8 or 4 SMs).
    Reported: time per circuit between CUDA events on the engine's stream around reset, apply_ops
    and flush (host planning and launches included), end to end through quantum_sim_v3 with the op
    list in one call and with one Python call per gate (each with the full host readback), and the
    published reference time."""
    import llgpu
    import quantum_sim_v3
    import workloads
    from llgpu import OP_CNOT, OP_H

    n, reps = 12, 50
    ops = workloads.mixed_h_cnot(n, 1000, seed=1234)
    st = llgpu.State(n)
    tune = st.autotune(ops)  # tile width and CTA threads for this small register
    stream = torch.cuda.ExternalStream(st.stream)

    def one():
        st.reset(n)
        st.apply_ops(ops)
        st.flush()

    one()
    st.sync()
    launches0 = llgpu.kernel_launches()
    dt, _ = _timed(stream, torch, one, reps=reps)
    launches = (llgpu.kernel_launches() - launches0) / reps
    got = st.state()
    st.close()
    sv = quantum_sim_v3.StateVector(n)
    sv.autotune(ops)  # the cached result
    sv.get_numpy_view()
    t0 = time.perf_counter()
    for _ in range(reps):
        sv.reset(n)
        sv.apply_ops(ops)
        view = sv.get_numpy_view()
    e2e_batch = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        sv.reset(n)
        for o in ops:
            if o["kind"] == OP_H:
                sv.h(int(o["q0"]))
            else:
                sv.cnot(int(o["q0"]), int(o["q1"]))
        view = sv.get_numpy_view()
    e2e_calls = (time.perf_counter() - t0) / reps
    res = {"workload": "12 qubits, 1000 ops (H p=0.5 else CNOT), seed 1234, from |0..0>", "device_ms": dt * 1e3,
           "launches_per_circuit": launches, "e2e_ms_op_list": e2e_batch * 1e3, "e2e_ms_per_gate_calls": e2e_calls * 1e3,
           "autotune": tune,
           "ops_per_s_device": 1000 / dt, "published_reference_ms": 25.91,
           "published_reference_note": "8 cores, README.md:17-27 / docs/RESULTS.md:19-25"}
    del view
    if cpu:
        import oracle

        want = oracle.run_ops(n, ops)
        res["max_abs_diff_vs_oracle"] = float(np.max(np.abs(got - want)))
        for threads in (1, os.cpu_count() or 1):
            oracle.set_threads(threads)
            best = 1e9
            for _ in range(5):
                t0 = time.perf_counter()
                oracle.run_ops(n, ops)
                best = min(best, time.perf_counter() - t0)
            res[f"cpu_ms_{threads}t"] = best * 1e3
    return res


def run_tsolver_bench(args, torch, cpu: bool):
    """The dense trajectory solver: (a) the reference's published case, 1 qubit, T1 = 2 amplitude
    damping from |1>, STANDARD, duration 2, dt 0.02, 20000 trajectories (published: 0.00635 ms per
    trajectory on 2 cores); (b) 10 qubits (dim 1024), random Hermitian H, sigma_- on qubit 0 and Z
    on qubit 1, PROJECTOR, 20 steps, 1024 trajectories: one dense complex matrix-vector product per
    step and trajectory, 8 dim^2 real FLOP, FP64."""
    import llgpu

    sm = np.array([[0, 1], [0, 0]], dtype=complex)
    res = {}
    s = llgpu.TrajectorySolver(1)
    s.add_lindblad(sm, 0.5)
    p1 = np.diag([0.0, 1.0])
    s.estimate_observable([0, 1], 2.0, 0.02, 2000, "STANDARD", p1, seed=1)  # warm-up
    t0 = time.perf_counter()
    e = s.estimate_observable([0, 1], 2.0, 0.02, 20000, "STANDARD", p1, seed=101)
    dt1 = time.perf_counter() - t0
    s.close()
    res["one_qubit_t1"] = {"ms_per_trajectory": dt1 / 20000 * 1e3, "trajectories_per_s": 20000 / dt1,
                           "mean_p1": e["mean"], "exact": float(np.exp(-1.0)), "std_error": e["std_error"],
                           "published_reference_ms_per_trajectory": 0.00635,
                           "published_note": "2 cores, docs/trajectory_benchmark.json:221"}
    rng = np.random.default_rng(11)
    d, steps, ntraj = 1024, 20, 1024
    a = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    h = (a + a.conj().T) / (4 * np.sqrt(d))
    s = llgpu.TrajectorySolver(10)
    s.set_hamiltonian(h)
    s.add_lindblad(np.kron(np.eye(d // 2), sm), 0.4)
    s.add_lindblad(np.diag(np.where(np.arange(d) & 2, -1.0, 1.0)).astype(complex), 0.3)
    psi0 = rng.normal(size=d) + 1j * rng.normal(size=d)
    s.states(psi0, 0.02 * steps, 0.02, 64, "PROJECTOR", seed=4)  # warm-up (plan + kernel)
    t0 = time.perf_counter()
    st = s.states(psi0, 0.02 * steps, 0.02, ntraj, "PROJECTOR", seed=5)
    dt10 = time.perf_counter() - t0
    plan = s.plan()
    flop = 8.0 * d * d * steps * ntraj
    res["ten_qubit_dense"] = {"trajectories_per_s": ntraj / dt10, "seconds": dt10, "steps": steps,
                              "tflops_fp64_incl_plan": flop / dt10 / 1e12,
                              "note": "seconds include the plan (expm of the 1024 x 1024 H_eff on the GPU) "
                                      "and the host copy of all final states"}
    if cpu:
        import oracle

        oracle.set_threads(os.cpu_count() or 1)
        sample = 32
        t0 = time.perf_counter()
        oracle.tsolver_run(plan, psi0, 5, 0, sample)
        dtc = time.perf_counter() - t0
        res["ten_qubit_dense"]["cpu_baseline"] = {"value": sample / dtc, "unit": "traj/s", "cores": os.cpu_count(),
                                                  "kind": "port", "sample": f"{sample} trajectories, oracle "
                                                  "restatement of the solver's jump step with the GPU's plan"}
    del st
    s.close()
    return res


def run_zne_bench(args, torch, cpu: bool):
    """Zero-noise extrapolation with the reference NoisyBackend's depolarizing model: a 12-qubit,
    4-layer RX/RY + CNOT-chain circuit (100 gates), p = 0.005 per site, fold scales {1, 3, 5},
    4096 trajectories per scale, observable sum_i Z_i Z_i+1 (ring); complex128."""
    import llgpu
    import workloads

    n, p, scales, ntraj, seed = 12, 0.005, [1, 3, 5], 4096, 909
    ops = workloads.noisy_layers(n, 4)
    terms = [(q, (q + 1) % n, 1.0) for q in range(n)]
    llgpu.zne(n, ops, p, scales, 256, seed, terms)  # warm-up (module load, first launches)
    t0 = time.perf_counter()
    r = llgpu.zne(n, ops, p, scales, ntraj, seed, terms)
    dt = time.perf_counter() - t0
    st = llgpu.State(n)
    st.apply_ops(ops)
    ideal = st.expect_zz([t[0] for t in terms], [t[1] for t in terms], [t[2] for t in terms])
    st.close()
    total = ntraj * len(scales)
    res = {"workload": f"ZNE: {n} qubits, {len(ops)} gates, p = {p}, scales {scales}, {ntraj} trajectories per "
                       f"scale, observable ring ZZ", "traj_per_s": total / dt, "seconds": dt,
           "value": r["value"], "std_error": r["std_error"], "values": [float(v) for v in r["values"]],
           "ideal": ideal, "unmitigated_error": abs(float(r["values"][0]) - ideal),
           "mitigated_error": abs(r["value"] - ideal)}
    if cpu:
        import oracle

        oracle.set_threads(os.cpu_count() or 1)
        sample = 64
        t0 = time.perf_counter()
        for s in scales:
            oracle.noisy_run(n, ops, p, s, seed, 0, sample, terms)
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": sample * len(scales) / dt, "unit": "traj/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": f"{sample} trajectories per scale, oracle restatement of "
                                                         "NoisyBackend with folding"}
    return res


def run_dm_bench(args, torch, cpu: bool):
    """Density matrices (the reference's KrausChannel::apply, src/Noise.cpp:174-258): rho on n
    qubits is a 2n-qubit state.  Amplitude damping (gamma 0.01) on every qubit is a 2-qubit block
    Sum_k K (x) conj(K) on (q, q + n); 2-qubit depolarizing (p 0.01) on (q, q + 1) a 4-qubit block.
    n = 10 is the reference's limit (MAX_DM_QUBITS, a 16 MiB state); n = 13 is a 1 GiB state, larger
    than L2.  Algorithmic bytes per channel: 32 B x 4^n (every element read and written)."""
    import llgpu

    peak, _ = peaks()
    ad = llgpu.amplitude_damping(0.01)
    dp = llgpu.depolarizing(0.01, 2)
    out = {"workload": "density matrices: amplitude damping on every qubit and 2-qubit depolarizing on "
                       "neighbouring pairs, complex128 (IEEE FP64); df64_n13: the 13-qubit case in double-float, "
                       "whose 2-qubit channels run on the tensor cores"}
    for prec, n in (("complex128", 10), ("complex128", 13), ("df64", 13)):
        dm = llgpu.DensityMatrix(n, prec)
        dm.apply_ops(llgpu.make_ops([(llgpu.OP_H, q) for q in range(n)] + [(llgpu.OP_RX, q, 0, 0.3 * q) for q in range(n)]))
        st = dm.state
        res = {"state_bytes": 16 << (2 * n)}
        for name, kops, tg in (("amplitude_damping_1q", ad, [[q] for q in range(n)]),
                               ("depolarizing_2q", dp, [[q, q + 1] for q in range(n - 1)])):
            for t in tg[:2]:
                dm.kraus(kops, t)  # warm-up
            st.sync()
            st.profile(True)
            st.profile_read(reset=True)
            t0 = time.perf_counter()
            reps = 3
            for _ in range(reps):
                for t in tg:
                    dm.kraus(kops, t)
            st.sync()
            wall = time.perf_counter() - t0
            ms, cnt = st.profile_read(reset=True)["gate"]
            st.profile(False)
            per = ms / max(1, cnt) / 1e3
            gbs = 32 * (1 << (2 * n)) / per / 1e9
            res[name] = {"channels": reps * len(tg), "kernel_ms_per_channel": per * 1e3,
                         "channels_per_s_wall": reps * len(tg) / wall, "gbs": gbs, "frac_of_hbm": gbs / peak,
                         "block_qubits": 2 * len(tg[0])}
        tr = dm.trace()
        res["trace_minus_1"] = abs(tr - 1.0)
        dm.close()
        out[f"n{n}" if prec == "complex128" else f"{prec}_n{n}"] = res
    if cpu:
        # the oracle's restatement timed on one channel of each kind at the reference's size; its
        # result is also compared with the GPU's on the same input
        import oracle

        n = 10
        rng = np.random.default_rng(5)
        a = rng.normal(size=(1 << n, 1 << n)) + 1j * rng.normal(size=(1 << n, 1 << n))
        rho = a @ a.conj().T
        rho /= np.trace(rho)
        dm = llgpu.DensityMatrix(n, "complex128", rho=rho)
        dm.kraus(ad, [3])
        dm.kraus(dp, [4, 5])
        got = dm.rho()
        dm.close()
        t0 = time.perf_counter()
        want = oracle.kraus_apply(rho, n, ad, [3])
        t1 = time.perf_counter()
        want = oracle.kraus_apply(want, n, dp, [4, 5])
        t2 = time.perf_counter()
        out["max_abs_diff_vs_oracle_n10"] = float(np.max(np.abs(got - want)))
        out["cpu_baseline"] = {"value": 2.0 / (t2 - t0), "unit": "channels/s", "cores": 1, "kind": "port",
                               "sample": "one amplitude-damping and one 2-qubit depolarizing channel on a "
                                         "10-qubit rho, oracle restatement of KrausChannel::apply",
                               "ms_amplitude_damping": (t1 - t0) * 1e3, "ms_depolarizing_2q": (t2 - t1) * 1e3}
    return out


def run_batch_bench(args, torch, cpu: bool):
    """512 circuits with n uniform in 10..22 and 200 random gates each in one persistent launch;
    complex128 and complex64 with the per-circuit fidelity of the complex64 result."""
    import llgpu
    import workloads

    nq, ops, off = workloads.mixed_batch(512, 10, 22, 200)
    ngates = int(off[-1])
    res = {"workload": f"512 circuits, n in 10..22 (total {int(np.sum(2.0 ** nq))} amplitudes), 200 gates each"}
    batches = {}
    for prec in ("complex128", "df64", "complex64"):
        tune = llgpu.batch_autotune(nq, ops, off, prec)  # tile width by measurement (cached)
        b = llgpu.Batch(nq, ops, off, prec, llgpu.TUNE_AUTO)
        stream = torch.cuda.ExternalStream(b.stream)
        b.run()  # captures the CUDA graph; later runs replay it
        dt, _ = _timed(stream, torch, b.run, reps=max(1, args.steps))
        key = {"complex128": "c128", "df64": "df64", "complex64": "c64"}[prec]
        info = b.info()
        res[key] = {"circuits_per_s": 512 / dt, "gates_per_s": ngates / dt, "seconds": dt,
                    "work_items": info["work_items"], "tile_qubits": info["tile_qubits"],
                    "autotune": tune}
        batches[key] = b
    f = batches["c64"].fidelity(batches["c128"])
    res["c64_fidelity_error"] = {"max": float(np.max(1 - f[:, 0])), "median": float(np.median(1 - f[:, 0]))}
    f = batches["df64"].fidelity(batches["c128"])
    res["df64_fidelity_error"] = {"max": float(np.max(1 - f[:, 0])), "median": float(np.median(1 - f[:, 0]))}
    for b in batches.values():
        b.close()
    if cpu:
        import oracle

        oracle.set_threads(os.cpu_count() or 1)
        idx = list(range(0, 512, 32))  # 16 circuits spread over the batch
        t0 = time.perf_counter()
        for i in idx:
            oracle.run_ops(int(nq[i]), ops[off[i]:off[i + 1]])
        dt = time.perf_counter() - t0
        frac = float(np.sum(2.0 ** nq[idx]) / np.sum(2.0 ** nq))  # share of the batch's work in the sample
        res["cpu_baseline"] = {"value": 512 / (dt / frac), "unit": "circuits/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": f"circuits {idx[0]}..{idx[-1]} step 32, scaled to the batch by amplitude count"}
    return res


def run_e2e(args, precision, ops, xops, table_bytes, n, elem, world, torch):
    import quantum_sim_v3

    sv = quantum_sim_v3.StateVector(n, precision)
    if args.tile < 0:
        sv.autotune(ops, 4 * len(ops) // max(1, args.layers))  # the headline's tuning, from the cache
    else:
        sv.set_fusion("tile", args.tile)
    sv.apply_ops(ops)
    sv.get_numpy_view()  # allocates the pinned host mirror once
    steps = max(1, min(args.steps, E2E_STEPS_MAX))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        sv.reset(n)
        sv.apply_ops(ops)
        view = sv.get_numpy_view()  # flushes the queued gates; the last pass also fills the host mirror
    _ = float(view[0].real)
    t1 = time.perf_counter()
    # untimed breakdown of one step: the passes alone (flushed and synchronised), then the readback
    # with nothing queued
    a = time.perf_counter()
    sv.reset(n)
    sv.apply_ops(ops)
    sv.flush()
    torch.cuda.synchronize()
    b = time.perf_counter()
    view = sv.get_numpy_view()
    c = time.perf_counter()
    del sv, view
    return {"value": len(ops) * steps * world / (t1 - t0), "unit": "gates/s", "steps": steps,
            "ms_per_step": 1e3 * (t1 - t0) / steps, "passes_alone_ms": 1e3 * (b - a), "readback_alone_ms": 1e3 * (c - b),
            "h2d_bytes_per_step": int(xops.nbytes + table_bytes),
            "h2d_note": "the planned executor ops and phase tables uploaded by the flush",
            "d2h_bytes_per_step": int((1 << n) * 16),
            "api": "quantum_sim_v3.StateVector: reset, apply_ops, get_numpy_view (host copy of all amplitudes; "
                   "the last tile pass writes the pinned host mirror as it stores its tiles)"}


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
