#!/usr/bin/env python
"""Benchmark: 30-qubit complex128 layered circuit on one GB300 (the headline workload).

Workload (seeded, synthetic): a 30-qubit state from |0..0> (16 GiB of complex128), 20 layers of
RX, RY, RZ on every qubit (angles U[0, 2pi)) plus a CNOT brickwork on (i, i+1) with alternating
offsets -- 1800 rotations + 290 CNOTs = 2090 gates.  One step = reset the state and run the whole
circuit through the engine (fused shared-memory tile passes, complex128 as double-float).

Printed as one JSON line:
  value        gates/s over the whole job (logical, pre-fusion gates), device-timed with CUDA
               events on the engine's stream, inputs resident in HBM;
  e2e          the same metric through the drop-in API (quantum_sim_v3.StateVector) with the
               final amplitudes read back to host memory (get_numpy_view) every step;
  roofline     the dominant kernel (the tile pass): algorithmic bytes per launch (32 B x 2^30
               amplitudes: one read and one write of the state) / its mean launch time, measured
               with CUDA events around every launch inside the timed region;
  cpu_baseline the reference's per-gate algorithm (the oracle's restatement of
               ll::StateVectorBackend, OpenMP on every host core) on the first gates of the same
               30-qubit circuit.
`--impl reference` times that CPU implementation alone as the reference arm.

Beside the headline the line carries, each with its own workload description and, where the
oracle can run a sample of it, a CPU baseline: per-gate and dense-block sweeps against HBM
(`gate_sweeps`), adjoint gradients against parameter shift (`adjoint`), noisy trajectories
(`trajectories`), mixed circuit batches (`mixed_batch`), zero-noise extrapolation (`zne`), the
12-qubit published workload (`config1_12q`), the dense trajectory solver (`trajectory_solver`) and
density-matrix channels (`density_matrix`).  `--no-sweeps`, `--no-adjoint`, `--no-forms` skip them.

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


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--layers", type=int, default=20)
    ap.add_argument("--precision", default="complex128")
    ap.add_argument("--tile", type=int, default=-1,
                    help="tile width in qubits; -1 (default): the autotuner picks width and CTA threads")
    ap.add_argument("--cta-threads", type=int, default=0, help="tile-kernel CTA threads with an explicit --tile")
    ap.add_argument("--cpu-gates", type=int, default=12, help="gates in each CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
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
# CPU side: the reference's per-gate algorithm (oracle restatement), bounded sample
# --------------------------------------------------------------------------------------------
def cpu_sample(n: int, ops: np.ndarray, gates: int, reps: int, warm: int):
    """Times `gates` gates of the circuit on an n-qubit state with every host core; returns
    (gates/s best-of, threads, seconds per sample)."""
    import oracle

    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    psi = oracle.zero_state(n)
    sample = np.ascontiguousarray(ops[:gates])
    times = []
    for k in range(warm + reps):
        t0 = time.perf_counter()
        rc = oracle.lib().orc_run_ops(psi.ctypes.data, n, sample.ctypes.data, sample.size)
        t1 = time.perf_counter()
        if rc:
            raise RuntimeError("oracle rejected the sample")
        if k >= warm:
            times.append(t1 - t0)
    best = min(times)
    return gates / best, threads, best, times


def run_reference(args, rank, world):
    if rank != 0:
        return
    import workloads

    ops = workloads.layered_rotations(args.qubits, args.layers)
    warm = max(1, args.warmup)
    rate, threads, best, times = cpu_sample(args.qubits, ops, args.cpu_gates, args.steps, warm)
    sample = (f"first {args.cpu_gates} gates of the {args.qubits}-qubit layered circuit per step, "
              f"{args.steps} steps after {warm} warm-up; per-gate OpenMP passes of the reference algorithm")
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "gates/s", "n_gpus": world,
        "steps": args.steps, "warmup": warm, "ms_per_step": 1e3 * statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.qubits}-qubit complex128 layered circuit ({args.layers} layers), "
                               f"per-gate CPU sample", "qubits": args.qubits, "layers": args.layers},
        "cpu_baseline": {"value": rate, "unit": "gates/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": "gates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------------------------
# GPU side
# --------------------------------------------------------------------------------------------
def run_ours(args, rank, world, local):
    import __graft_entry__

    __graft_entry__.build()
    import llgpu
    import workloads

    torch = None
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
    st = llgpu.State(n, args.precision)
    tune = None
    if args.tile < 0:
        # autotuner: two layers of the circuit on a scratch state, outside the timed region
        tune = st.autotune(ops, sample_ops=2 * len(ops) // max(1, args.layers))
    else:
        st.set_fusion("tile", args.tile)
        st.set_tile_threads(args.cta_threads)
    tuning = st.tuning()
    tile_q = tuning["tile_qubits"]
    passes, xops = llgpu.plan_export(n, ops, tile_q, zyz=args.precision == "complex128")
    if tuning["fuse_mode"] == "none":
        passes = np.zeros(ngates)  # one streaming pass per gate
    elem = 8 if args.precision == "complex64" else 16
    state_bytes = elem * (1 << n)

    stream = torch.cuda.ExternalStream(st.stream)
    # warm-up
    for _ in range(args.warmup):
        st.reset(n)
        st.apply_ops(ops)
        st.flush()
    st.sync()
    st.profile(True)
    st.profile_read(reset=True)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    launches0 = llgpu.kernel_launches()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        st.sync()
        ev0.record(stream)
        for _ in range(args.steps):
            st.reset(n)
            st.apply_ops(ops)
            st.flush()
        ev1.record(stream)
        st.sync()
        torch.cuda.synchronize()
        barrier()
    launches = llgpu.kernel_launches() - launches0
    elapsed_ms = ev0.elapsed_time(ev1)
    prof = st.profile_read(reset=True)
    st.profile(False)
    # replicas: every rank ran the same circuit on its own state; the job's rate is all ranks'
    # gates over the slowest rank's time
    import replicas

    value, slowest_s = replicas.job_rate(ngates * args.steps, elapsed_ms / 1e3,
                                         torch.distributed if world > 1 else None, device="cuda")
    elapsed_ms = slowest_s * 1e3
    ms_step = elapsed_ms / args.steps

    tile_ms, tile_n = prof["tile"] if prof["tile"][1] else prof["gate"]
    peak, peak_kind = peaks()
    per_launch_s = (tile_ms / tile_n) / 1e3 if tile_n else float("nan")
    achieved = state_bytes * 2 / per_launch_s / 1e9 if tile_n else None
    # the committed ncu capture is of the complex128 (double-float) tile pass at this workload
    traffic = profile_traffic() if args.precision == "complex128" and n == 30 else None
    st.close()

    # end to end through the drop-in module: op records in, final amplitudes out, every step
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, ops, xops, n, elem, world, torch)

    sweeps = None
    if not args.no_sweeps:
        sweeps = run_sweep_bench(args, torch)

    adj = None
    if not args.no_adjoint:
        adj = run_adjoint_bench(args, torch)
    traj = batch = zne = config1 = tsolver = dmat = None
    if not args.no_forms:
        traj = run_traj_bench(args, torch, cpu=(rank == 0 and world == 1 and not args.no_cpu_baseline))
        batch = run_batch_bench(args, torch, cpu=(rank == 0 and world == 1 and not args.no_cpu_baseline))
        zne = run_zne_bench(args, torch, cpu=(rank == 0 and world == 1 and not args.no_cpu_baseline))
        config1 = run_config1_bench(args, torch, cpu=(rank == 0 and world == 1 and not args.no_cpu_baseline))
        tsolver = run_tsolver_bench(args, torch, cpu=(rank == 0 and world == 1 and not args.no_cpu_baseline))
        dmat = run_dm_bench(args, torch, cpu=(rank == 0 and world == 1 and not args.no_cpu_baseline))

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rate, threads, best, _ = cpu_sample(n, ops, args.cpu_gates, 1, 1)
        cpu = {"value": rate, "unit": "gates/s", "cores": threads, "kind": "port",
               "sample": f"first {args.cpu_gates} gates of the same {n}-qubit circuit, best of 1 after 1 warm-up, "
                         f"{best:.1f} s per sample; oracle restatement of ll::StateVectorBackend (OpenMP)"}

    if rank != 0:
        return
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": "gates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "df64" if args.precision == "complex128" else args.precision,
        "data": "synthetic (seeded layered circuit)",
        "config": {"workload": f"{n}-qubit complex128 layered circuit: {args.layers} layers of RX/RY/RZ on every "
                               f"qubit + CNOT brickwork, {ngates} gates, fused into {len(passes)} shared-memory tile "
                               f"passes of {tile_q} qubits", "qubits": n, "layers": args.layers, "gates": ngates,
                   "tile_passes": int(len(passes)), "tile_qubits": tile_q, "precision": args.precision,
                   "fusion": tuning, "autotune": tune,
                   "l2": f"inputs larger than L2 ({state_bytes / 2**30:g} GiB state), no flush needed"},
        "sweeps_per_s": len(passes) * args.steps * world / (elapsed_ms / 1e3),
        "hbm_gbs_algorithmic": len(passes) * 2 * state_bytes * args.steps * world / (elapsed_ms / 1e3) / 1e9,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "kernel": f"k_tile<{TILE_POLICY.get(args.precision, args.precision)}> (tile pass)",
                     "launches": tile_n,
                     "mean_launch_ms": tile_ms / tile_n if tile_n else None,
                     "peak_source": f"{peak_kind} hbm_gbs"},
        "compute_roofline": compute_roofline(args.precision, n, xops if tuning["fuse_mode"] == "tile" else [],
                                             prof["tile"][0] / args.steps, (clocks or {}).get("sm_mhz")),
        "kernel_ms_per_step": {k: v[0] / args.steps for k, v in prof.items()},
        "gpu_launches": launches,
        "clocks": clocks,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "gate_sweeps": sweeps,
        "adjoint": adj,
        "trajectories": traj,
        "mixed_batch": batch,
        "zne": zne,
        "config1_12q": config1,
        "trajectory_solver": tsolver,
        "density_matrix": dmat,
    }
    print(json.dumps(line), flush=True)


# FP32 lane instructions per amplitude pair of each executor op kind (0 U2, 1 RX, 2 RY, 3 H, 4 X,
# 5 DIAG, 6 CNOT, 7 MCZ), counted from the double-float routines of the kernels.  Results are stored
# without the closing Fast2Sum: a 4-term double-float dot product (df_lin4_raw) is 40 instructions
# (4 FMUL + 4 FFMA product errors, 3 TwoSum of 6, 8 FFMA cross terms, 6 FADD), a 2-term one
# (df_lin2_raw) 16, an x + a*y update (df_fma_raw) 12.  A U2 pair needs four 4-term products;
# RX/RY/H four 2-term ones; a diagonal two 2-term ones per amplitude; a ZYZ (phase-free unitary)
# eight; a ZY (RY after an input phase) six; a carried-phase flush (13) two per amplitude pair; a
# tangent-form rotation (14, 15) two 2-term products and four updates.  A CNOT carrying a pushed
# phase multiplies a quarter of the amplitudes.  CNOT, MCZ and X otherwise move or negate data
# without arithmetic.
FP32_INST_PER_PAIR = {"complex128": {0: 160, 1: 64, 2: 64, 3: 64, 4: 0, 5: 64, 6: 0, 7: 0, 11: 128, 12: 96, 13: 32, 14: 80,
                                     15: 80},
                      "complex64": {0: 16, 1: 8, 2: 8, 3: 8, 4: 0, 5: 8, 6: 0, 7: 0, 11: 16, 12: 12, 13: 4, 14: 8, 15: 8}}
PHASED_CNOT_PER_PAIR = {"complex128": 16, "complex64": 2}  # a complex multiply on a quarter of the amplitudes
SMS, FP32_LANES_PER_SM = 152, 128
TILE_POLICY = {"complex128": "PolDF64", "complex64": "PolF32", "fp64": "PolF64"}


def compute_roofline(precision, n, xops, tile_ms_step, sm_mhz):
    """FP32-issue roofline of the tile passes: algorithmic FP32 lane instructions per step over
    the measured tile-pass time, against 152 SMs x 128 lanes x the sampled SM clock."""
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


def profile_traffic():
    """DRAM bytes per tile-pass launch from the committed ncu summary, if present."""
    path = os.path.join(REPO, "profiles", "k_tile_df64_30q.md")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if line.startswith("traffic_bytes_per_launch:"):
                try:
                    return float(line.split(":", 1)[1].strip())
                except ValueError:
                    return None
    return None


def run_adjoint_bench(args, torch):
    """Adjoint gradients of the 20-qubit, 10-layer RY/RZ + CZ-ring ansatz (400 parameters,
    observable sum_i Z_i Z_{i+1} periodic) for a batch of 64 parameter sets, against the
    parameter-shift rule evaluated on the same GPU (batched shifted circuits) for one set."""
    import llgpu
    import workloads

    n, layers, batch = 20, 10, 64
    ops = workloads.hea_ansatz(n, layers)
    nparams = layers * 2 * n
    params = workloads.hea_params(n, layers, batch)
    adj = llgpu.Adjoint(n, ops, nparams, llgpu.ring_zz_terms(n), max_batch=batch, precision=args.precision)
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
            "precision": args.precision}


def run_sweep_bench(args, torch):
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
    out = {"qubits": n, "peak_gbs": peak, "peak_source": f"{peak_kind} hbm_gbs"}
    for prec in ("complex128", "fp64"):
        st = llgpu.State(n, prec)
        st.set_fusion("none")
        res = {}
        for name, recs in kinds.items():
            ops = make_ops(recs)
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
            gbs = bytes_per.get(name, 32) * (1 << n) / per / 1e9
            res[name] = {"ms_per_sweep": per * 1e3, "gbs": gbs, "frac": gbs / peak}
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
            res[f"block{k}"] = {"ms_per_sweep": per * 1e3, "gbs": gbs, "frac": gbs / peak,
                                "tflops": 8 * (4 ** k) * (1 << (n - k)) / per / 1e12, "qubits": qs}
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
    for prec in ("complex128", "complex64"):
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
        key = "c128" if prec == "complex128" else "c64"
        out[key] = {"traj_per_s": ntraj / dt, "seconds": dt, "mean_z0": float(z.mean()),
                    "std_error": float(z.std(ddof=1) / np.sqrt(ntraj)), "jumps_per_traj": float(j.mean()),
                    "config": h.config(), "default_config": default_cfg,
                    "default_traj_per_s": ntraj / dt_default, "autotune": tune}
        h.close()
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
                       "neighbouring pairs, complex128"}
    for n in (10, 13):
        dm = llgpu.DensityMatrix(n, "complex128")
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
        out[f"n{n}"] = res
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
    for prec in ("complex128", "complex64"):
        tune = llgpu.batch_autotune(nq, ops, off, prec)  # tile width by measurement (cached)
        b = llgpu.Batch(nq, ops, off, prec, llgpu.TUNE_AUTO)
        stream = torch.cuda.ExternalStream(b.stream)
        b.run()  # captures the CUDA graph; later runs replay it
        dt, _ = _timed(stream, torch, b.run, reps=max(1, args.steps))
        key = "c128" if prec == "complex128" else "c64"
        info = b.info()
        res[key] = {"circuits_per_s": 512 / dt, "gates_per_s": ngates / dt, "seconds": dt,
                    "work_items": info["work_items"], "tile_qubits": info["tile_qubits"],
                    "autotune": tune}
        batches[key] = b
    f = batches["c64"].fidelity(batches["c128"])
    res["c64_fidelity_error"] = {"max": float(np.max(1 - f[:, 0])), "median": float(np.median(1 - f[:, 0]))}
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


def run_e2e(args, ops, xops, n, elem, world, torch):
    import quantum_sim_v3

    sv = quantum_sim_v3.StateVector(n, args.precision)
    if args.tile < 0:
        sv.autotune(ops, 2 * len(ops) // max(1, args.layers))  # the headline's tuning, from the cache
    else:
        sv.set_fusion("tile", args.tile)
    sv.apply_ops(ops)
    sv.get_numpy_view()  # allocates the pinned host mirror once
    steps = max(1, args.steps)
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
    return {"value": len(ops) * steps * world / (t1 - t0), "unit": "gates/s",
            "ms_per_step": 1e3 * (t1 - t0) / steps, "passes_alone_ms": 1e3 * (b - a), "readback_alone_ms": 1e3 * (c - b),
            "h2d_bytes_per_step": int(ops.nbytes + xops.nbytes), "d2h_bytes_per_step": int((1 << n) * 16),
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
