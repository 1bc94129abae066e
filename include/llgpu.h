/*
 * llgpu.h -- C ABI of the GB300 state-vector engine (libllgpu.so).
 *
 * This is the drop-in boundary under the Python `quantum_sim_v3.StateVector` / `quantum_sim_v2`
 * modules and the C++ `ll::GpuBackend` (include/ll_gpu_backend.h).  Plain pointers and sizes
 * only.  Each entry point names the reference interface it replaces (paths inside the reference
 * project Athleity/lightning-lite-quantum-simulator).
 *
 * Conventions (src/Backend.h:3-8): qubit q is bit q of the basis-state index; RX/RY/RZ(t) =
 * exp(-i t P/2); mcz negates every amplitude whose bits are all 1 on the listed qubits.
 * Amplitudes cross the boundary as complex128: 2 doubles (re, im) per basis state, 16 bytes,
 * the std::complex<double> / numpy complex128 layout.
 *
 * Errors: every call returns an llg status.  LLG_EINVAL is the reference's
 * std::invalid_argument (Python ValueError), LLG_ERUNTIME its std::runtime_error (Python
 * RuntimeError).  llg_last_error() gives the message of the calling thread's last failure.
 * Arguments are validated on the host before anything is enqueued; a rejected call leaves the
 * state untouched.
 *
 * Execution: each state owns one CUDA stream.  Gate calls are validated and appended to the
 * state's pending-gate queue; the queue is flushed (planned into fused passes and launched
 * asynchronously) when a readout needs the amplitudes, on llg_sync/llg_flush, or when it grows
 * past an internal limit.  A state object is not thread-safe (the reference's are not either).
 */
#ifndef LLGPU_H
#define LLGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define LLG_OK 0
#define LLG_EINVAL 1   /* invalid argument (reference: std::invalid_argument) */
#define LLG_ERUNTIME 2 /* runtime failure (reference: std::runtime_error) */
#define LLG_ENOMEM 3   /* device or pinned-host allocation failed */
#define LLG_ECUDA 4    /* a CUDA call failed; the message names it */
#define LLG_ETIMEOUT 5 /* a bounded device-side wait gave up; the kernel returned early */

/* ---- amplitude precisions (how the state is held in HBM) ---- */
#define LLG_F64 0  /* complex128 as IEEE double pairs, FP64 arithmetic (plain path) */
#define LLG_DF64 1 /* complex128 class: each real part as an fp32 (hi, lo) pair, 16 B/amplitude,
                      FP32-pipe error-free arithmetic, ~48-bit significand */
#define LLG_F32 2  /* complex64: fp32 pairs, FP32 arithmetic */

/* ---- fusion modes for the pending-gate queue ---- */
#define LLG_FUSE_NONE 0 /* one streaming kernel per gate: the reference's own algorithm */
#define LLG_FUSE_TILE 1 /* shared-memory tile passes over chosen qubit sets (cache blocking) */
#define LLG_FUSE_REG 2  /* register-tiled passes: complex64 states, tiles of 9..13 qubits held in
                           registers (16 amplitudes per thread), shared memory only between layouts */

/* ---- gate record (96 bytes).  Kinds 0..6 are the Op kinds of the reference's random-circuit
 * test, tests/test_backends.cpp:78-83 (h, x, rx, ry, rz, cnot, mcz). ---- */
#define LLG_OP_H 0
#define LLG_OP_X 1
#define LLG_OP_RX 2
#define LLG_OP_RY 3
#define LLG_OP_RZ 4
#define LLG_OP_CNOT 5 /* q0 = control, q1 = target */
#define LLG_OP_MCZ 6  /* mask = OR of 1 << q over the listed qubits */
#define LLG_OP_CZ 7   /* mcz({q0, q1}) */
#define LLG_OP_U2 8   /* generic 2x2 on q0, m = {g00, g01, g10, g11} interleaved re/im */

typedef struct llg_op {
    int32_t kind;
    int32_t q0;
    int32_t q1;
    int32_t param; /* index into a parameter vector (rotations), -1 if fixed */
    uint64_t mask;
    double theta;
    double m[8];
} llg_op;

typedef struct llg_state llg_state;

/* ---- library ---- */
const char* llg_last_error(void);
const char* llg_version(void);
/* Number of CUDA devices visible; 0 when none (every compute call then fails with LLG_ECUDA). */
int llg_device_count(void);

/* ---- state lifetime ---- */

/* New n-qubit state |0...0>.  Replaces StateVectorOptimized(int) (src/StateVectorOptimized.cpp:17-24)
 * and Backend::reset (src/Backend.h:30, src/StateVectorBackend.h:49-57).  n in [1, 34]. */
int llg_create(int n_qubits, int precision, llg_state** out);

/* New state holding a copy of `len` complex128 amplitudes (2*len doubles).  Replaces the
 * ndarray constructor (src/StateVectorOptimized.cpp:26-47): len must be a power of two
 * (else LLG_ERUNTIME "Array size must be power of 2"); the data is copied to HBM, not aliased. */
int llg_create_from_host(const double* amps, size_t len, int precision, llg_state** out);

int llg_destroy(llg_state* st);

/* Back to |0...0> on n qubits (src/Backend.h:30).  n outside [1, 34] is LLG_EINVAL. */
int llg_reset(llg_state* st, int n_qubits);

/* src/StateVectorOptimized.cpp:108-109 get_num_qubits / get_size. */
int llg_num_qubits(const llg_state* st, int* out);
int llg_size(const llg_state* st, uint64_t* out);
int llg_get_precision(const llg_state* st, int* out);

/* Fusion mode for this state's queue (LLG_FUSE_*) and tile width in qubits (0 = the default:
 * 12 for 16-byte amplitudes, 13 for complex64; llg_autotune picks one by measurement). */
int llg_set_fusion(llg_state* st, int mode, int tile_qubits);
/* Threads per CTA of the tile kernel: 0 (default: 512 for tiles of 10+ qubits, else half the
 * tile) or a multiple of 32 in [32, 1024]. */
int llg_set_tile_threads(llg_state* st, int threads);
/* The settings the next flush uses (tile_qubits with the default resolved). */
int llg_get_tuning(const llg_state* st, int* fuse_mode, int* tile_qubits, int* tile_threads);

/* ---- autotuning ----
 * Fusion width and CTA shape picked by timing candidates on the device (CUDA events on the
 * object's own stream), cached process-wide under a hash of the workload's shape (sizes, gate
 * kinds and qubits; angles do not change the work).  No reference counterpart: the reference's
 * cache blocking uses fixed sizes (src/StateVectorOptimized.cpp:56-78). */
typedef struct llg_tune_result {
    int32_t fuse_mode;   /* LLG_FUSE_NONE / LLG_FUSE_TILE (states) */
    int32_t tile_qubits; /* fusion width: qubits per shared-memory tile */
    int32_t cta_threads; /* threads per CTA (0: the kernel's default) */
    int32_t cluster;     /* CTAs per trajectory (trajectories; 1 elsewhere) */
    int32_t candidates;  /* configurations timed (0 when taken from the cache) */
    int32_t cached;      /* 1 if the result came from the cache */
    double best_ms;      /* the chosen configuration on the sample */
    double default_ms;   /* the default configuration on the same sample */
} llg_tune_result;
#define LLG_TUNE_AUTO (-1)

/* Times ops[0 .. sample_ops) (0: all) on a scratch state of st's size and precision under each
 * candidate -- per-gate kernels; tile passes of 8..max qubits with 256 threads per CTA, 512 from
 * 10 qubits, and 1024 from 11 qubits on registers of at most 16 qubits -- and applies the fastest
 * to st.  Needs device memory for a second state;
 * st's amplitudes are not touched. */
int llg_autotune(llg_state* st, const llg_op* ops, int nops, int sample_ops, llg_tune_result* out);
/* Forget every cached tuning result. */
void llg_tune_cache_clear(void);

/* ---- gates (validated now, executed at the next flush) ---- */

/* quantum_sim_v3 apply_gate_cache_optimized / apply_gate_standard and quantum_sim_v2 apply_gate
 * (src/StateVectorOptimized.cpp:56-97, src/bindings_v2.cpp:56-72): generic 2x2 `g` = 8 doubles,
 * row-major {g00, g01, g10, g11} as (re, im).  As in the reference a target >= n is a no-op;
 * a negative target is LLG_EINVAL. */
int llg_apply_gate(llg_state* st, int target, const double* g);

/* ll::StateVectorBackend gate set (src/StateVectorBackend.h:61-151, interface src/Backend.h:33-39):
 * a qubit outside [0, n), a non-finite angle, cnot(q, q), an empty or repeated mcz list are
 * LLG_EINVAL. */
int llg_h(llg_state* st, int q);
int llg_x(llg_state* st, int q);
int llg_rx(llg_state* st, int q, double theta);
int llg_ry(llg_state* st, int q, double theta);
int llg_rz(llg_state* st, int q, double theta);
int llg_cnot(llg_state* st, int control, int target);
int llg_cz(llg_state* st, int a, int b);
int llg_mcz(llg_state* st, const int* qubits, int nq);

/* A list of gate records appended in order (the op-list form of the calls above; U2 records
 * follow llg_apply_gate and are LLG_EINVAL for a target outside [0, n)). */
int llg_apply_ops(llg_state* st, const llg_op* ops, int nops);

/* Dense k-qubit block (the fused form of python/gate_fusion.py:7-37 widened to k qubits):
 * `m` is 2^k x 2^k complex, row-major, interleaved; qubits[0] is the least-significant bit of
 * the block's local index.  k in [1, 5], distinct qubits in [0, n). */
int llg_apply_matrix(llg_state* st, int k, const int* qubits, const double* m);

/* Other names of four entry points above, for FFI bindings written against them:
 *   llg_wrap_host      = llg_create_from_host (the ndarray constructor, copied, not aliased);
 *   llg_apply_1q       = llg_apply_gate with ll::Backend validation: a qubit outside [0, n) is
 *                        LLG_EINVAL instead of the v3 no-op (src/StateVectorBackend.h:176-186);
 *   llg_apply_block    = llg_apply_matrix;
 *   llg_expect_diag_zz = llg_expect_zz. */
int llg_wrap_host(const double* amps, size_t len, int precision, llg_state** out);
int llg_apply_1q(llg_state* st, int q, const double* m);
int llg_apply_block(llg_state* st, int k, const int* qubits, const double* m);
int llg_expect_diag_zz(llg_state* st, int nterms, const int* a, const int* b, const double* coeff, double* out);

/* ---- density matrices (the reference's KrausChannel, src/Noise.h:85-147) ----
 * rho on n qubits lives in a state of 2n qubits: element (row, col) is amplitude
 * row + col * 2^n, so qubit q is bit q of the row and qubit n + q bit q of the column.  Create it
 * with llg_create(2n, ...) (|0..0> of 2n qubits is |0..0><0..0|) or llg_create_from_host. */
/* U rho U^+ for one gate record on qubits [0, n): U on the row qubits, conj(U) on the column
 * qubits. */
int llg_dm_apply_op(llg_state* st, int n, const llg_op* op);
/* KrausChannel::apply (src/Noise.cpp:174-258): rho <- sum_k K_k rho K_k^+ for nkraus operators
 * of 2^m x 2^m (m = 1 or 2; row-major, interleaved; bit j of an operator's index is
 * targets[j]), applied as one dense block sum_k K_k (x) conj(K_k) on the 2m row and column
 * qubits.  Operators must be trace preserving to 1e-10 (src/Noise.cpp:166-172). */
int llg_dm_apply_kraus(llg_state* st, int n, int nkraus, const double* kraus, int m, const int* targets);

/* ---- execution and readout ---- */

/* Plan and launch the pending queue without waiting. */
int llg_flush(llg_state* st);
/* Flush and wait for the state's stream. */
int llg_sync(llg_state* st);

/* Amplitudes to host memory (2*2^n doubles) after a flush; replaces get_numpy_view
 * (src/StateVectorOptimized.cpp:99-106) and Backend::state (src/Backend.h:44) as an explicit
 * device-to-host copy.  Into pinned memory (llg_host_alloc, cudaHostRegister) one conversion
 * kernel writes the host buffer directly; other memory is filled through a staging buffer. */
int llg_copy_to_host(llg_state* st, double* out);
/* Overwrite the amplitudes from host memory (2*2^n doubles). */
int llg_copy_from_host(llg_state* st, const double* amps);

/* |a_i|^2 for every basis state into host memory (2^n doubles); replaces
 * StateVectorBackend::probabilities (src/StateVectorBackend.h:153-161). */
int llg_probabilities(llg_state* st, double* out);

/* sum_i |a_i|^2 (FP64 result). */
int llg_norm2(llg_state* st, double* out);
/* Two states of the same qubit count, any precisions, compared on the device in double:
 * fidelity |<a|b>|^2 / (<a|a><b|b>) and max over i of |Re(a_i - b_i)|, |Im(a_i - b_i)| (either
 * output may be NULL).  No reference counterpart: a check for parity tests at sizes whose host
 * copies would be too large. */
int llg_compare(llg_state* a, llg_state* b, double* fidelity, double* max_abs_diff);
/* llg_compare that also returns the largest |re| or |im| of b's amplitudes (the scale that a
 * relative amplitude error is taken against); any output may be NULL. */
int llg_compare_ex(llg_state* a, llg_state* b, double* fidelity, double* max_abs_diff, double* max_abs_b);

/* sum_k coeff_k <Z_{a_k} Z_{b_k}>; b_k < 0 selects the single-qubit term <Z_{a_k}>.  The
 * diagonal of python/algorithms.py:139-152 (ising_diagonal) evaluated on the fly: any number of
 * terms with any coefficients (up to 64 terms with at most 4 distinct values run a kernel that
 * counts parities per coefficient class; anything larger, e.g. an SK model's all-to-all
 * couplings, runs a chunked kernel whose cost per amplitude does not grow with the terms). */
int llg_expect_zz(llg_state* st, int nterms, const int* a, const int* b, const double* coeff, double* out);

/* sum_i |a_i|^2 diag[i] for a full 2^n diagonal: the reference's energy = probabilities() . diag
 * (python/algorithms.py:172-181, run_vqe(hamiltonian_diag=...)).  on_device = 0: `diag` is host
 * memory, copied to a device buffer the state keeps; else it is device memory of the state's
 * device, read in place. */
int llg_expect_diagonal(llg_state* st, const double* diag, int on_device, double* out);

/* No counterpart in the reference.  llg_expect_zz for callers that cannot allocate GPU memory:
 * callers whose device memory belongs to another allocator (a framework that reserves most of
 * the GPU up front) and callers in latency-critical loops where cudaMalloc/cudaFree would
 * synchronise the device.  The caller passes the amplitudes (d_amps: 2^n elements in the
 * `precision` layout, memory of the current device or managed memory; another device's memory is
 * LLG_EINVAL) and d_out (2 device doubles, receiving
 * [sum_k coeff_k <Z..>, sum |a|^2]); kernels are enqueued on `stream` (a cudaStream_t, NULL for
 * the default stream) and the call returns without waiting.  Nothing is allocated: the partial
 * sums go to a fixed 40 KiB device array inside the library (1024 blocks x 5 doubles), held by
 * every GPU that loads it until exit.  The first call on a device resolves that array's address
 * and should come before any stream capture on that device.  All calls share the array; each
 * call writes every partial it reads, but calls that overlap on the GPU race.  The array's
 * address is cached per device for the process: do not call this after cudaDeviceReset.  A CUDA
 * error already pending before the call is returned as LLG_ECUDA without launching.  Limits:
 * n_qubits in [1, 34], at most 64 terms with at most 4 distinct coefficients. */
int llg_expect_zz_noalloc(const void* d_amps, int n_qubits, int precision, int nterms, const int* a, const int* b,
                          const double* coeff, double* d_out, void* stream);

/* Scale the state to unit norm (the periodic renormalisation of the complex64 path). */
int llg_renormalize(llg_state* st);

/* ---- batched parametrised circuits: adjoint gradients and parameter shift ----
 * A circuit whose RX/RY/RZ records carry param >= 0 takes theta = params[set][param] for each
 * parameter set of a batch; the states of a batch live side by side in HBM ([batch][2^n]).
 * The observable is O = sum_k coeff_k Z_{za[k]} Z_{zb[k]} (zb[k] < 0: single Z), as in
 * python/algorithms.py:141-153; E = <psi|O|psi>.  Parameters, energies and gradients may be host
 * or device pointers.  Calls block until their results are written. */
typedef struct llg_adjoint llg_adjoint;

/* Plans the circuit once for up to max_batch parameter sets.  n in [1, 30]. */
int llg_adjoint_create(int n, const llg_op* ops, int nops, int nparams, int max_batch, int precision, int nterms,
                       const int* za, const int* zb, const double* zcoeff, llg_adjoint** out);
int llg_adjoint_destroy(llg_adjoint* h);
int llg_adjoint_info(const llg_adjoint* h, int* fwd_passes, int* bwd_passes, int* n_param_ops);
/* Threads per CTA of the forward and reverse tile passes: 0 (default: 128 for tiles of 8+
 * qubits) or a multiple of 32 in [32, 512]. */
int llg_adjoint_set_threads(llg_adjoint* h, int threads);

/* E(theta) for `batch` parameter sets (params [batch][nparams]) and, if grads != NULL, every
 * dE/dtheta by the adjoint method: one forward sweep, one reverse sweep of psi and lambda = O psi
 * with one inner-product reduction per parametrised gate.  The reference's gradient is the
 * parameter-shift rule (src/Algorithms.h:277-292).  checkpoint_every = C > 0 stores the forward
 * state every C tile passes and restarts the reverse sweep from those states. */
int llg_adjoint_run(llg_adjoint* h, const double* params, int batch, double* energies, double* grads, int checkpoint_every);

/* The same gradients by the reference's parameter-shift rule (src/Algorithms.h:210-212, :277-292),
 * each shifted circuit evaluated as one member of a batched forward sweep: 1 + 2 * (number of
 * parametrised gates) evaluations per parameter set. */
int llg_param_shift_run(llg_adjoint* h, const double* params, int sets, double* energies, double* grads);

/* The handle's CUDA stream (cudaStream_t). */
int llg_adjoint_stream(const llg_adjoint* h, void** out);

/* ---- batched noisy trajectories ----
 * Runs trajectories [traj_begin, traj_begin + n_traj) of an n-qubit circuit (n in [1, 14]) in one
 * persistent launch, each state resident in shared memory (a 2-CTA cluster for 14-qubit complex128
 * states).  After every gate, for each qubit it touches (1-qubit gates: its qubit; cnot/cz:
 * control then target; mcz: its qubits in increasing order -- the noise sites of
 * src/Mitigation.h:146-204), amplitude damping (gamma_ad) then phase damping (lambda_pd) are
 * unravelled with the jump rule of src/TrajectorySolver.h:421-455 using Philox4x32-10 uniforms
 * (key = seed, counter = (site, trajectory); u = (x >> 11) * 2^-53 as src/Mitigation.h:207).
 * Writes <Z_0> of each trajectory's final state to z0_out, and optionally the jump count per
 * trajectory and a jump log (one byte per touched-qubit site: bit 0 amplitude-damping jump, bit 1
 * dephasing jump; row stride log_stride >= sites).  *min_margin receives the smallest
 * |u - survive| seen (a decision closer than rounding could go either way).  Outputs may be host
 * or device pointers; the call blocks until they are written. */
int llg_traj_run(int n, const llg_op* ops, int nops, double gamma_ad, double lambda_pd, uint64_t seed,
                 uint64_t traj_begin, uint64_t n_traj, int precision, double* z0_out, uint32_t* jumps_out,
                 uint8_t* jump_log, int64_t log_stride, double* min_margin);

/* The same trajectories from a handle planned once: gates uploaded, outputs for up to max_traj
 * trajectories, and the persistent launch captured as a CUDA graph that every llg_traj_launch
 * replays with its own seed and trajectory range.  cluster: CTAs per trajectory (1, or 2 with the
 * state split on its top qubit; 0: 1 when the state fits one CTA's shared memory, else 2);
 * cta_threads: 0 for the default (half the CTA's amplitudes, at most 1024), else a multiple of 32.
 * LLG_TUNE_AUTO in either runs llg_traj_autotune at creation. */
typedef struct llg_traj llg_traj;
int llg_traj_create(int n, const llg_op* ops, int nops, double gamma_ad, double lambda_pd, int precision,
                    uint64_t max_traj, int cluster, int cta_threads, llg_traj** out);
int llg_traj_destroy(llg_traj* h);
/* Trajectories [traj_begin, traj_begin + n_traj), n_traj <= max_traj; outputs as llg_traj_run
 * (no jump log); blocks until they are written. */
int llg_traj_launch(llg_traj* h, uint64_t seed, uint64_t traj_begin, uint64_t n_traj, double* z0_out,
                    uint32_t* jumps_out, double* min_margin);
/* Times `sample_traj` trajectories (0: two per persistent CTA group) under each feasible
 * (cluster, 256/512/1024 threads) and keeps the fastest (cached by the circuit's shape). */
int llg_traj_autotune(llg_traj* h, uint64_t sample_traj, llg_tune_result* out);
int llg_traj_config(const llg_traj* h, int* cluster, int* cta_threads, int* grid, int64_t* sites);
int llg_traj_stream(const llg_traj* h, void** out);

/* ---- depolarizing noise with gate folding, and zero-noise extrapolation ----
 * Batched form of ll::NoisyBackend (src/Mitigation.h:110-240): every gate U of `ops` runs as
 * U (U^+ U)^k for scale = 2k + 1 (odd, 1..99), each application followed by its noise site(s):
 * one 2-qubit depolarizing site over (q0, q1) for cnot, cz and 2-qubit mcz, else a 1-qubit site
 * per touched qubit.  A site draws u; u < p applies a non-identity Pauli chosen by a second
 * uniform u2: 1 + floor(3 u2) in {X, Y, Z}, or 1 + floor(15 u2) with the low two bits on the
 * first qubit and the high two on the second; Y = Z then X.  u and u2 come from one
 * Philox4x32-10 call (key = seed, counter = (site, trajectory)) instead of the reference's
 * sequential mt19937_64 stream.  The handle is an llg_traj: llg_traj_launch writes, per
 * trajectory, the observable sum_k zcoeff[k] Z_za[k] Z_zb[k] (zb[k] < 0: Z_za[k] alone; at most
 * 16 terms with at most 3 distinct coefficients; nterms = 0: <Z_0>) of the final state, and the
 * number of non-identity Paulis applied. */
int llg_noisy_create(int n, const llg_op* ops, int nops, double p, int scale, int precision, uint64_t max_traj,
                     int nterms, const int* za, const int* zb, const double* zcoeff, int cluster, int cta_threads,
                     llg_traj** out);

/* ll::ZNE (src/Mitigation.h:243-377). */
#define LLG_ZNE_MAX_SCALES 8
typedef struct llg_zne_result {
    double value;                           /* E(0) = sum_k weights[k] values[k] */
    double std_error;                       /* sqrt(sum_k weights[k]^2 std_errors[k]^2); NaN if not estimable */
    int32_t nscales;
    int32_t pad;
    int64_t trajectories;                   /* run per scale (1 when p == 0) */
    double scales[LLG_ZNE_MAX_SCALES];
    double values[LLG_ZNE_MAX_SCALES];      /* trajectory mean at each scale */
    double std_errors[LLG_ZNE_MAX_SCALES];  /* sample std / sqrt(N) (Welford) */
    double weights[LLG_ZNE_MAX_SCALES];     /* Richardson weights */
} llg_zne_result;
/* c_k = prod_{j != k} s_j / (s_j - s_k) (ZNE::richardson_weights, src/Mitigation.h:287-301). */
int llg_richardson_weights(const double* scales, int nscales, double* weights);
/* ZNE::extrapolate (src/Mitigation.h:313-377) over the circuit: `trajectories` runs per scale
 * (scales: 2..8 distinct odd integers in [1, 99]) in one persistent launch each, trajectory
 * indices [k N, (k + 1) N) for scale k; Richardson extrapolation to zero noise.  Errors as the
 * reference: bad scales, p, trajectories or observable are LLG_EINVAL; an empty circuit is
 * LLG_ERUNTIME ("applied no gates"). */
int llg_zne_run(int n, const llg_op* ops, int nops, double p, int precision, const double* scales, int nscales,
                int64_t trajectories, uint64_t seed, int nterms, const int* za, const int* zb, const double* zcoeff,
                llg_zne_result* out);

/* ---- dense trajectory solver (the reference's TrajectorySolver, src/TrajectorySolver.h) ----
 * Lindblad equation d rho/dt = -i [H(t), rho] + sum_k gamma_k (L rho L^+ - {L^+L, rho}/2) on
 * n <= 10 qubits with dense dim x dim operators (row-major, interleaved), unravelled into
 * trajectories that run together in one persistent launch: STANDARD (norm-loss quantum jumps),
 * PROJECTOR (Pauli-like channels as sqrt(g)(1 - P)) and ANALOG (homodyne diffusion).  Plans,
 * step sizes, the jump selection and the error contract follow src/TrajectorySolver.h:124-514.
 * Uniforms come from Philox4x32-10 (key = seed, counter = (draw, trajectory)), not the
 * reference's per-trajectory mt19937_64 streams. */
#define LLG_UNRAVEL_STANDARD 0
#define LLG_UNRAVEL_PROJECTOR 1
#define LLG_UNRAVEL_ANALOG 2
typedef struct llg_tsolver llg_tsolver;
/* H(t) callback: writes the dim x dim Hermitian matrix (row-major, interleaved) at time t. */
typedef void (*llg_hamiltonian_fn)(double t, double* h_out, void* user);
int llg_tsolver_create(int n_qubits, llg_tsolver** out);
int llg_tsolver_destroy(llg_tsolver* s);
int llg_tsolver_set_hamiltonian(llg_tsolver* s, const double* h);
int llg_tsolver_set_hamiltonian_fn(llg_tsolver* s, llg_hamiltonian_fn fn, void* user);
/* Adds gamma (L rho L^+ - 1/2 {L^+L, rho}); gamma = 0 adds nothing; at most 64 channels. */
int llg_tsolver_add_lindblad(llg_tsolver* s, const double* l, double gamma);
int llg_tsolver_clear_lindblad(llg_tsolver* s);
int llg_tsolver_info(const llg_tsolver* s, int* n_channels, int* dim);
int llg_tsolver_projector_applies(const llg_tsolver* s, int channel, int* out);
/* n_traj trajectories from psi0 (normalised here) over `duration` with step ~dt.  Optional
 * outputs: states_out (n_traj x dim complex), rho_out = (1/N) sum |psi><psi| (dim x dim, in
 * trajectory order), obs_out[t] = <psi_t| obs |psi_t> for a Hermitian obs.  run_one is
 * n_traj = 1. */
int llg_tsolver_run(llg_tsolver* s, const double* psi0, double duration, double dt, int64_t n_traj, int kind,
                    uint64_t seed, double* states_out, double* rho_out, const double* obs, double* obs_out);
/* The last run's plan (row-major, interleaved): steps, h, constant H or not, the unraveling,
 * the propagator, the RK4 / diffusion nodes (written when n_nodes <= max_nodes), the jump
 * operators and their J^+ J. */
int llg_tsolver_plan_export(const llg_tsolver* s, long long* steps, double* h, int* constant, int* kind, double* prop,
                            double* nodes, int64_t max_nodes, double* ops, double* ops_dop, int* n_ops, int64_t* n_nodes);

/* ---- mixed-size batches ----
 * `count` circuits (circuit c: n_qubits[c] in [1, 30], ops[op_offsets[c] .. op_offsets[c+1]))
 * planned into shared-memory tile passes of tile_qubits qubits (0: default, 12 or 13 for
 * complex64; LLG_TUNE_AUTO: picked by llg_batch_autotune) and run together from |0..0> in ONE
 * persistent launch: persistent CTAs take (circuit, pass, tile) work items from a queue; a tile
 * waits, with a bounded poll, for the previous pass of its own circuit.  Each run replays a CUDA
 * graph captured at the first run (state reset + the persistent kernel).  The reference runs such
 * circuits one at a time on StateVectorBackend (src/StateVectorBackend.h). */
typedef struct llg_batch llg_batch;
int llg_batch_create(int count, const int* n_qubits, const llg_op* ops, const int64_t* op_offsets, int precision,
                     int tile_qubits, llg_batch** out);
int llg_batch_destroy(llg_batch* b);
/* Builds and times the batch once per (tile width from 8 qubits to the maximum) x (256 or 512
 * threads per CTA), one untimed run each, and returns the fastest in out->tile_qubits and
 * out->cta_threads (cached by the batch's shape).  Batches created with an explicit tile width
 * use 256 threads. */
int llg_batch_autotune(int count, const int* n_qubits, const llg_op* ops, const int64_t* op_offsets, int precision,
                       llg_tune_result* out);
int llg_batch_config(const llg_batch* b, int* tile_qubits, int* grid, int* cta_threads);
int llg_batch_info(const llg_batch* b, int64_t* work_items, int64_t* total_amps, int* total_passes);
/* Reset every state to |0..0> and run all circuits; spin_limit bounds each dependency wait in
 * polls (0: about a second).  A wait that runs out makes the call return LLG_ETIMEOUT. */
int llg_batch_run(llg_batch* b, int64_t spin_limit);
/* Test hook: make one work item wait for a count no tile reaches, so the next run's bounded wait
 * runs out and reports LLG_ETIMEOUT (the kernel returns normally). */
int llg_batch_debug_block_item(llg_batch* b, int64_t item);
/* Amplitudes of circuit `index` as complex128 into host memory (2 * 2^n doubles). */
int llg_batch_copy_state(llg_batch* b, int index, double* out);
/* Per circuit: fidelity |<a|b>|^2 / (|a|^2 |b|^2) (FP64 accumulation), |a|^2, |b|^2 into
 * out[3 * i + 0..2].  a and b hold the same circuit sizes (e.g. complex64 vs complex128 runs). */
int llg_batch_fidelity(llg_batch* a, llg_batch* b, double* out);
int llg_batch_stream(const llg_batch* b, void** out);

/* ---- tracing ----
 * Per-state kernel timing with CUDA events recorded on the state's own stream around every
 * engine launch, summed per kernel class.  Off by default (a few microseconds per launch). */
#define LLG_PROF_TILE 0    /* fused shared-memory tile passes */
#define LLG_PROF_GATE 1    /* per-gate streaming kernels */
#define LLG_PROF_INIT 2    /* state initialisation */
#define LLG_PROF_READOUT 3 /* conversions, |a|^2, reductions, scaling */
#define LLG_PROF_CLASSES 4
int llg_profile(llg_state* st, int on);
/* Waits for the stream, then writes the summed milliseconds and launch counts per class
 * (arrays of LLG_PROF_CLASSES); reset != 0 clears the sums. */
int llg_profile_read(llg_state* st, double* ms, int64_t* launches, int reset);
/* Process-wide number of kernels the engine has launched (all states). */
int64_t llg_kernel_launches(void);
/* The state's CUDA stream (a cudaStream_t), for callers that order their own work after it. */
int llg_get_stream(const llg_state* st, void** out);
/* Measurement aid with no counterpart in the reference: the current device's FP64 fused
 * multiply-add throughput, timed with CUDA events over one launch of `iters` iterations of eight
 * independent FMA chains per thread (after one untimed launch).  The FP64 roofline of the IEEE
 * complex128 path is taken against this number. */
int llg_fp64_fma_rate(int iters, double* fma_per_s);

/* Pinned host memory, mapped into the device's address space, for fast transfers
 * (cudaHostAlloc); NULL on failure. */
void* llg_host_alloc(size_t bytes);
void llg_host_free(void* p);

/* ---- planner introspection (host only; no GPU needed) ----
 * Plans `ops` on n qubits into shared-memory tile passes of `tile_qubits` qubits exactly as a
 * flush does, and exports the passes and the executor ops they run (coefficients as doubles).
 * Used by the CPU tests to execute a plan in numpy against the oracle.  Writes at most
 * max_passes / max_xops records and the true counts to *npasses / *nxops. */
typedef struct llg_pass_info {
    uint64_t local_mask; /* qubits held in the tile */
    int32_t t;           /* tile width in qubits */
    int32_t low;         /* the low `low` qubits are always local (coalesced runs) */
    int32_t op_begin;    /* first executor op of the pass */
    int32_t nops;        /* number of executor ops */
} llg_pass_info;

/* Executor op: kind 0 U2, 1 RX, 2 RY, 3 H, 4 X, 5 DIAG, 6 CNOT, 7 MCZ, 11 ZYZ (a unitary 2x2
 * without its global phase: diag(1, c4 + i c5) [c2, -c3; c3, c2] diag(1, c0 + i c1); the dropped
 * phases are multiplied into the plan's first U2).  Qubit fields are tile-local indices unless
 * flags bit 0 marks q0 as a global qubit outside the tile; nl_mask holds global qubits that must
 * all be 1 in the tile for the op to act. */
typedef struct llg_exec_op {
    int32_t kind;
    int32_t q0;
    int32_t q1;
    int32_t flags;
    uint64_t mask;
    uint64_t nl_mask;
    double c[8];
} llg_exec_op;

int llg_plan_export(int n, const llg_op* ops, int nops, int tile_qubits, llg_pass_info* passes, int max_passes,
                    int* npasses, llg_exec_op* xops, int max_xops, int* nxops);
/* The same with planner options: LLG_PLAN_ZYZ lowers fused unitary 2x2s to carried-phase
 * rotations as the engine does for complex128 and double-float states; LLG_PLAN_TABLES (with
 * LLG_PLAN_ZYZ) also gathers their input phases and the phased CNOTs' controlled phases into
 * phase tables (kind 18: every tile amplitude l times table entry l; kinds 16 / 17: the real
 * rotations [1, -c2; c2, 1] and [c2, -1; 1, c2] whose input phase a table applied), as the engine
 * does for those states.  llg_plan_export plans without either. */
#define LLG_PLAN_ZYZ 1
#define LLG_PLAN_TABLES 2
/* LLG_PLAN_REGS: the register programs of the register-tiled pass (kind 19 switches the layout:
 * register positions in mask, 4 bits each; thread-index positions in nl_mask; 1-qubit ops name a
 * register slot in q0, CNOTs their target slot in q1 and, with flags bit 4, a control slot in q0),
 * as the engine runs complex64 states (tables are not combined with it). */
#define LLG_PLAN_REGS 4
/* LLG_PLAN_FUSE2: two-qubit blocks as the engine plans complex64 shared-memory passes (kind 20: a
 * 4x4 matrix on local qubits q0 (index bit 0) and q1 (index bit 1), 16 entries from table entry
 * `mask`, row-major); alone, without the other options. */
#define LLG_PLAN_FUSE2 8
/* LLG_PLAN_DF64: with LLG_PLAN_ZYZ, the plan a double-float state gets (the tangent rotations'
 * dropped scale is absorbed before it reaches 2^-40 instead of 2^-300); the coefficients are
 * exported as doubles either way. */
#define LLG_PLAN_DF64 16
/* LLG_PLAN_STREAM: alone, the per-gate lowering an IEEE complex128 state runs without fusion (one
 * pass per op over the whole register, exported as a single pass of t = n): RX / RY / H without
 * their real factors (kinds 22 / 23: [1, -i c2; -i c2, 1] and [c2, -i; -i, c2]; 16 / 17 as above;
 * 24: [1, 1; 1, -1]), RZ as diag(1, e^{it}) (kind 13), the factors and RZ's global phase
 * absorbed once per flush by rewriting one op to its full form (kinds 0, 1, 2, 3 or 5). */
#define LLG_PLAN_STREAM 32
int llg_plan_export_ex(int n, const llg_op* ops, int nops, int tile_qubits, int flags, llg_pass_info* passes,
                       int max_passes, int* npasses, llg_exec_op* xops, int max_xops, int* nxops);
/* The eigenvalue d(i) of the diagonal observable sum_k coeff_k Z_{a_k} Z_{b_k} (b_k < 0: Z_{a_k}) for
 * every basis index i < 2^n, computed on the host by the same chunked decomposition the GPU
 * kernel uses (n <= 26).  For tests. */
int llg_diag_export(int n, int nterms, const int* a, const int* b, const double* coeff, double* out);
/* The phase tables of the same plan: (re, im) doubles, 2^tile_qubits entries per table; a kind-18
 * op's `mask` is the index of its first entry.  Writes at most max_doubles values and the true
 * count to *ndoubles. */
int llg_plan_export_tables(int n, const llg_op* ops, int nops, int tile_qubits, int flags, double* tables,
                           int64_t max_doubles, int64_t* ndoubles);

#ifdef __cplusplus
}
#endif

#endif /* LLGPU_H */
