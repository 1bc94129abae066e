// llg_engine.cu -- the C ABI of libllgpu.so (include/llgpu.h): state objects resident in HBM,
// argument validation with the reference's error contract, the pending-gate queue and its
// flush into fused tile passes or per-gate streaming kernels, and chunked host transfers.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/llgpu.h"
#include "llg_common_host.h"
#include "llg_diag.h"
#include "llg_diag_launch.h"
#include "llg_internal.h"
#include "llg_launch.h"

using namespace llg;

namespace llg {

thread_local std::string g_last_error;

int set_error(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return set_error(LLG_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace llg

#define LLG_CUDA(call, what)                            \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

static constexpr int kMaxQubits = 34;
static constexpr size_t kQueueFlushAt = 1 << 16;
static constexpr uint64_t kStageAmps = 1ULL << 24;  // 256 MiB of complex128 per transfer chunk

struct llg_state {
    int n = 0;
    int P = LLG_DF64;
    uint64_t size = 1;
    void* d_psi = nullptr;
    cudaStream_t stream = nullptr;
    int fuse_mode = LLG_FUSE_TILE;
    int tile_qubits = 0;   // 0 = default
    int tile_threads = 0;  // CTA size of the tile kernel, 0 = default
    std::vector<llg_op> queue;
    // op upload
    ExecOp* d_ops = nullptr;
    size_t d_ops_cap = 0;
    ExecOp* h_ops = nullptr;
    size_t h_ops_cap = 0;
    // phase tables of the plan (device, pinned staging), uploaded with the ops
    uint64_t* d_tables = nullptr;
    size_t d_tables_cap = 0;
    uint64_t* h_tables = nullptr;
    size_t h_tables_cap = 0;
    cudaEvent_t ops_done = nullptr;
    // dense-block matrix upload (pinned staging, reused once the previous copy has finished)
    uint64_t* d_block = nullptr;
    uint64_t* h_block = nullptr;
    cudaEvent_t block_done = nullptr;
    bool block_pending = false;
    // tensor-core 5-qubit blocks: sliced matrix (device, pinned staging) and a launch to check
    void* d_block_tc = nullptr;
    unsigned char* h_block_tc = nullptr;
    bool block_tc_launched = false;
    bool tiles_launched = false;  // a tile pass ran since the last sync (its load-timeout flag to check)
    // this state's timeout flags on the device: [0] a bulk tile load, [1] tensor-core products
    int* d_flags = nullptr;
    // reductions
    double* d_partials = nullptr;
    double* d_red = nullptr;
    // the last general diagonal observable (llg_diag.h), its device copy, and a full diagonal
    DiagObsHost obs;
    void* d_obs = nullptr;
    size_t d_obs_cap = 0;
    double* d_diag = nullptr;
    uint64_t d_diag_size = 0;
    // transfer staging (two chunks of complex128 = double2)
    double* d_stage[2] = {nullptr, nullptr};
    cudaEvent_t stage_ev[2] = {nullptr, nullptr};
    // tracing
    bool prof_on = false;
    struct ProfRec {
        int cls;
        cudaEvent_t a, b;
    };
    std::vector<ProfRec> prof_recs;
    std::vector<cudaEvent_t> ev_pool;
    double prof_ms[LLG_PROF_CLASSES] = {0, 0, 0, 0};
    int64_t prof_n[LLG_PROF_CLASSES] = {0, 0, 0, 0};
};

static std::atomic<int64_t> g_launches{0};

namespace {

bool finite(double x) { return std::isfinite(x); }

cudaEvent_t pool_event(llg_state* st) {
    if (!st->ev_pool.empty()) {
        cudaEvent_t e = st->ev_pool.back();
        st->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

// Launch through `f` (returns cudaError_t), count `nk` kernels, and time it when tracing is on.
template <class F>
int traced(llg_state* st, int cls, int nk, const char* what, F&& f) {
    cudaEvent_t a = nullptr, b = nullptr;
    if (st->prof_on) {
        a = pool_event(st);
        b = pool_event(st);
        if (a) cudaEventRecord(a, st->stream);
    }
    const cudaError_t e = f();
    if (e != cudaSuccess) return cuda_fail(e, what);
    g_launches += nk;
    if (st->prof_on && a && b) {
        cudaEventRecord(b, st->stream);
        st->prof_recs.push_back({cls, a, b});
    }
    return LLG_OK;
}

int check_qubit(const llg_state* st, int q, const char* who) {
    if (q < 0 || q >= st->n)
        return set_error(LLG_EINVAL, std::string(who) + ": qubit " + std::to_string(q) + " outside [0, " +
                                         std::to_string(st->n) + ")");
    return LLG_OK;
}

int check_angle(double t, const char* who) {
    if (!finite(t)) return set_error(LLG_EINVAL, std::string(who) + ": non-finite angle");
    return LLG_OK;
}

int default_tile(int P) { return P == LLG_F32 ? 13 : 12; }

int ensure_device_buffers(llg_state* st) {
    if (!st->stream) LLG_CUDA(cudaStreamCreateWithFlags(&st->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    if (!st->ops_done) LLG_CUDA(cudaEventCreateWithFlags(&st->ops_done, cudaEventDisableTiming), "cudaEventCreate");
    if (!st->d_partials) {
        LLG_CUDA(cudaMalloc(&st->d_partials, sizeof(double) * kRedBlocks * kPartialSlots), "cudaMalloc(partials)");
        LLG_CUDA(cudaMalloc(&st->d_red, sizeof(double) * kRedSlots), "cudaMalloc(red)");
    }
    if (!st->d_flags) {
        LLG_CUDA(cudaMalloc(&st->d_flags, 2 * sizeof(int)), "cudaMalloc(flags)");
        LLG_CUDA(cudaMemsetAsync(st->d_flags, 0, 2 * sizeof(int), st->stream), "cudaMemsetAsync(flags)");
    }
    return LLG_OK;
}

int alloc_state(llg_state* st, int n) {
    const uint64_t size = 1ULL << n;
    const size_t bytes = size * elem_bytes(st->P);
    if (st->d_psi && st->n == n) return LLG_OK;
    if (st->d_psi) {
        cudaStreamSynchronize(st->stream);
        cudaFree(st->d_psi);
        st->d_psi = nullptr;
    }
    cudaError_t e = cudaMalloc(&st->d_psi, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        st->d_psi = nullptr;
        return set_error(LLG_ENOMEM, "cannot allocate " + std::to_string(bytes) + " bytes of HBM for " +
                                         std::to_string(n) + " qubits: " + cudaGetErrorString(e));
    }
    st->n = n;
    st->size = size;
    return LLG_OK;
}

int stage_buffers(llg_state* st) {
    for (int i = 0; i < 2; ++i) {
        if (!st->d_stage[i]) LLG_CUDA(cudaMalloc(&st->d_stage[i], kStageAmps * 2 * sizeof(double)), "cudaMalloc(stage)");
        if (!st->stage_ev[i]) LLG_CUDA(cudaEventCreateWithFlags(&st->stage_ev[i], cudaEventDisableTiming), "cudaEventCreate");
    }
    return LLG_OK;
}

int run_streaming(llg_state* st, const std::vector<llg_op>& q) {
    std::vector<ExecOp> lowered;
    std::string err;
    if (st->P == LLG_F64) {
        // IEEE complex128: one pass per gate, the gates' real factors and RZ's global phase
        // carried through the flush and absorbed once (4 FP64 operations per pair, not 8)
        if (!lower_stream_f64(st->n, q.data(), (int)q.size(), lowered, err)) return set_error(LLG_EINVAL, err);
        for (const ExecOp& e : lowered) {
            int rc = traced(st, LLG_PROF_GATE, 1, "gate kernel",
                            [&] { return launch_exec_op(st->P, st->d_psi, st->n, e, st->stream); });
            if (rc) return rc;
        }
        return LLG_OK;
    }
    for (const llg_op& op : q) {
        lowered.clear();
        if (!lower_op(st->n, op, st->P, lowered, err)) return set_error(LLG_EINVAL, err);
        for (const ExecOp& e : lowered) {
            int rc = traced(st, LLG_PROF_GATE, 1, "gate kernel",
                            [&] { return launch_exec_op(st->P, st->d_psi, st->n, e, st->stream); });
            if (rc) return rc;
        }
    }
    return LLG_OK;
}

int upload_ops(llg_state* st, const std::vector<ExecOp>& ops, const std::vector<uint64_t>* tables = nullptr) {
    const size_t count = std::max<size_t>(ops.size(), 1);
    if (count > st->d_ops_cap) {
        if (st->d_ops) {
            cudaStreamSynchronize(st->stream);
            cudaFree(st->d_ops);
        }
        const size_t cap = std::max<size_t>(count, 1024);
        LLG_CUDA(cudaMalloc(&st->d_ops, cap * sizeof(ExecOp)), "cudaMalloc(ops)");
        st->d_ops_cap = cap;
    }
    // the pinned staging buffer may still feed an earlier copy
    LLG_CUDA(cudaEventSynchronize(st->ops_done), "cudaEventSynchronize");
    if (count > st->h_ops_cap) {
        if (st->h_ops) cudaFreeHost(st->h_ops);
        const size_t cap = std::max<size_t>(count, 1024);
        LLG_CUDA(cudaHostAlloc((void**)&st->h_ops, cap * sizeof(ExecOp), cudaHostAllocDefault), "cudaHostAlloc(ops)");
        st->h_ops_cap = cap;
    }
    if (!ops.empty()) {
        std::memcpy(st->h_ops, ops.data(), ops.size() * sizeof(ExecOp));
        LLG_CUDA(cudaMemcpyAsync(st->d_ops, st->h_ops, ops.size() * sizeof(ExecOp), cudaMemcpyHostToDevice, st->stream),
                 "cudaMemcpyAsync(ops)");
    }
    if (tables && !tables->empty()) {
        const size_t words = tables->size();
        if (words > st->d_tables_cap) {
            if (st->d_tables) {
                cudaStreamSynchronize(st->stream);
                cudaFree(st->d_tables);
                st->d_tables = nullptr;
            }
            LLG_CUDA(cudaMalloc(&st->d_tables, words * sizeof(uint64_t)), "cudaMalloc(tables)");
            st->d_tables_cap = words;
        }
        if (words > st->h_tables_cap) {
            if (st->h_tables) cudaFreeHost(st->h_tables);
            st->h_tables = nullptr;
            LLG_CUDA(cudaHostAlloc((void**)&st->h_tables, words * sizeof(uint64_t), cudaHostAllocDefault),
                     "cudaHostAlloc(tables)");
            st->h_tables_cap = words;
        }
        std::memcpy(st->h_tables, tables->data(), words * sizeof(uint64_t));
        LLG_CUDA(cudaMemcpyAsync(st->d_tables, st->h_tables, words * sizeof(uint64_t), cudaMemcpyHostToDevice, st->stream),
                 "cudaMemcpyAsync(tables)");
    }
    LLG_CUDA(cudaEventRecord(st->ops_done, st->stream), "cudaEventRecord");
    return LLG_OK;
}

// mirror (optional): the device address of a mapped host buffer that the last pass also fills;
// *mirrored tells whether a pass did (a plan may have no pass with work)
int run_tiles(llg_state* st, const std::vector<llg_op>& q, double* mirror = nullptr, bool* mirrored = nullptr) {
    Plan plan;
    std::string err;
    const int t = st->tile_qubits > 0 ? st->tile_qubits : default_tile(st->P);
    // register-tiled passes on registers of 9+ qubits (smaller ones keep the shared-memory tiles).
    // The 16-byte precisions plan carried-phase tangent rotations and phase tables (their passes
    // are arithmetic-bound); complex64 shared-memory passes, bound by shared-memory traffic, merge
    // each CNOT with its neighbouring one-qubit ops into a 4x4 block instead
    const bool reg = st->fuse_mode == LLG_FUSE_REG && std::min(st->n, std::min(t, 13)) >= 9;
    const bool f32_tiles = !reg && st->P == LLG_F32;
    if (!plan_tiles(st->n, q.data(), (int)q.size(), reg ? std::min(t, 13) : std::min(t, tile_max_qubits(st->P)), st->P,
                    plan, err, false, f32_tiles ? ZYZ_OFF : ZYZ_ON, !reg && st->P != LLG_F32, f32_tiles))
        return set_error(LLG_EINVAL, err);
    if (reg) to_register_program(plan);
    int rc = upload_ops(st, plan.ops, &plan.tables);
    if (rc) return rc;
    st->tiles_launched = true;
    size_t last = plan.passes.size();
    for (size_t i = 0; i < plan.passes.size(); ++i)
        if (plan.passes[i].nops > 0) last = i;
    for (size_t i = 0; i < plan.passes.size(); ++i) {
        const PassDesc& pd = plan.passes[i];
        if (pd.nops <= 0) continue;
        double* m = i == last ? mirror : nullptr;
        rc = traced(st, LLG_PROF_TILE, 1, "tile kernel",
                    [&] {
                        if (reg) return launch_tile_reg(st->P, st->d_psi, st->n, pd, st->d_ops, st->stream, m);
                        return launch_tile_pass(st->P, st->d_psi, st->n, pd, st->d_ops, st->d_tables, st->tile_threads,
                                                st->d_flags, st->stream, m);
                    });
        if (rc) return rc;
    }
    if (mirrored) *mirrored = mirror && last < plan.passes.size();
    return LLG_OK;
}

int enqueue(llg_state* st, const llg_op& op) {
    st->queue.push_back(op);
    if (st->queue.size() >= kQueueFlushAt) return llg_flush(st);
    return LLG_OK;
}

llg_op make_op(int kind, int q0, int q1 = 0, double theta = 0.0, uint64_t mask = 0) {
    llg_op op;
    std::memset(&op, 0, sizeof(op));
    op.kind = kind;
    op.q0 = q0;
    op.q1 = q1;
    op.param = -1;
    op.theta = theta;
    op.mask = mask;
    return op;
}

// Validate one record against the state (host side, before anything is enqueued).
int validate_op(const llg_state* st, const llg_op& op, const char* who) {
    int rc;
    switch (op.kind) {
        case LLG_OP_H:
        case LLG_OP_X:
            return check_qubit(st, op.q0, who);
        case LLG_OP_RX:
        case LLG_OP_RY:
        case LLG_OP_RZ:
            if ((rc = check_qubit(st, op.q0, who))) return rc;
            return check_angle(op.theta, who);
        case LLG_OP_U2:
            if ((rc = check_qubit(st, op.q0, who))) return rc;
            for (int k = 0; k < 8; ++k)
                if (!finite(op.m[k])) return set_error(LLG_EINVAL, std::string(who) + ": non-finite gate entry");
            return LLG_OK;
        case LLG_OP_CNOT:
            if ((rc = check_qubit(st, op.q0, who)) || (rc = check_qubit(st, op.q1, who))) return rc;
            if (op.q0 == op.q1) return set_error(LLG_EINVAL, std::string(who) + ": control == target");
            return LLG_OK;
        case LLG_OP_CZ:
            if ((rc = check_qubit(st, op.q0, who)) || (rc = check_qubit(st, op.q1, who))) return rc;
            if (op.q0 == op.q1) return set_error(LLG_EINVAL, std::string(who) + ": duplicate qubit");
            return LLG_OK;
        case LLG_OP_MCZ:
            if (op.mask == 0) return set_error(LLG_EINVAL, std::string(who) + ": empty qubit list");
            if (st->n < 64 && (op.mask >> st->n) != 0) return set_error(LLG_EINVAL, std::string(who) + ": qubit outside [0, n)");
            return LLG_OK;
        default:
            return set_error(LLG_EINVAL, std::string(who) + ": unknown op kind " + std::to_string(op.kind));
    }
}

}  // namespace

// ------------------------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------------------------
extern "C" {

const char* llg_last_error(void) { return g_last_error.c_str(); }

const char* llg_version(void) { return "llgpu 0.1 (sm_103a)"; }

int llg_device_count(void) {
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return c;
}

int llg_create(int n_qubits, int precision, llg_state** out) {
    if (!out) return set_error(LLG_EINVAL, "llg_create: out is NULL");
    *out = nullptr;
    if (n_qubits < 1 || n_qubits > kMaxQubits)
        return set_error(LLG_EINVAL, "llg_create: n_qubits must be in [1, " + std::to_string(kMaxQubits) + "]");
    if (precision != LLG_F64 && precision != LLG_DF64 && precision != LLG_F32)
        return set_error(LLG_EINVAL, "llg_create: unknown precision");
    llg_state* st = new llg_state();
    st->P = precision;
    int rc = ensure_device_buffers(st);
    if (!rc) rc = alloc_state(st, n_qubits);
    if (!rc)
        rc = traced(st, LLG_PROF_INIT, 1, "init", [&] { return launch_init_basis(st->P, st->d_psi, st->size, 0, st->stream); });
    if (rc) {
        llg_destroy(st);
        return rc;
    }
    *out = st;
    return LLG_OK;
}

int llg_create_from_host(const double* amps, size_t len, int precision, llg_state** out) {
    if (!out) return set_error(LLG_EINVAL, "llg_create_from_host: out is NULL");
    *out = nullptr;
    int n = 0;
    while ((len >> n) > 1) ++n;
    if (len == 0 || (1ULL << n) != len) return set_error(LLG_ERUNTIME, "Array size must be power of 2");
    if (n > kMaxQubits) return set_error(LLG_EINVAL, "llg_create_from_host: too many amplitudes");
    if (precision != LLG_F64 && precision != LLG_DF64 && precision != LLG_F32)
        return set_error(LLG_EINVAL, "llg_create_from_host: unknown precision");
    if (!amps) return set_error(LLG_EINVAL, "llg_create_from_host: amps is NULL");
    llg_state* st = new llg_state();
    st->P = precision;
    int rc = ensure_device_buffers(st);
    if (!rc) {
        // n == 0 is a one-amplitude state: kept (the reference accepts it), every gate is a no-op
        const uint64_t size = 1ULL << n;
        cudaError_t e = cudaMalloc(&st->d_psi, size * elem_bytes(precision));
        if (e != cudaSuccess) {
            cudaGetLastError();
            rc = set_error(LLG_ENOMEM, std::string("cannot allocate HBM: ") + cudaGetErrorString(e));
        } else {
            st->n = n;
            st->size = size;
            rc = llg_copy_from_host(st, amps);
        }
    }
    if (rc) {
        llg_destroy(st);
        return rc;
    }
    *out = st;
    return LLG_OK;
}

int llg_destroy(llg_state* st) {
    if (!st) return LLG_OK;
    if (st->stream) cudaStreamSynchronize(st->stream);
    if (st->d_psi) cudaFree(st->d_psi);
    if (st->d_ops) cudaFree(st->d_ops);
    if (st->h_ops) cudaFreeHost(st->h_ops);
    if (st->d_tables) cudaFree(st->d_tables);
    if (st->h_tables) cudaFreeHost(st->h_tables);
    if (st->d_partials) cudaFree(st->d_partials);
    if (st->d_red) cudaFree(st->d_red);
    if (st->d_flags) cudaFree(st->d_flags);
    if (st->d_obs) cudaFree(st->d_obs);
    if (st->d_diag) cudaFree(st->d_diag);
    for (int i = 0; i < 2; ++i) {
        if (st->d_stage[i]) cudaFree(st->d_stage[i]);
        if (st->stage_ev[i]) cudaEventDestroy(st->stage_ev[i]);
    }
    if (st->ops_done) cudaEventDestroy(st->ops_done);
    if (st->d_block) cudaFree(st->d_block);
    if (st->h_block) cudaFreeHost(st->h_block);
    if (st->d_block_tc) cudaFree(st->d_block_tc);
    if (st->h_block_tc) cudaFreeHost(st->h_block_tc);
    if (st->block_done) cudaEventDestroy(st->block_done);
    for (auto& r : st->prof_recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (cudaEvent_t e : st->ev_pool) cudaEventDestroy(e);
    if (st->stream) cudaStreamDestroy(st->stream);
    delete st;
    return LLG_OK;
}

int llg_reset(llg_state* st, int n_qubits) {
    if (!st) return set_error(LLG_EINVAL, "llg_reset: NULL state");
    if (n_qubits < 1 || n_qubits > kMaxQubits)
        return set_error(LLG_EINVAL, "llg_reset: n_qubits must be in [1, " + std::to_string(kMaxQubits) + "]");
    st->queue.clear();
    int rc = alloc_state(st, n_qubits);
    if (rc) return rc;
    return traced(st, LLG_PROF_INIT, 1, "init", [&] { return launch_init_basis(st->P, st->d_psi, st->size, 0, st->stream); });
}

int llg_num_qubits(const llg_state* st, int* out) {
    if (!st || !out) return set_error(LLG_EINVAL, "llg_num_qubits: NULL argument");
    *out = st->n;
    return LLG_OK;
}

int llg_size(const llg_state* st, uint64_t* out) {
    if (!st || !out) return set_error(LLG_EINVAL, "llg_size: NULL argument");
    *out = st->size;
    return LLG_OK;
}

int llg_get_precision(const llg_state* st, int* out) {
    if (!st || !out) return set_error(LLG_EINVAL, "llg_get_precision: NULL argument");
    *out = st->P;
    return LLG_OK;
}

int llg_set_fusion(llg_state* st, int mode, int tile_qubits) {
    if (!st) return set_error(LLG_EINVAL, "llg_set_fusion: NULL state");
    if (mode != LLG_FUSE_NONE && mode != LLG_FUSE_TILE && mode != LLG_FUSE_REG)
        return set_error(LLG_EINVAL, "llg_set_fusion: unknown mode");
    if (mode == LLG_FUSE_REG && (st->P != LLG_F32 || (tile_qubits != 0 && (tile_qubits < 9 || tile_qubits > 13))))
        return set_error(LLG_EINVAL, "llg_set_fusion: register-tiled passes take complex64 states and tiles of 9..13 qubits");
    if (tile_qubits < 0 || tile_qubits > tile_max_qubits(st->P) || (tile_qubits > 0 && tile_qubits < 5))
        return set_error(LLG_EINVAL, "llg_set_fusion: tile_qubits must be 0 or in [5, " +
                                         std::to_string(tile_max_qubits(st->P)) + "]");
    int rc = llg_flush(st);
    if (rc) return rc;
    st->fuse_mode = mode;
    st->tile_qubits = tile_qubits;
    return LLG_OK;
}

int llg_set_tile_threads(llg_state* st, int threads) {
    if (!st) return set_error(LLG_EINVAL, "llg_set_tile_threads: NULL state");
    if (threads != 0 && (threads < 32 || threads > 1024 || (threads & 31)))
        return set_error(LLG_EINVAL, "llg_set_tile_threads: threads must be 0 or a multiple of 32 in [32, 1024]");
    int rc = llg_flush(st);
    if (rc) return rc;
    st->tile_threads = threads;
    return LLG_OK;
}

int llg_get_tuning(const llg_state* st, int* fuse_mode, int* tile_qubits, int* tile_threads) {
    if (!st) return set_error(LLG_EINVAL, "llg_get_tuning: NULL state");
    if (fuse_mode) *fuse_mode = st->fuse_mode;
    if (tile_qubits) *tile_qubits = st->tile_qubits > 0 ? st->tile_qubits : default_tile(st->P);
    if (tile_threads) *tile_threads = st->tile_threads;
    return LLG_OK;
}

int llg_apply_gate(llg_state* st, int target, const double* g) {
    if (!st || !g) return set_error(LLG_EINVAL, "apply_gate: NULL argument");
    if (target < 0) return set_error(LLG_EINVAL, "apply_gate: negative target " + std::to_string(target));
    if (target >= st->n) return LLG_OK;  // reference: num_blocks = size >> (k+1) = 0, a no-op
    llg_op op = make_op(LLG_OP_U2, target);
    std::memcpy(op.m, g, 8 * sizeof(double));
    return enqueue(st, op);
}

#define LLG_GATE1(name, KIND, who)                                    \
    int name(llg_state* st, int q) {                                  \
        if (!st) return set_error(LLG_EINVAL, who ": NULL state");    \
        llg_op op = make_op(KIND, q);                                 \
        int rc = validate_op(st, op, who);                            \
        return rc ? rc : enqueue(st, op);                             \
    }
LLG_GATE1(llg_h, LLG_OP_H, "h")
LLG_GATE1(llg_x, LLG_OP_X, "x")

#define LLG_ROT(name, KIND, who)                                      \
    int name(llg_state* st, int q, double theta) {                    \
        if (!st) return set_error(LLG_EINVAL, who ": NULL state");    \
        llg_op op = make_op(KIND, q, 0, theta);                       \
        int rc = validate_op(st, op, who);                            \
        return rc ? rc : enqueue(st, op);                             \
    }
LLG_ROT(llg_rx, LLG_OP_RX, "rx")
LLG_ROT(llg_ry, LLG_OP_RY, "ry")
LLG_ROT(llg_rz, LLG_OP_RZ, "rz")

int llg_cnot(llg_state* st, int control, int target) {
    if (!st) return set_error(LLG_EINVAL, "cnot: NULL state");
    llg_op op = make_op(LLG_OP_CNOT, control, target);
    int rc = validate_op(st, op, "cnot");
    return rc ? rc : enqueue(st, op);
}

int llg_cz(llg_state* st, int a, int b) {
    if (!st) return set_error(LLG_EINVAL, "cz: NULL state");
    llg_op op = make_op(LLG_OP_CZ, a, b);
    int rc = validate_op(st, op, "cz");
    return rc ? rc : enqueue(st, op);
}

int llg_mcz(llg_state* st, const int* qubits, int nq) {
    if (!st) return set_error(LLG_EINVAL, "mcz: NULL state");
    if (nq <= 0 || !qubits) return set_error(LLG_EINVAL, "mcz: empty qubit list");
    uint64_t mask = 0;
    for (int i = 0; i < nq; ++i) {
        int rc = check_qubit(st, qubits[i], "mcz");
        if (rc) return rc;
        const uint64_t b = 1ULL << qubits[i];
        if (mask & b) return set_error(LLG_EINVAL, "mcz: duplicate qubit");
        mask |= b;
    }
    return enqueue(st, make_op(LLG_OP_MCZ, qubits[0], 0, 0.0, mask));
}

int llg_apply_ops(llg_state* st, const llg_op* ops, int nops) {
    if (!st || (nops > 0 && !ops)) return set_error(LLG_EINVAL, "apply_ops: NULL argument");
    if (nops < 0) return set_error(LLG_EINVAL, "apply_ops: negative count");
    for (int i = 0; i < nops; ++i) {
        int rc = validate_op(st, ops[i], "apply_ops");
        if (rc) return set_error(rc, g_last_error + " (op " + std::to_string(i) + ")");
    }
    for (int i = 0; i < nops; ++i) {
        int rc = enqueue(st, ops[i]);
        if (rc) return rc;
    }
    return LLG_OK;
}

int llg_wrap_host(const double* amps, size_t len, int precision, llg_state** out) {
    return llg_create_from_host(amps, len, precision, out);
}

int llg_apply_1q(llg_state* st, int q, const double* m) {
    if (!st || !m) return set_error(LLG_EINVAL, "apply_1q: NULL argument");
    if (int rc = check_qubit(st, q, "StateVectorBackend")) return rc;
    return llg_apply_gate(st, q, m);
}

int llg_apply_block(llg_state* st, int k, const int* qubits, const double* m) { return llg_apply_matrix(st, k, qubits, m); }

int llg_expect_diag_zz(llg_state* st, int nterms, const int* a, const int* b, const double* coeff, double* out) {
    return llg_expect_zz(st, nterms, a, b, coeff, out);
}

int llg_apply_matrix(llg_state* st, int k, const int* qubits, const double* m) {
    if (!st || !qubits || !m) return set_error(LLG_EINVAL, "apply_matrix: NULL argument");
    if (k < 1 || k > kMaxBlockQubits || k > st->n)
        return set_error(LLG_EINVAL, "apply_matrix: k must be in [1, 5] and at most the register size");
    BlockDesc bd;
    std::memset(&bd, 0, sizeof(bd));
    bd.k = k;
    for (int j = 0; j < k; ++j) {
        int rc = check_qubit(st, qubits[j], "apply_matrix");
        if (rc) return rc;
        if ((bd.tmask >> qubits[j]) & 1) return set_error(LLG_EINVAL, "apply_matrix: repeated qubit");
        bd.tmask |= 1ULL << qubits[j];
        bd.q[j] = qubits[j];
    }
    const int slots = 2 << (2 * k);  // 2 * 4^k
    for (int i = 0; i < slots; ++i)
        if (!std::isfinite(m[i])) return set_error(LLG_EINVAL, "apply_matrix: non-finite matrix entry");
    int rc = llg_flush(st);  // earlier gates first
    if (rc) return rc;
    const size_t cap = (size_t)2 * kMaxBlockDim * kMaxBlockDim;
    if (!st->d_block) {
        LLG_CUDA(cudaMalloc(&st->d_block, cap * sizeof(uint64_t)), "cudaMalloc(block)");
        LLG_CUDA(cudaHostAlloc((void**)&st->h_block, cap * sizeof(uint64_t), cudaHostAllocDefault), "cudaHostAlloc(block)");
        LLG_CUDA(cudaEventCreateWithFlags(&st->block_done, cudaEventDisableTiming), "cudaEventCreate");
    }
    if (st->block_pending) LLG_CUDA(cudaEventSynchronize(st->block_done), "block staging");
    // a mostly-zero block (noise-channel superoperators) runs only its nonzero entries: two
    // multiply-adds per real entry, four per complex one, against four per entry dense
    BlockSparsity nz;
    std::memset(&nz, 0, sizeof(nz));
    int sparse_cost = 0;
    const int dim = 1 << k;
    for (int r = 0; r < dim; ++r)
        for (int c = 0; c < dim; ++c) {
            const double re = m[2 * (r * dim + c)], im = m[2 * (r * dim + c) + 1];
            if (re == 0.0 && im == 0.0) continue;
            nz.rows[r] |= 1u << c;
            if (im == 0.0) nz.real[r] |= 1u << c;
            sparse_cost += im == 0.0 ? 2 : 4;
        }
    if (k <= 4 && 2 * sparse_cost <= 4 * dim * dim) {
        for (int i = 0; i < slots; ++i) st->h_block[i] = pack_coef(st->P, m[i]);
        LLG_CUDA(cudaMemcpyAsync(st->d_block, st->h_block, slots * sizeof(uint64_t), cudaMemcpyHostToDevice, st->stream),
                 "cudaMemcpyAsync(block)");
        LLG_CUDA(cudaEventRecord(st->block_done, st->stream), "cudaEventRecord");
        st->block_pending = true;
        return traced(st, LLG_PROF_GATE, 1, "block kernel (sparse)",
                      [&] { return launch_block_sparse(st->P, st->d_psi, st->n, bd, st->d_block, nz, st->stream); });
    }
    // An IEEE complex128 2-qubit block runs as a 3-qubit one, and a double-float 3-qubit block as
    // a 4-qubit one: M on its qubits and the identity on the lowest other qubit, on the tensor
    // cores, which beat the CUDA-core forms there (30 qubits: FP64 k = 2 28.2 -> 18.2 ms,
    // double-float k = 3 13.2 -> 10.4 ms)
    double mx[2 * 16 * 16];
    if (((st->P == LLG_F64 && k == 2) || (st->P == LLG_DF64 && k == 3)) && block_tc_eligible(st->P, st->n, k + 1)) {
        int x = 0;
        while ((bd.tmask >> x) & 1) ++x;
        const int d = 1 << k, dx = 2 * d;
        std::memset(mx, 0, sizeof(mx));
        for (int r = 0; r < dx; ++r)
            for (int c = 0; c < dx; ++c)
                if ((r >> k) == (c >> k)) {  // bit k of the index is qubit x
                    mx[2 * (r * dx + c)] = m[2 * ((r & (d - 1)) * d + (c & (d - 1)))];
                    mx[2 * (r * dx + c) + 1] = m[2 * ((r & (d - 1)) * d + (c & (d - 1))) + 1];
                }
        bd.q[k] = x;
        bd.tmask |= 1ULL << x;
        bd.k = ++k;
        m = mx;
    }
    if (block_tc_eligible(st->P, st->n, k)) {
        const size_t wb = block_tc_weight_bytes(st->P, k);
        if (!st->d_block_tc) {
            // the largest weight set of any precision (the eight-slice FP64 one)
            const size_t cap = std::max(block_tc_weight_bytes(LLG_DF64, kMaxBlockQubits),
                                        block_tc_weight_bytes(LLG_F64, kMaxBlockQubits));
            LLG_CUDA(cudaMalloc(&st->d_block_tc, cap), "cudaMalloc(block weights)");
            LLG_CUDA(cudaHostAlloc((void**)&st->h_block_tc, cap, cudaHostAllocDefault), "cudaHostAlloc(block weights)");
        }
        if (wb > std::max(block_tc_weight_bytes(LLG_DF64, kMaxBlockQubits), block_tc_weight_bytes(LLG_F64, kMaxBlockQubits)))
            return set_error(LLG_ERUNTIME, "apply_matrix: block weights larger than their staging buffer");
        block_tc_prepare(st->P, k, m, st->h_block_tc);
        LLG_CUDA(cudaMemcpyAsync(st->d_block_tc, st->h_block_tc, wb, cudaMemcpyHostToDevice, st->stream),
                 "cudaMemcpyAsync(block weights)");
        LLG_CUDA(cudaEventRecord(st->block_done, st->stream), "cudaEventRecord");
        st->block_pending = true;
        st->block_tc_launched = true;
        return traced(st, LLG_PROF_GATE, 1, "block kernel (tensor cores)",
                      [&] { return launch_block_tc(st->P, st->d_psi, st->n, bd, st->d_block_tc, st->d_flags, st->stream); });
    }
    for (int i = 0; i < slots; ++i) st->h_block[i] = pack_coef(st->P, m[i]);
    LLG_CUDA(cudaMemcpyAsync(st->d_block, st->h_block, slots * sizeof(uint64_t), cudaMemcpyHostToDevice, st->stream),
             "cudaMemcpyAsync(block)");
    LLG_CUDA(cudaEventRecord(st->block_done, st->stream), "cudaEventRecord");
    st->block_pending = true;
    return traced(st, LLG_PROF_GATE, 1, "block kernel",
                  [&] { return launch_block(st->P, st->d_psi, st->n, bd, st->d_block, st->stream); });
}

int llg_dm_apply_op(llg_state* st, int n, const llg_op* op) {
    if (!st || !op) return set_error(LLG_EINVAL, "dm_apply_op: NULL argument");
    if (n < 1 || n > 17 || st->n != 2 * n) return set_error(LLG_EINVAL, "dm_apply_op: the state must hold 2n qubits");
    const bool two = op->kind == LLG_OP_CNOT || op->kind == LLG_OP_CZ;
    if (op->kind == LLG_OP_MCZ) {
        if (op->mask == 0 || (op->mask >> n) != 0) return set_error(LLG_EINVAL, "dm_apply_op: mcz mask outside the register");
    } else if (op->q0 < 0 || op->q0 >= n || (two && (op->q1 < 0 || op->q1 >= n))) {
        return set_error(LLG_EINVAL, "dm_apply_op: qubit outside the register");
    }
    // U rho U^+: U on the row qubits [0, n), conj(U) on the column qubits [n, 2n)
    llg_op col = *op;
    col.q0 = op->q0 + n;
    col.q1 = op->q1 + n;
    col.mask = op->mask << n;
    if (op->kind == LLG_OP_RX || op->kind == LLG_OP_RZ) col.theta = -op->theta;
    if (op->kind == LLG_OP_U2)
        for (int i = 0; i < 4; ++i) col.m[2 * i + 1] = -op->m[2 * i + 1];
    const llg_op pair[2] = {*op, col};
    return llg_apply_ops(st, pair, 2);
}

int llg_dm_apply_kraus(llg_state* st, int n, int nkraus, const double* kraus, int m, const int* targets) {
    if (!st || !kraus || !targets) return set_error(LLG_EINVAL, "KrausChannel::apply: NULL argument");
    if (n < 1 || n > 17 || st->n != 2 * n) return set_error(LLG_EINVAL, "KrausChannel::apply: the state must hold 2n qubits");
    if (m < 1 || m > 2 || nkraus < 1) return set_error(LLG_EINVAL, "KrausChannel::apply: 1 or 2 targets and at least one operator");
    for (int j = 0; j < m; ++j) {
        if (targets[j] < 0 || targets[j] >= n) return set_error(LLG_EINVAL, "KrausChannel::apply: target qubit outside the register");
        for (int i = 0; i < j; ++i)
            if (targets[i] == targets[j]) return set_error(LLG_EINVAL, "KrausChannel: repeated target qubit");
    }
    const int d = 1 << m;
    typedef std::complex<double> cd;
    auto K = [&](int k, int r, int c) { return cd(kraus[2 * ((size_t)k * d * d + r * d + c)], kraus[2 * ((size_t)k * d * d + r * d + c) + 1]); };
    // trace preservation to 1e-10 (src/Noise.cpp:166-172, DEFAULT_TOL)
    double worst = 0.0;
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) {
            cd sum = 0.0;
            for (int k = 0; k < nkraus; ++k)
                for (int r = 0; r < d; ++r) sum += std::conj(K(k, r, i)) * K(k, r, j);
            if (i == j) sum -= 1.0;
            if (!std::isfinite(sum.real()) || !std::isfinite(sum.imag())) return set_error(LLG_EINVAL, "KrausChannel: non-finite operator entry");
            worst = std::max(worst, std::abs(sum));
        }
    if (!(worst <= 1e-10)) return set_error(LLG_EINVAL, "KrausChannel: operators are not trace preserving");
    // superoperator S = sum_k K (x) conj(K) on qubits [targets..., n + targets...]: block index
    // bits 0..m-1 are the row targets, bits m..2m-1 the column targets
    const int D = d * d;
    std::vector<double> S((size_t)2 * D * D, 0.0);
    for (int k = 0; k < nkraus; ++k)
        for (int r = 0; r < d; ++r)
            for (int c = 0; c < d; ++c)
                for (int r2 = 0; r2 < d; ++r2)
                    for (int c2 = 0; c2 < d; ++c2) {
                        const cd v = K(k, r, r2) * std::conj(K(k, c, c2));
                        const size_t e = (size_t)(r | (c << m)) * D + (size_t)(r2 | (c2 << m));
                        S[2 * e] += v.real();
                        S[2 * e + 1] += v.imag();
                    }
    int qs[4];
    for (int j = 0; j < m; ++j) {
        qs[j] = targets[j];
        qs[m + j] = targets[j] + n;
    }
    return llg_apply_matrix(st, 2 * m, qs, S.data());
}

int llg_flush(llg_state* st) {
    if (!st) return set_error(LLG_EINVAL, "flush: NULL state");
    if (st->queue.empty()) return LLG_OK;
    std::vector<llg_op> q;
    q.swap(st->queue);
    if (st->n == 0) return LLG_OK;
    return st->fuse_mode != LLG_FUSE_NONE ? run_tiles(st, q) : run_streaming(st, q);
}

// After the state's stream has drained: the timeout flags of the kernels that wait on the
// asynchronous units (tensor-core products, bulk tile loads), for the launches since the last check.
// The flags are this state's own, read and cleared on its own stream.
static int device_checks(llg_state* st) {
    if (!st->block_tc_launched && !st->tiles_launched) return LLG_OK;
    const bool tc = st->block_tc_launched, tiles = st->tiles_launched;
    st->block_tc_launched = st->tiles_launched = false;
    int h[2] = {0, 0};
    LLG_CUDA(cudaMemcpyAsync(h, st->d_flags, sizeof(h), cudaMemcpyDeviceToHost, st->stream), "cudaMemcpyAsync(flags)");
    LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");
    if (h[0] || h[1]) LLG_CUDA(cudaMemsetAsync(st->d_flags, 0, sizeof(h), st->stream), "cudaMemsetAsync(flags)");
    if (tc && h[1]) return set_error(LLG_ECUDA, "apply_matrix: a tensor-core block kernel timed out waiting for its products");
    if (tiles && h[0]) return set_error(LLG_ECUDA, "tile pass: a bulk tile load timed out");
    return LLG_OK;
}

int llg_sync(llg_state* st) {
    int rc = llg_flush(st);
    if (rc) return rc;
    LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");
    return device_checks(st);
}

// Device address of pinned, mapped host memory (cudaHostAlloc / cudaHostRegister), else nullptr.
static void* mapped_device_pointer(void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int llg_copy_to_host(llg_state* st, double* out) {
    if (!st || !out) return set_error(LLG_EINVAL, "copy_to_host: NULL argument");
    void* const dev_out = mapped_device_pointer(out);
    int rc;
    // Gates still queued for tile passes: the last pass writes the host buffer as it stores its
    // tiles, so the transfer runs under that pass's arithmetic instead of after it.
    if (dev_out && !st->queue.empty() && st->n > 0 && st->fuse_mode != LLG_FUSE_NONE) {
        std::vector<llg_op> q;
        q.swap(st->queue);
        bool mirrored = false;
        if ((rc = run_tiles(st, q, static_cast<double*>(dev_out), &mirrored))) return rc;
        if (mirrored) {
            LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");
            return device_checks(st);
        }
    }
    rc = llg_flush(st);
    if (rc) return rc;
    // A pinned destination is written by the conversion kernel itself (a plain copy for FP64
    // states), over the host link: one pass at the link's rate, with no staging copy and no
    // copy-engine step after each chunk.
    if (dev_out) {
        rc = traced(st, LLG_PROF_READOUT, 1, "to_f64",
                    [&] { return launch_to_f64(st->P, st->d_psi, static_cast<double*>(dev_out), st->size, st->stream); });
        if (rc) return rc;
        LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");
        return device_checks(st);
    }
    if (st->P == LLG_F64) {  // pageable destination, same layout: one copy
        LLG_CUDA(cudaMemcpyAsync(out, st->d_psi, st->size * 16, cudaMemcpyDeviceToHost, st->stream), "cudaMemcpyAsync(D2H)");
        LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");
        return device_checks(st);
    }
    if ((rc = stage_buffers(st))) return rc;
    const size_t eb = elem_bytes(st->P);
    int which = 0;
    for (uint64_t off = 0; off < st->size; off += kStageAmps, which ^= 1) {
        const uint64_t cnt = std::min<uint64_t>(kStageAmps, st->size - off);
        LLG_CUDA(cudaEventSynchronize(st->stage_ev[which]), "cudaEventSynchronize");
        rc = traced(st, LLG_PROF_READOUT, 1, "to_f64", [&] {
            return launch_to_f64(st->P, (const char*)st->d_psi + off * eb, st->d_stage[which], cnt, st->stream);
        });
        if (rc) return rc;
        LLG_CUDA(cudaMemcpyAsync(out + 2 * off, st->d_stage[which], cnt * 16, cudaMemcpyDeviceToHost, st->stream),
                 "cudaMemcpyAsync(D2H)");
        LLG_CUDA(cudaEventRecord(st->stage_ev[which], st->stream), "cudaEventRecord");
    }
    LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");
    return device_checks(st);
}

int llg_copy_from_host(llg_state* st, const double* amps) {
    if (!st || !amps) return set_error(LLG_EINVAL, "copy_from_host: NULL argument");
    st->queue.clear();  // overwritten anyway
    if (st->P == LLG_F64) {
        LLG_CUDA(cudaMemcpyAsync(st->d_psi, amps, st->size * 16, cudaMemcpyHostToDevice, st->stream), "cudaMemcpyAsync(H2D)");
        LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");
        return LLG_OK;
    }
    int rc = stage_buffers(st);
    if (rc) return rc;
    const size_t eb = elem_bytes(st->P);
    int which = 0;
    for (uint64_t off = 0; off < st->size; off += kStageAmps, which ^= 1) {
        const uint64_t cnt = std::min<uint64_t>(kStageAmps, st->size - off);
        LLG_CUDA(cudaEventSynchronize(st->stage_ev[which]), "cudaEventSynchronize");
        LLG_CUDA(cudaMemcpyAsync(st->d_stage[which], amps + 2 * off, cnt * 16, cudaMemcpyHostToDevice, st->stream),
                 "cudaMemcpyAsync(H2D)");
        rc = traced(st, LLG_PROF_READOUT, 1, "from_f64", [&] {
            return launch_from_f64(st->P, st->d_stage[which], (char*)st->d_psi + off * eb, cnt, st->stream);
        });
        if (rc) return rc;
        LLG_CUDA(cudaEventRecord(st->stage_ev[which], st->stream), "cudaEventRecord");
    }
    LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");
    return LLG_OK;
}

int llg_probabilities(llg_state* st, double* out) {
    if (!st || !out) return set_error(LLG_EINVAL, "probabilities: NULL argument");
    int rc = llg_flush(st);
    if (rc) return rc;
    if ((rc = stage_buffers(st))) return rc;
    const size_t eb = elem_bytes(st->P);
    const uint64_t chunk = kStageAmps * 2;  // doubles per staging buffer
    int which = 0;
    for (uint64_t off = 0; off < st->size; off += chunk, which ^= 1) {
        const uint64_t cnt = std::min<uint64_t>(chunk, st->size - off);
        LLG_CUDA(cudaEventSynchronize(st->stage_ev[which]), "cudaEventSynchronize");
        rc = traced(st, LLG_PROF_READOUT, 1, "probabilities", [&] {
            return launch_probabilities(st->P, (const char*)st->d_psi + off * eb, st->d_stage[which], cnt, st->stream);
        });
        if (rc) return rc;
        LLG_CUDA(cudaMemcpyAsync(out + off, st->d_stage[which], cnt * 8, cudaMemcpyDeviceToHost, st->stream),
                 "cudaMemcpyAsync(D2H)");
        LLG_CUDA(cudaEventRecord(st->stage_ev[which], st->stream), "cudaEventRecord");
    }
    LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");
    return device_checks(st);
}

// The class-counting kernel takes up to kMaxZTerms terms with up to kMaxZClasses distinct
// coefficient values; it counts parities per class in integers.
static bool fits_class_kernel(int nterms, const double* coeff) {
    if (nterms < 0 || nterms > kMaxZTerms) return false;
    double seen[kMaxZClasses];
    int ns = 0;
    for (int k = 0; k < nterms; ++k) {
        bool found = false;
        for (int j = 0; j < ns; ++j) found |= seen[j] == coeff[k];
        if (!found) {
            if (ns == kMaxZClasses) return false;
            seen[ns++] = coeff[k];
        }
    }
    return true;
}

static int build_zterms(int nterms, const int* a, const int* b, const double* coeff, int n, ZTerms& z) {
    if (nterms < 0 || nterms > kMaxZTerms)
        return set_error(LLG_EINVAL, "expect_zz: at most " + std::to_string(kMaxZTerms) + " terms");
    std::memset(&z, 0, sizeof(z));
    z.nterms = nterms;
    for (int k = 0; k < nterms; ++k) {
        if (a[k] < 0 || a[k] >= n || b[k] >= n || b[k] == a[k])
            return set_error(LLG_EINVAL, "expect_zz: term " + std::to_string(k) + " has a bad qubit");
        if (!std::isfinite(coeff[k])) return set_error(LLG_EINVAL, "expect_zz: non-finite coefficient");
        int c = -1;
        for (int j = 0; j < z.nclass; ++j)
            if (z.coef[j] == coeff[k]) c = j;
        if (c < 0) {
            if (z.nclass == kMaxZClasses)
                return set_error(LLG_EINVAL, "expect_zz: at most " + std::to_string(kMaxZClasses) + " distinct coefficients");
            c = z.nclass++;
            z.coef[c] = coeff[k];
        }
        z.a[k] = a[k];
        z.b[k] = b[k] < 0 ? -1 : b[k];
        z.cls[k] = c;
    }
    return LLG_OK;
}

static int reduce(llg_state* st, const ZTerms& z, double* slots) {
    int rc = llg_flush(st);
    if (rc) return rc;
    rc = traced(st, LLG_PROF_READOUT, 2, "reduce",
                [&] { return launch_reduce_z(st->P, st->d_psi, st->n, z, st->d_partials, st->d_red, st->stream); });
    if (rc) return rc;
    LLG_CUDA(cudaMemcpyAsync(slots, st->d_red, sizeof(double) * kRedSlots, cudaMemcpyDeviceToHost, st->stream),
             "cudaMemcpyAsync(D2H)");
    LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");
    return device_checks(st);
}

int llg_compare(llg_state* a, llg_state* b, double* fidelity, double* max_abs_diff) {
    return llg_compare_ex(a, b, fidelity, max_abs_diff, nullptr);
}

int llg_compare_ex(llg_state* a, llg_state* b, double* fidelity, double* max_abs_diff, double* max_abs_b) {
    if (!a || !b) return set_error(LLG_EINVAL, "compare: NULL state");
    if (a->n != b->n) return set_error(LLG_EINVAL, "compare: the states have different qubit counts");
    int rc = llg_flush(a);
    if (!rc) rc = llg_flush(b);
    if (rc) return rc;
    if ((rc = ensure_device_buffers(a))) return rc;  // the partial-sum buffer
    LLG_CUDA(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    int nblocks = 0;
    LLG_CUDA(launch_compare(a->P, a->d_psi, b->P, b->d_psi, a->size, a->d_partials, &nblocks, a->stream), "compare kernel");
    std::vector<double> part((size_t)nblocks * kCmpSlots);
    LLG_CUDA(cudaMemcpyAsync(part.data(), a->d_partials, part.size() * sizeof(double), cudaMemcpyDeviceToHost, a->stream),
             "cudaMemcpyAsync(D2H)");
    LLG_CUDA(cudaStreamSynchronize(a->stream), "cudaStreamSynchronize");
    if ((rc = device_checks(a)) || (rc = device_checks(b))) return rc;
    double re = 0.0, im = 0.0, na = 0.0, nb = 0.0, mx = 0.0, mb = 0.0;
    for (int k = 0; k < nblocks; ++k) {  // fixed order
        re += part[(size_t)k * kCmpSlots];
        im += part[(size_t)k * kCmpSlots + 1];
        na += part[(size_t)k * kCmpSlots + 2];
        nb += part[(size_t)k * kCmpSlots + 3];
        mx = std::max(mx, part[(size_t)k * kCmpSlots + 4]);
        mb = std::max(mb, part[(size_t)k * kCmpSlots + 5]);
    }
    if (fidelity) *fidelity = (na > 0.0 && nb > 0.0) ? (re * re + im * im) / (na * nb) : 0.0;
    if (max_abs_diff) *max_abs_diff = mx;
    if (max_abs_b) *max_abs_b = mb;
    return LLG_OK;
}

int llg_norm2(llg_state* st, double* out) {
    if (!st || !out) return set_error(LLG_EINVAL, "norm2: NULL argument");
    ZTerms z;
    std::memset(&z, 0, sizeof(z));
    double slots[kRedSlots];
    int rc = reduce(st, z, slots);
    if (rc) return rc;
    *out = slots[0];
    return LLG_OK;
}

// sum_i |a_i|^2 d(i) for a general diagonal observable: out[0] the energy, out[1] the norm^2
static int reduce_diag(llg_state* st, const DiagObs& o, double* out2) {
    int rc = llg_flush(st);
    if (rc) return rc;
    if ((rc = ensure_device_buffers(st))) return rc;
    rc = traced(st, LLG_PROF_READOUT, 2, "diagonal observable",
                [&] { return launch_expect_diag(st->P, st->d_psi, o, st->d_partials, st->d_red, st->stream); });
    if (rc) return rc;
    LLG_CUDA(cudaMemcpyAsync(out2, st->d_red, 2 * sizeof(double), cudaMemcpyDeviceToHost, st->stream),
             "cudaMemcpyAsync(D2H)");
    LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");
    return device_checks(st);
}

// The observable's layout on the device (rebuilt and uploaded only when the terms change).
static int upload_obs(llg_state* st, int nterms, const int* a, const int* b, const double* coeff, DiagObs* view) {
    if (!diag_obs_same(st->obs, st->n, nterms, a, b, coeff)) {
        std::string err;
        DiagObsHost h;
        if (!build_diag_obs(st->n, nterms, a, b, coeff, h, err)) return set_error(LLG_EINVAL, "expect_zz: " + err);
        int rc = ensure_device_buffers(st);
        if (rc) return rc;
        if (h.bytes.size() > st->d_obs_cap) {
            LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");
            if (st->d_obs) cudaFree(st->d_obs);
            st->d_obs = nullptr;
            st->d_obs_cap = 0;
            LLG_CUDA(cudaMalloc(&st->d_obs, h.bytes.size()), "cudaMalloc(observable)");
            st->d_obs_cap = h.bytes.size();
        }
        // ordered on the stream after any kernel still reading the previous observable
        LLG_CUDA(cudaMemcpyAsync(st->d_obs, h.bytes.data(), h.bytes.size(), cudaMemcpyHostToDevice, st->stream),
                 "cudaMemcpyAsync(observable)");
        LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");  // h's bytes are freed below
        st->obs = std::move(h);
    }
    *view = diag_obs_view(st->obs, st->d_obs);
    return LLG_OK;
}

int llg_expect_zz(llg_state* st, int nterms, const int* a, const int* b, const double* coeff, double* out) {
    if (!st || !out || (nterms > 0 && (!a || !b || !coeff))) return set_error(LLG_EINVAL, "expect_zz: NULL argument");
    int rc;
    if (!fits_class_kernel(nterms, coeff)) {
        // more terms or coefficient values than the class-counting kernel takes: the general
        // chunked kernel (any number of terms, any coefficients)
        DiagObs o;
        if ((rc = upload_obs(st, nterms, a, b, coeff, &o))) return rc;
        double r[2];
        if ((rc = reduce_diag(st, o, r))) return rc;
        *out = r[0];
        return LLG_OK;
    }
    ZTerms z;
    if ((rc = build_zterms(nterms, a, b, coeff, st->n, z))) return rc;
    double slots[kRedSlots];
    if ((rc = reduce(st, z, slots))) return rc;
    // sum_k c_k <Z..> = sum_c c_c * (count_c * N - 2 W_c)
    double e = 0.0;
    for (int c = 0; c < z.nclass; ++c) {
        int cnt = 0;
        for (int k = 0; k < nterms; ++k) cnt += z.cls[k] == c;
        e += z.coef[c] * (cnt * slots[0] - 2.0 * slots[1 + c]);
    }
    *out = e;
    return LLG_OK;
}

int llg_expect_diagonal(llg_state* st, const double* diag, int on_device, double* out) {
    if (!st || !diag || !out) return set_error(LLG_EINVAL, "expect_diagonal: NULL argument");
    int rc = ensure_device_buffers(st);
    if (rc) return rc;
    const double* d = diag;
    if (!on_device) {
        if (st->d_diag_size != st->size) {
            LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");
            if (st->d_diag) cudaFree(st->d_diag);
            st->d_diag = nullptr;
            st->d_diag_size = 0;
            cudaError_t e = cudaMalloc(&st->d_diag, st->size * sizeof(double));
            if (e != cudaSuccess) {
                cudaGetLastError();
                return set_error(LLG_ENOMEM, std::string("expect_diagonal: cannot allocate the diagonal: ") +
                                                 cudaGetErrorString(e));
            }
            st->d_diag_size = st->size;
        }
        LLG_CUDA(cudaMemcpyAsync(st->d_diag, diag, st->size * sizeof(double), cudaMemcpyHostToDevice, st->stream),
                 "cudaMemcpyAsync(diagonal)");
        d = st->d_diag;
    } else {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, diag) != cudaSuccess) cudaGetLastError();
        else if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
            return set_error(LLG_EINVAL, "expect_diagonal: on_device set but diag is not device memory");
    }
    DiagObs o;
    std::memset(&o, 0, sizeof(o));
    o.n = st->n;
    o.diag = d;
    double r[2];
    if ((rc = reduce_diag(st, o, r))) return rc;
    *out = r[0];
    return LLG_OK;
}

int llg_renormalize(llg_state* st) {
    double nrm = 0.0;
    int rc = llg_norm2(st, &nrm);
    if (rc) return rc;
    if (!(nrm > 0.0) || !std::isfinite(nrm)) return set_error(LLG_ERUNTIME, "renormalize: state norm vanished");
    return traced(st, LLG_PROF_READOUT, 1, "scale",
                  [&] { return launch_scale(st->P, st->d_psi, st->size, 1.0 / std::sqrt(nrm), st->stream); });
}

void* llg_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocMapped) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void llg_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

int llg_profile(llg_state* st, int on) {
    if (!st) return set_error(LLG_EINVAL, "profile: NULL state");
    st->prof_on = on != 0;
    return LLG_OK;
}

int llg_profile_read(llg_state* st, double* ms, int64_t* launches, int reset) {
    if (!st) return set_error(LLG_EINVAL, "profile_read: NULL state");
    LLG_CUDA(cudaStreamSynchronize(st->stream), "cudaStreamSynchronize");
    for (auto& r : st->prof_recs) {
        float t = 0.0f;
        if (cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) st->prof_ms[r.cls] += t;
        else cudaGetLastError();
        st->prof_n[r.cls] += 1;
        st->ev_pool.push_back(r.a);
        st->ev_pool.push_back(r.b);
    }
    st->prof_recs.clear();
    for (int c = 0; c < LLG_PROF_CLASSES; ++c) {
        if (ms) ms[c] = st->prof_ms[c];
        if (launches) launches[c] = st->prof_n[c];
        if (reset) {
            st->prof_ms[c] = 0.0;
            st->prof_n[c] = 0;
        }
    }
    return LLG_OK;
}

int64_t llg_kernel_launches(void) { return g_launches.load(); }

int llg_fp64_fma_rate(int iters, double* fma_per_s) {
    if (!fma_per_s || iters < 1) return set_error(LLG_EINVAL, "fp64_fma_rate: bad argument");
    LLG_CUDA(fp64_fma_rate(iters, fma_per_s), "fp64_fma_rate");
    return LLG_OK;
}

int llg_get_stream(const llg_state* st, void** out) {
    if (!st || !out) return set_error(LLG_EINVAL, "get_stream: NULL argument");
    *out = (void*)st->stream;
    return LLG_OK;
}

int llg_plan_export(int n, const llg_op* ops, int nops, int tile_qubits, llg_pass_info* passes, int max_passes,
                    int* npasses, llg_exec_op* xops, int max_xops, int* nxops) {
    return llg_plan_export_ex(n, ops, nops, tile_qubits, 0, passes, max_passes, npasses, xops, max_xops, nxops);
}

}  // extern "C"

namespace {
int export_plan(int n, const llg_op* ops, int nops, int tile_qubits, int flags, Plan& plan) {
    if (n < 1 || n > kMaxQubits || nops < 0 || (nops > 0 && !ops))
        return set_error(LLG_EINVAL, "plan_export: bad argument");
    if ((tile_qubits < 1 || tile_qubits > 14) && !(flags & LLG_PLAN_STREAM))
        return set_error(LLG_EINVAL, "plan_export: tile_qubits out of range");
    llg_state tmp;
    tmp.n = n;
    for (int i = 0; i < nops; ++i) {
        int rc = validate_op(&tmp, ops[i], "plan_export");
        if (rc) return rc;
    }
    std::string err;
    if (flags & LLG_PLAN_STREAM) {
        // the per-gate lowering of an IEEE complex128 flush, as one pass over the whole register
        if (flags & ~LLG_PLAN_STREAM) return set_error(LLG_EINVAL, "plan_export: the streaming lowering is exported alone");
        plan.passes.clear();
        plan.ops.clear();
        plan.tables.clear();
        if (!lower_stream_f64(n, ops, nops, plan.ops, err)) return set_error(LLG_EINVAL, err);
        PassDesc pd;
        std::memset(&pd, 0, sizeof(pd));
        pd.local_mask = n >= 64 ? ~0ULL : ((1ULL << n) - 1);
        pd.t = n;
        pd.low = n;
        pd.nops = (int)plan.ops.size();
        plan.passes.push_back(pd);
        return LLG_OK;
    }
    if ((flags & LLG_PLAN_FUSE2) && (flags & (LLG_PLAN_ZYZ | LLG_PLAN_TABLES | LLG_PLAN_REGS)))
        return set_error(LLG_EINVAL, "plan_export: two-qubit blocks are planned alone");
    const int prec = (flags & LLG_PLAN_DF64) ? LLG_DF64 : LLG_F64;
    if (!plan_tiles(n, ops, nops, tile_qubits, prec, plan, err, false, (flags & LLG_PLAN_ZYZ) ? ZYZ_ON : ZYZ_OFF,
                    (flags & LLG_PLAN_TABLES) != 0 && (flags & LLG_PLAN_REGS) == 0, (flags & LLG_PLAN_FUSE2) != 0))
        return set_error(LLG_EINVAL, err);
    if (prec == LLG_DF64) {
        // back from the fp32 (hi, lo) slots of a double-float plan to doubles (hi + lo is exact)
        auto unpack = [](uint64_t& c) {
            float h, l;
            const uint32_t bh = (uint32_t)c, bl = (uint32_t)(c >> 32);
            std::memcpy(&h, &bh, 4);
            std::memcpy(&l, &bl, 4);
            const double v = (double)h + (double)l;
            std::memcpy(&c, &v, 8);
        };
        for (ExecOp& e : plan.ops)
            for (uint64_t& c : e.c) unpack(c);
        for (uint64_t& c : plan.tables) unpack(c);
    }
    if (flags & LLG_PLAN_REGS) {
        if (tile_qubits < 9) return set_error(LLG_EINVAL, "plan_export: register programs need tiles of 9+ qubits");
        to_register_program(plan);
    }
    return LLG_OK;
}
}  // namespace

extern "C" {

int llg_diag_export(int n, int nterms, const int* a, const int* b, const double* coeff, double* out) {
    if (n < 1 || n > 26 || !out) return set_error(LLG_EINVAL, "diag_export: bad argument");
    DiagObsHost h;
    std::string err;
    if (!build_diag_obs(n, nterms, a, b, coeff, h, err)) return set_error(LLG_EINVAL, "diag_export: " + err);
    diag_obs_eval_host(h, out);
    return LLG_OK;
}

int llg_plan_export_tables(int n, const llg_op* ops, int nops, int tile_qubits, int flags, double* tables,
                           int64_t max_doubles, int64_t* ndoubles) {
    if (!ndoubles) return set_error(LLG_EINVAL, "plan_export_tables: NULL count");
    Plan plan;
    int rc = export_plan(n, ops, nops, tile_qubits, flags, plan);
    if (rc) return rc;
    *ndoubles = (int64_t)plan.tables.size();
    if (tables)
        for (int64_t i = 0; i < (int64_t)plan.tables.size() && i < max_doubles; ++i)
            std::memcpy(&tables[i], &plan.tables[(size_t)i], sizeof(double));
    return LLG_OK;
}

int llg_plan_export_ex(int n, const llg_op* ops, int nops, int tile_qubits, int flags, llg_pass_info* passes,
                       int max_passes, int* npasses, llg_exec_op* xops, int max_xops, int* nxops) {
    if (!npasses || !nxops) return set_error(LLG_EINVAL, "plan_export: bad argument");
    Plan plan;
    int rc = export_plan(n, ops, nops, tile_qubits, flags, plan);
    if (rc) return rc;
    *npasses = (int)plan.passes.size();
    *nxops = (int)plan.ops.size();
    if (passes)
        for (int p = 0; p < (int)plan.passes.size() && p < max_passes; ++p) {
            const PassDesc& d = plan.passes[p];
            passes[p].local_mask = d.local_mask;
            passes[p].t = d.t;
            passes[p].low = d.low;
            passes[p].op_begin = d.op_begin;
            passes[p].nops = d.nops;
        }
    if (xops)
        for (int i = 0; i < (int)plan.ops.size() && i < max_xops; ++i) {
            static_assert(sizeof(llg_exec_op) == sizeof(ExecOp), "llg_exec_op mirrors ExecOp");
            std::memcpy(&xops[i], &plan.ops[i], sizeof(ExecOp));
        }
    return LLG_OK;
}

}  // extern "C"
