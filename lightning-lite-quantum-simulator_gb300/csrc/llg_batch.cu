// llg_batch.cu -- many circuits of uneven qubit counts in one persistent launch (include/llgpu.h,
// "mixed-size batches" section).
//
// Every circuit is planned into shared-memory tile passes (llg_plan.cpp) and its state placed in
// one HBM arena.  The work items (circuit c, pass j, tile k) form one queue ordered by pass round
// j, then circuit, then tile, and persistent CTAs take items with an atomic counter.  A tile of
// pass j may only start once every tile of passes 0..j-1 of its circuit has finished: each
// circuit keeps a completion counter, bumped after a tile's stores are fenced.  Every item a CTA
// waits for was taken from the queue earlier by a running CTA that does not wait on anything
// later, so the waits always end; they are bounded all the same (spin_limit polls), and a wait
// that runs out sets an error flag the host reports as LLG_ETIMEOUT instead of hanging.
// Tiles are read with L1-bypassing loads (other SMs wrote them).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/llgpu.h"
#include "llg_common.cuh"
#include "llg_internal.h"
#include "llg_launch.h"
#include "llg_tile.cuh"

namespace llg {
int set_error(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
}  // namespace llg

using namespace llg;

namespace {

constexpr int kBatchThreads = 512;  // largest CTA; the default and the tuner's other choice is 256
constexpr int kBatchOpChunk = 32;   // op records staged per shared-memory chunk
constexpr long long kDefaultSpinLimit = 1LL << 24;  // ~1 s of 64 ns polls

struct CircDesc {
    uint64_t offset;  // first amplitude in the arena
    int32_t n;
    int32_t t;
    int32_t pass_begin;
    int32_t npasses;
};

struct Item {
    int32_t c, j, k;
    uint32_t need;  // completed tiles of circuit c required before this tile starts
};

template <class P>
__global__ void __launch_bounds__(kBatchThreads) k_batch(typename P::S* __restrict__ arena, const CircDesc* __restrict__ circs,
                                                         const PassDesc* __restrict__ passes, const ExecOp* __restrict__ ops,
                                                         const Item* __restrict__ items, long long nitems,
                                                         unsigned long long* __restrict__ next, unsigned* __restrict__ completed,
                                                         int* __restrict__ err, long long spin_limit,
                                                         const uint64_t* __restrict__ tables) {
    using S = typename P::S;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ long long s_item;
    __shared__ int s_ok;
    for (;;) {
        if (threadIdx.x == 0) s_item = (long long)atomicAdd(next, 1ULL);
        __syncthreads();
        const long long it = s_item;
        if (it >= nitems) break;
        const Item w = items[it];
        const CircDesc cd = circs[w.c];
        const PassDesc pd = passes[cd.pass_begin + w.j];
        if (threadIdx.x == 0) {
            long long polls = 0;
            int ok = 1;
            while (*(volatile unsigned*)&completed[w.c] < w.need) {
                if (++polls > spin_limit) {
                    atomicExch(err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
            __threadfence();
            s_ok = ok;
        }
        __syncthreads();
        if (s_ok) {
            const int t = pd.t, low = pd.low;
            const uint32_t tsize = 1u << t, nhi = 1u << (t - low);
            S* tile = reinterpret_cast<S*>(smem_raw);
            uint64_t* hi_off = reinterpret_cast<uint64_t*>(smem_raw + (size_t)tsize * sizeof(S));
            S* psi = arena + cd.offset;
            const uint64_t base = insert0_mask((uint64_t)w.k, pd.local_mask);
            for (uint32_t h = threadIdx.x; h < nhi; h += blockDim.x) {
                uint64_t off = 0;
                for (int j = 0; j < t - low; ++j)
                    if ((h >> j) & 1) off |= 1ULL << pd.hi_pos[j];
                hi_off[h] = off;
            }
            __syncthreads();
            const uint32_t lowmask = (1u << low) - 1;
            for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) tile[l] = __ldcg(&psi[base | hi_off[l >> low] | (l & lowmask)]);
            __syncthreads();
            // op records staged through shared memory in chunks (as in the single-state tile pass)
            __shared__ __align__(16) ExecOp sops[kBatchOpChunk];
            constexpr int kWords = (int)(sizeof(ExecOp) / 16);
            for (int k = 0; k < pd.nops; ++k) {
                if (k % kBatchOpChunk == 0) {
                    const int cnt = min(kBatchOpChunk, pd.nops - k);
                    const uint4* src = reinterpret_cast<const uint4*>(ops + pd.op_begin + k);
                    for (int q = threadIdx.x; q < cnt * kWords; q += blockDim.x) reinterpret_cast<uint4*>(sops)[q] = src[q];
                    __syncthreads();
                }
                tile_apply<P>(tile, tsize, base, sops[k % kBatchOpChunk], nullptr, tables);
                __syncthreads();
            }
            for (uint32_t l = threadIdx.x; l < tsize; l += blockDim.x) psi[base | hi_off[l >> low] | (l & lowmask)] = tile[l];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(&completed[w.c], 1u);
        }
    }
}

template <class P>
__global__ void k_batch_init(typename P::S* arena, const CircDesc* circs, int count) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= count) return;
    typename P::C one;
    one.re = P::r_from_float(1.0f);
    one.im = P::zero();
    arena[circs[c].offset] = P::store(one);
}

// per-circuit <a|b> and norms: grid (kOvBlocks, count); partial[c][blk][4]
constexpr int kOvBlocks = 32;

template <class PA, class PB>
__global__ void __launch_bounds__(256) k_overlap(const typename PA::S* __restrict__ a, const typename PB::S* __restrict__ b,
                                                 const CircDesc* __restrict__ ca, const CircDesc* __restrict__ cb,
                                                 double* __restrict__ part) {
    __shared__ double sh[4][8];
    const int c = blockIdx.y;
    const uint64_t size = 1ULL << ca[c].n;
    const typename PA::S* pa = a + ca[c].offset;
    const typename PB::S* pb = b + cb[c].offset;
    double re = 0, im = 0, na = 0, nb = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < size; i += (uint64_t)gridDim.x * blockDim.x) {
        const double2 x = PA::to_f64(PA::load(pa[i]));
        const double2 y = PB::to_f64(PB::load(pb[i]));
        re = fma(x.x, y.x, fma(x.y, y.y, re));
        im = fma(x.x, y.y, fma(-x.y, y.x, im));
        na = fma(x.x, x.x, fma(x.y, x.y, na));
        nb = fma(y.x, y.x, fma(y.y, y.y, nb));
    }
    double v[4] = {re, im, na, nb};
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        double s = v[q];
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (lane == 0) sh[q][warp] = s;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[threadIdx.x][w];
        part[((size_t)c * gridDim.x + blockIdx.x) * 4 + threadIdx.x] = s;
    }
}

__global__ void k_overlap_finish(const double* __restrict__ part, int blocks, int count, double* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= count) return;
    double v[4] = {0, 0, 0, 0};
    for (int b = 0; b < blocks; ++b)
        for (int q = 0; q < 4; ++q) v[q] += part[((size_t)c * blocks + b) * 4 + q];
    out[3 * c + 0] = (v[0] * v[0] + v[1] * v[1]) / (v[2] * v[3]);  // fidelity
    out[3 * c + 1] = v[2];                                          // |a|^2
    out[3 * c + 2] = v[3];                                          // |b|^2
}

template <class P>
size_t batch_smem(int t) {
    return ((size_t)1 << t) * sizeof(typename P::S) + ((size_t)1 << t) * sizeof(uint64_t) / 16 + 64;
}

}  // namespace

struct llg_batch {
    int P = LLG_DF64;
    int count = 0;
    int tile = 12;
    std::vector<CircDesc> circs;
    std::vector<PassDesc> passes;
    std::vector<ExecOp> ops;
    std::vector<uint64_t> tables;  // phase tables of every circuit's plan, (re, im) slots per entry
    std::vector<Item> items;
    uint64_t total_amps = 0;
    cudaStream_t stream = nullptr;
    void* d_arena = nullptr;
    CircDesc* d_circs = nullptr;
    PassDesc* d_passes = nullptr;
    ExecOp* d_ops = nullptr;
    uint64_t* d_tables = nullptr;
    Item* d_items = nullptr;
    unsigned long long* d_next = nullptr;
    unsigned* d_completed = nullptr;
    int* d_err = nullptr;
    int grid = 0;
    int threads = 256;
    size_t smem = 0;
    // the run captured as a CUDA graph (state reset + persistent kernel), re-captured when the
    // spin limit changes
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long graph_spin = -1;
};

namespace {

// Grid and shared memory of the persistent kernel (once per batch, outside any capture).
template <class P>
int setup_batch(llg_batch* b) {
    if (b->grid) return LLG_OK;
    b->smem = batch_smem<P>(b->tile);
    cudaError_t e = cudaFuncSetAttribute(k_batch<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem);
    if (e != cudaSuccess) return cuda_fail(e, "batch attributes");
    int per_sm = 1, dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<P>, b->threads, b->smem)))
        return cuda_fail(e, "batch occupancy");
    b->grid = std::max(1, sms * std::max(per_sm, 1));
    return LLG_OK;
}

// Stream work of one run: every state to |0..0>, queue and counters reset, the persistent kernel.
template <class P>
cudaError_t enqueue_batch(llg_batch* b, long long spin_limit) {
    cudaStream_t s = b->stream;
    cudaError_t e;
    if ((e = cudaMemsetAsync(b->d_arena, 0, b->total_amps * sizeof(typename P::S), s))) return e;
    k_batch_init<P><<<(b->count + 255) / 256, 256, 0, s>>>(static_cast<typename P::S*>(b->d_arena), b->d_circs, b->count);
    if ((e = cudaGetLastError())) return e;
    if ((e = cudaMemsetAsync(b->d_next, 0, sizeof(unsigned long long), s))) return e;
    if ((e = cudaMemsetAsync(b->d_completed, 0, b->count * sizeof(unsigned), s))) return e;
    if ((e = cudaMemsetAsync(b->d_err, 0, sizeof(int), s))) return e;
    k_batch<P><<<b->grid, b->threads, b->smem, s>>>(static_cast<typename P::S*>(b->d_arena), b->d_circs, b->d_passes,
                                                       b->d_ops, b->d_items, (long long)b->items.size(), b->d_next,
                                                       b->d_completed, b->d_err, spin_limit, b->d_tables);
    return cudaGetLastError();
}

void drop_graph(llg_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graph_spin = -1;
}

template <class P>
int launch_batch(llg_batch* b, long long spin_limit) {
    int rc = setup_batch<P>(b);
    if (rc) return rc;
    cudaError_t e = cudaSuccess;
    if (!b->exec || b->graph_spin != spin_limit) {
        drop_graph(b);
        e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const cudaError_t le = enqueue_batch<P>(b, spin_limit);
            e = cudaStreamEndCapture(b->stream, &b->graph);
            if (le != cudaSuccess) e = le;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
        if (e != cudaSuccess) {
            drop_graph(b);
            return cuda_fail(e, "batch graph capture");
        }
        b->graph_spin = spin_limit;
    }
    if ((e = cudaGraphLaunch(b->exec, b->stream))) return cuda_fail(e, "batch launch");
    return LLG_OK;
}

}  // namespace

extern "C" {

static int batch_build(int count, const int* n_qubits, const llg_op* ops, const int64_t* op_offsets, int precision,
                       int tile, int threads, llg_batch** out) {
    llg_batch* b = new llg_batch();
    b->threads = threads;
    b->P = precision;
    b->count = count;
    b->tile = tile;
    std::vector<std::vector<std::pair<int, int>>> rounds;  // per pass round j: (circuit, tiles)
    for (int c = 0; c < count; ++c) {
        const int n = n_qubits[c];
        const int64_t o0 = op_offsets[c], o1 = op_offsets[c + 1];
        if (n < 1 || n > 30 || o1 < o0) {
            delete b;
            return set_error(LLG_EINVAL, "batch_create: circuit " + std::to_string(c) + " has a bad size");
        }
        for (int64_t i = o0; i < o1; ++i) {
            const llg_op& o = ops[i];
            bool ok = o.q0 >= 0 && o.q0 < n && o.kind >= 0 && o.kind <= LLG_OP_U2;
            if (o.kind == LLG_OP_CNOT || o.kind == LLG_OP_CZ) ok = ok && o.q1 >= 0 && o.q1 < n && o.q1 != o.q0;
            if (o.kind == LLG_OP_MCZ) ok = o.mask != 0 && (o.mask >> n) == 0;
            if ((o.kind == LLG_OP_RX || o.kind == LLG_OP_RY || o.kind == LLG_OP_RZ) && !std::isfinite(o.theta)) ok = false;
            if (!ok) {
                delete b;
                return set_error(LLG_EINVAL, "batch_create: circuit " + std::to_string(c) + " op " + std::to_string(i - o0));
            }
        }
        Plan plan;
        std::string err;
        // 16-byte precisions gather diagonal factors into phase tables (one table buffer for the
        // batch; each circuit's EX_PTAB offsets are shifted to its part of it)
        if (!plan_tiles(n, ops + o0, (int)(o1 - o0), tile, precision, plan, err, false, ZYZ_DEFAULT,
                        precision != LLG_F32)) {
            delete b;
            return set_error(LLG_EINVAL, "batch_create: " + err);
        }
        CircDesc cd;
        cd.offset = b->total_amps;
        cd.n = n;
        cd.t = std::min(n, tile);
        cd.pass_begin = (int)b->passes.size();
        cd.npasses = (int)plan.passes.size();
        for (PassDesc pd : plan.passes) {
            pd.op_begin += (int)b->ops.size();
            b->passes.push_back(pd);
        }
        const uint64_t table_base = b->tables.size() / 2;  // entries of (re, im) slots
        for (ExecOp& x : plan.ops)
            if (x.kind == EX_PTAB) x.mask += table_base;
        b->tables.insert(b->tables.end(), plan.tables.begin(), plan.tables.end());
        b->ops.insert(b->ops.end(), plan.ops.begin(), plan.ops.end());
        b->circs.push_back(cd);
        b->total_amps += 1ULL << n;
        const int tiles = 1 << (n - cd.t);
        if ((int)rounds.size() < cd.npasses) rounds.resize(cd.npasses);
        for (int j = 0; j < cd.npasses; ++j) rounds[j].push_back({c, tiles});
    }
    for (size_t j = 0; j < rounds.size(); ++j)
        for (auto& ct : rounds[j])
            for (int k = 0; k < ct.second; ++k) b->items.push_back({ct.first, (int)j, k, (uint32_t)(j * ct.second)});
    const size_t eb = elem_bytes(precision);
    int rc = LLG_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    auto alloc = [&](void** p, size_t bytes, const char* what) {
        if (rc) return;
        cudaError_t ee = cudaMalloc(p, std::max<size_t>(bytes, 16));
        if (ee != cudaSuccess) {
            cudaGetLastError();
            rc = set_error(LLG_ENOMEM, std::string("batch_create: cannot allocate ") + what);
        }
    };
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamCreate");
    alloc(&b->d_arena, b->total_amps * eb, "the state arena");
    alloc((void**)&b->d_circs, b->circs.size() * sizeof(CircDesc), "circuit table");
    alloc((void**)&b->d_passes, b->passes.size() * sizeof(PassDesc), "pass table");
    alloc((void**)&b->d_ops, b->ops.size() * sizeof(ExecOp), "op table");
    if (!b->tables.empty()) alloc((void**)&b->d_tables, b->tables.size() * sizeof(uint64_t), "phase tables");
    alloc((void**)&b->d_items, b->items.size() * sizeof(Item), "work queue");
    alloc((void**)&b->d_next, sizeof(unsigned long long), "queue head");
    alloc((void**)&b->d_completed, count * sizeof(unsigned), "counters");
    alloc((void**)&b->d_err, sizeof(int), "error flag");
    auto up = [&](void* dst, const void* src, size_t bytes) {
        if (rc || bytes == 0) return;
        if (cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) rc = set_error(LLG_ECUDA, "batch_create: upload");
    };
    up(b->d_circs, b->circs.data(), b->circs.size() * sizeof(CircDesc));
    up(b->d_passes, b->passes.data(), b->passes.size() * sizeof(PassDesc));
    up(b->d_ops, b->ops.data(), b->ops.size() * sizeof(ExecOp));
    if (b->d_tables) up(b->d_tables, b->tables.data(), b->tables.size() * sizeof(uint64_t));
    up(b->d_items, b->items.data(), b->items.size() * sizeof(Item));
    if (rc) {
        llg_batch_destroy(b);
        return rc;
    }
    *out = b;
    return LLG_OK;
}

int llg_batch_create(int count, const int* n_qubits, const llg_op* ops, const int64_t* op_offsets, int precision,
                     int tile_qubits, llg_batch** out) {
    if (!out) return set_error(LLG_EINVAL, "batch_create: out is NULL");
    *out = nullptr;
    if (count < 1 || !n_qubits || !op_offsets || (op_offsets[count] > 0 && !ops))
        return set_error(LLG_EINVAL, "batch_create: bad arguments");
    if (precision != LLG_F64 && precision != LLG_DF64 && precision != LLG_F32)
        return set_error(LLG_EINVAL, "batch_create: unknown precision");
    if (tile_qubits < LLG_TUNE_AUTO) return set_error(LLG_EINVAL, "batch_create: tile_qubits must be -1, 0 or positive");
    const int tmax = tile_max_qubits(precision);
    if (tile_qubits != LLG_TUNE_AUTO) {
        const int tile = tile_qubits > 0 ? std::min(tile_qubits, tmax) : (precision == LLG_F32 ? 13 : 12);
        if (tile < 2) return set_error(LLG_EINVAL, "batch_create: tile_qubits too small");
        return batch_build(count, n_qubits, ops, op_offsets, precision, tile, 256, out);
    }
    llg_tune_result res;
    int rc = llg_batch_autotune(count, n_qubits, ops, op_offsets, precision, &res);
    if (rc) return rc;
    return batch_build(count, n_qubits, ops, op_offsets, precision, res.tile_qubits, res.cta_threads, out);
}

int llg_batch_autotune(int count, const int* n_qubits, const llg_op* ops, const int64_t* op_offsets, int precision,
                       llg_tune_result* out) {
    if (count < 1 || !n_qubits || !op_offsets || (op_offsets[count] > 0 && !ops) || !out)
        return set_error(LLG_EINVAL, "batch_autotune: bad arguments");
    if (precision != LLG_F64 && precision != LLG_DF64 && precision != LLG_F32)
        return set_error(LLG_EINVAL, "batch_autotune: unknown precision");
    uint64_t key = tune_hash(tune_hash(1469598103934665603ULL, 0x424154), (uint64_t)precision);
    int nmax = 1;
    for (int c = 0; c < count; ++c) {
        key = tune_hash(key, (uint64_t)n_qubits[c]);
        nmax = std::max(nmax, n_qubits[c]);
    }
    key = tune_hash_ops(key, ops, (int)op_offsets[count]);
    llg_tune_result res;
    std::memset(&res, 0, sizeof(res));
    if (tune_cache_get(key, &res)) {
        *out = res;
        return LLG_OK;
    }
    res.fuse_mode = LLG_FUSE_TILE;
    res.cluster = 1;
    res.cta_threads = 256;
    const int tdef = precision == LLG_F32 ? 13 : 12;
    const int tmax = std::min(tile_max_qubits(precision), std::max(nmax, 8));
    double best = 1e300;
    cudaEvent_t ea = nullptr, eb = nullptr;
    cudaError_t e = cudaEventCreate(&ea);
    if (e == cudaSuccess) e = cudaEventCreate(&eb);
    if (e != cudaSuccess) return cuda_fail(e, "batch autotune events");
    int rc = LLG_OK;
    for (int t = std::min(8, tmax); t <= tmax && !rc; ++t)
        for (int th : {256, 512}) {
            if (rc) break;
            llg_batch* b = nullptr;
            rc = batch_build(count, n_qubits, ops, op_offsets, precision, t, th, &b);
            if (rc) break;
            rc = llg_batch_run(b, 0);  // untimed (captures the graph)
            if (!rc) {
                e = cudaEventRecord(ea, b->stream);
                if (e == cudaSuccess) {
                    rc = llg_batch_run(b, 0);
                    if (!rc) e = cudaEventRecord(eb, b->stream);
                }
                if (!rc && e == cudaSuccess) e = cudaEventSynchronize(eb);
                float ms = 0.f;
                if (!rc && e == cudaSuccess) e = cudaEventElapsedTime(&ms, ea, eb);
                if (!rc && e != cudaSuccess) rc = cuda_fail(e, "batch autotune timing");
                if (!rc) {
                    ++res.candidates;
                    if (t == tdef && th == 256) res.default_ms = ms;
                    if (ms < best) {
                        best = ms;
                        res.best_ms = ms;
                        res.tile_qubits = t;
                        res.cta_threads = th;
                    }
                }
            }
            llg_batch_destroy(b);
        }
    cudaEventDestroy(ea);
    cudaEventDestroy(eb);
    if (rc) return rc;
    tune_cache_put(key, res);
    *out = res;
    return LLG_OK;
}

int llg_batch_config(const llg_batch* b, int* tile_qubits, int* grid, int* cta_threads) {
    if (!b) return set_error(LLG_EINVAL, "batch_config: NULL handle");
    if (tile_qubits) *tile_qubits = b->tile;
    if (grid) *grid = b->grid;
    if (cta_threads) *cta_threads = b->threads;
    return LLG_OK;
}

int llg_batch_destroy(llg_batch* b) {
    if (!b) return LLG_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graph(b);
    void* ptrs[] = {b->d_arena, b->d_circs, b->d_passes, b->d_ops, b->d_tables, b->d_items, b->d_next, b->d_completed,
                    b->d_err};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return LLG_OK;
}

int llg_batch_info(const llg_batch* b, int64_t* work_items, int64_t* total_amps, int* total_passes) {
    if (!b) return set_error(LLG_EINVAL, "batch_info: NULL handle");
    if (work_items) *work_items = (int64_t)b->items.size();
    if (total_amps) *total_amps = (int64_t)b->total_amps;
    if (total_passes) *total_passes = (int)b->passes.size();
    return LLG_OK;
}

int llg_batch_run(llg_batch* b, int64_t spin_limit) {
    if (!b) return set_error(LLG_EINVAL, "batch_run: NULL handle");
    const long long lim = spin_limit > 0 ? spin_limit : kDefaultSpinLimit;
    int rc;
    switch (b->P) {
        case LLG_F64: rc = launch_batch<PolF64>(b, lim); break;
        case LLG_F32: rc = launch_batch<PolF32>(b, lim); break;
        default: rc = launch_batch<PolDF64>(b, lim); break;
    }
    if (rc) return rc;
    int err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail(e, "batch kernel");
    if (err) return set_error(LLG_ETIMEOUT, "batch_run: a tile waited past its limit for its circuit's previous pass");
    return LLG_OK;
}

// Test hook: make work item `item` wait for a completion count no tile will reach, so that its
// bounded wait runs out and the run reports LLG_ETIMEOUT (the kernel returns; nothing hangs).
int llg_batch_debug_block_item(llg_batch* b, int64_t item) {
    if (!b || item < 0 || item >= (int64_t)b->items.size()) return set_error(LLG_EINVAL, "batch_debug_block_item: bad item");
    Item w = b->items[item];
    w.need = 0xFFFFFFFFu;
    cudaError_t e = cudaMemcpy(b->d_items + item, &w, sizeof(Item), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "batch_debug_block_item");
    return LLG_OK;
}

int llg_batch_copy_state(llg_batch* b, int index, double* out) {
    if (!b || !out || index < 0 || index >= b->count) return set_error(LLG_EINVAL, "batch_copy_state: bad argument");
    const CircDesc& cd = b->circs[index];
    const uint64_t size = 1ULL << cd.n;
    const size_t eb = elem_bytes(b->P);
    double* d_tmp = nullptr;
    cudaError_t e = cudaMalloc(&d_tmp, size * 16);
    if (e != cudaSuccess) return cuda_fail(e, "batch_copy_state");
    e = launch_to_f64(b->P, (const char*)b->d_arena + cd.offset * eb, d_tmp, size, b->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_tmp, size * 16, cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    cudaFree(d_tmp);
    if (e != cudaSuccess) return cuda_fail(e, "batch_copy_state");
    return LLG_OK;
}

// fidelity |<a_i|b_i>|^2 / (|a_i|^2 |b_i|^2) per circuit (FP64 accumulation), and both norms:
// out[3 * i + {0, 1, 2}].  The two batches must hold the same circuit sizes.
int llg_batch_fidelity(llg_batch* a, llg_batch* b, double* out) {
    if (!a || !b || !out || a->count != b->count) return set_error(LLG_EINVAL, "batch_fidelity: bad arguments");
    for (int c = 0; c < a->count; ++c)
        if (a->circs[c].n != b->circs[c].n) return set_error(LLG_EINVAL, "batch_fidelity: circuit sizes differ");
    double *d_part = nullptr, *d_out = nullptr;
    cudaError_t e = cudaMalloc(&d_part, (size_t)a->count * kOvBlocks * 4 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_out, (size_t)a->count * 3 * sizeof(double));
    if (e != cudaSuccess) {
        cudaFree(d_part);
        return cuda_fail(e, "batch_fidelity");
    }
    cudaStreamSynchronize(b->stream);
    const dim3 grid(kOvBlocks, a->count);
    auto go = [&](auto pa, auto pb) {
        using PA = decltype(pa);
        using PB = decltype(pb);
        k_overlap<PA, PB><<<grid, 256, 0, a->stream>>>(static_cast<const typename PA::S*>(a->d_arena),
                                                        static_cast<const typename PB::S*>(b->d_arena), a->d_circs, b->d_circs,
                                                        d_part);
    };
    auto dispatch_b = [&](auto pa) {
        switch (b->P) {
            case LLG_F64: go(pa, PolF64{}); break;
            case LLG_F32: go(pa, PolF32{}); break;
            default: go(pa, PolDF64{}); break;
        }
    };
    switch (a->P) {
        case LLG_F64: dispatch_b(PolF64{}); break;
        case LLG_F32: dispatch_b(PolF32{}); break;
        default: dispatch_b(PolDF64{}); break;
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_overlap_finish<<<(a->count + 127) / 128, 128, 0, a->stream>>>(d_part, kOvBlocks, a->count, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, (size_t)a->count * 3 * sizeof(double), cudaMemcpyDeviceToHost, a->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(a->stream);
    cudaFree(d_part);
    cudaFree(d_out);
    if (e != cudaSuccess) return cuda_fail(e, "batch_fidelity");
    return LLG_OK;
}

int llg_batch_stream(const llg_batch* b, void** out) {
    if (!b || !out) return set_error(LLG_EINVAL, "batch_stream: NULL argument");
    *out = (void*)b->stream;
    return LLG_OK;
}

}  // extern "C"
