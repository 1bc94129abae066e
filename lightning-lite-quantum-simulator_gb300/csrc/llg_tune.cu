// llg_tune.cu -- the autotuner for state-vector flushes (include/llgpu.h, "autotuning" section)
// and the process-wide tuning cache shared with the trajectory and batch tuners.
//
// A candidate is (fusion mode, tile width in qubits, CTA threads of the tile kernel).  Each one
// runs a sample of the caller's circuit on a scratch state of the same size and precision, timed
// with CUDA events on the scratch state's stream (one untimed run first, which also pays for the
// planning of a new shape), and the fastest is applied to the caller's state.  Results are cached
// under a hash of (state size, precision, the sample's gate kinds and qubits): rotation angles do
// not change the work, so a circuit family is tuned once per process.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/llgpu.h"
#include "llg_launch.h"

namespace llg {
int set_error(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

namespace {
std::mutex g_tune_mu;
std::map<uint64_t, llg_tune_result> g_tune_cache;
}  // namespace

uint64_t tune_hash(uint64_t h, uint64_t v) {
    // FNV-1a over the 8 bytes of v
    for (int i = 0; i < 8; ++i) {
        h ^= (v >> (8 * i)) & 0xFF;
        h *= 1099511628211ULL;
    }
    return h;
}

uint64_t tune_hash_ops(uint64_t h, const llg_op* ops, int nops) {
    for (int i = 0; i < nops; ++i) {
        h = tune_hash(h, (uint64_t)(uint32_t)ops[i].kind | ((uint64_t)(uint32_t)ops[i].q0 << 32));
        h = tune_hash(h, (uint64_t)(uint32_t)ops[i].q1);
        h = tune_hash(h, ops[i].mask);
    }
    return h;
}

bool tune_cache_get(uint64_t key, llg_tune_result* out) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it == g_tune_cache.end()) return false;
    *out = it->second;
    out->cached = 1;
    return true;
}

void tune_cache_put(uint64_t key, const llg_tune_result& r) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune_cache[key] = r;
}

}  // namespace llg

using namespace llg;

namespace {

struct Candidate {
    int mode, tile, threads;
};

// Mean milliseconds of one application of ops[0..nops) to `tmp` under its current settings:
// one untimed run, then enough timed repetitions for ~2 ms of device time (at most 16).
int time_sample(llg_state* tmp, const llg_op* ops, int nops, cudaStream_t s, cudaEvent_t a, cudaEvent_t b, double* ms) {
    int rc = llg_apply_ops(tmp, ops, nops);
    if (!rc) rc = llg_flush(tmp);
    if (!rc) rc = llg_sync(tmp);
    if (rc) return rc;
    int reps = 1;
    for (int round = 0; round < 2; ++round) {
        cudaError_t e = cudaEventRecord(a, s);
        for (int r = 0; r < reps && !rc && e == cudaSuccess; ++r) {
            rc = llg_apply_ops(tmp, ops, nops);
            if (!rc) rc = llg_flush(tmp);
        }
        if (rc) return rc;
        if (e == cudaSuccess) e = cudaEventRecord(b, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        float t = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
        if (e != cudaSuccess) return cuda_fail(e, "autotune timing");
        *ms = (double)t / reps;
        if (round == 0) {
            if (*ms * reps >= 2.0) break;
            reps = (int)std::min<double>(16.0, std::max(1.0, 2.0 / std::max(*ms, 1e-3)));
        }
    }
    return LLG_OK;
}

}  // namespace

extern "C" {

void llg_tune_cache_clear(void) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune_cache.clear();
}

int llg_autotune(llg_state* st, const llg_op* ops, int nops, int sample_ops, llg_tune_result* out) {
    if (!st || (nops > 0 && !ops) || nops < 0 || sample_ops < 0) return set_error(LLG_EINVAL, "autotune: bad argument");
    int n = 0, P = 0;
    llg_num_qubits(st, &n);
    llg_get_precision(st, &P);
    const int ns = (sample_ops > 0 && sample_ops < nops) ? sample_ops : nops;
    llg_tune_result res;
    std::memset(&res, 0, sizeof(res));
    res.cluster = 1;
    const uint64_t key = tune_hash_ops(tune_hash(tune_hash(1469598103934665603ULL, 0x5741), (uint64_t)n << 8 | (uint64_t)P),
                                       ops, ns);
    if (!tune_cache_get(key, &res)) {
        // candidates: per-gate kernels, then tile passes of 8..max qubits with 256 or 512 threads
        std::vector<Candidate> cands;
        cands.push_back({LLG_FUSE_NONE, 0, 0});
        const int tmax = std::min(n, tile_max_qubits(P));
        // 1024 threads only pays where few tiles leave SMs idle (small registers)
        const bool small = n <= 16;
        for (int t = std::max(5, std::min(8, tmax)); t <= tmax; ++t)
            for (int th : {256, 512, 1024})
                if (th == 256 || (th == 512 && t >= 10) || (th == 1024 && small && t >= 11)) cands.push_back({LLG_FUSE_TILE, t, th});
        if (P == LLG_F32)  // register-tiled passes (2^(t-4) threads per CTA)
            for (int t = 9; t <= std::min(n, 13); ++t) cands.push_back({LLG_FUSE_REG, t, 0});
        llg_state* tmp = nullptr;
        int rc = llg_create(n, P, &tmp);
        if (rc) return set_error(rc, "autotune: cannot create the scratch state (a second state of the same size)");
        void* sv = nullptr;
        llg_get_stream(tmp, &sv);
        cudaStream_t s = static_cast<cudaStream_t>(sv);
        cudaEvent_t a = nullptr, b = nullptr;
        cudaError_t e = cudaEventCreate(&a);
        if (e == cudaSuccess) e = cudaEventCreate(&b);
        if (e != cudaSuccess) rc = cuda_fail(e, "autotune events");
        double best = 1e300;
        // the default configuration first (the reference point reported as default_ms)
        if (!rc) rc = llg_set_fusion(tmp, LLG_FUSE_TILE, 0);
        if (!rc) rc = llg_set_tile_threads(tmp, 0);
        if (!rc) rc = time_sample(tmp, ops, ns, s, a, b, &res.default_ms);
        for (const Candidate& c : cands) {
            if (rc) break;
            rc = llg_set_fusion(tmp, c.mode, c.tile);
            if (!rc) rc = llg_set_tile_threads(tmp, c.threads);
            double ms = 0.0;
            if (!rc) rc = time_sample(tmp, ops, ns, s, a, b, &ms);
            if (rc) break;
            ++res.candidates;
            if (ms < best) {
                best = ms;
                res.fuse_mode = c.mode;
                res.tile_qubits = c.tile;
                res.cta_threads = c.threads;
                res.best_ms = ms;
            }
        }
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
        llg_destroy(tmp);
        if (rc) return rc;
        tune_cache_put(key, res);
    }
    int rc = llg_set_fusion(st, res.fuse_mode, res.tile_qubits);
    if (!rc) rc = llg_set_tile_threads(st, res.cta_threads);
    if (rc) return rc;
    if (out) *out = res;
    return LLG_OK;
}

}  // extern "C"
