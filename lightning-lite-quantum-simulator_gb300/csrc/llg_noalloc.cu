// llg_noalloc.cu -- llg_expect_zz_noalloc: the diagonal-observable reduction (sum_k c_k <Z Z>,
// the same result as llg_expect_zz) for callers that cannot allocate GPU memory.
//
// Who needs it: callers whose device memory belongs to another allocator -- a framework that
// reserves most of the GPU up front (a caching-allocator pool, a preallocating runtime) and so
// leaves no room for, or forbids, a library's own cudaMalloc -- and callers in latency-critical
// loops, where cudaMalloc/cudaFree would synchronise the device.  Such a caller owns the state
// (device memory it allocated itself) and the result slot; this entry point allocates nothing.
//
// How: the per-block partial sums that llg_expect_zz keeps in a per-state cudaMalloc buffer go
// instead to a file-scope device array, kScratchRows x kScratchSlots doubles (40 KiB).  Every GPU
// that loads this library holds that array until the process exits.  Host code cannot use the
// array's name as a device address (on the host it is only a stand-in), so the address is
// resolved once per device with cudaGetSymbolAddress and passed to the kernels.
//
// Contract:
//  * The first call on a device resolves that device's scratch address (cudaGetSymbolAddress);
//    make that first call before any stream capture on that device.  The address is cached per
//    device for the life of the process: it stays valid while the device's primary context lives,
//    so a caller that resets the device (cudaDeviceReset) must not use this entry point afterwards.
//  * d_amps and d_out must be memory of the current device (or managed memory); device memory of
//    another GPU is rejected with LLG_EINVAL.
//  * The call reports a CUDA error left pending by earlier work (cudaPeekAtLastError) as
//    LLG_ECUDA before launching anything, and does not clear it.
//  * Every call shares the one scratch array and it keeps the last call's contents.  Each call
//    writes every partial row it later reads, so nothing has to start at zero; but calls whose
//    kernels overlap on the GPU (different streams, or different host threads) race on the array.
//    Order such calls on one stream or serialise them.
//  * Limits: n_qubits in [1, 34]; at most 64 terms with at most 4 distinct coefficients; the
//    reduction grid is capped at kScratchRows blocks (the scratch size), whatever the state size.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/llgpu.h"
#include "llg_common.cuh"
#include "llg_launch.h"

namespace llg {
int set_error(int code, const std::string& msg);  // llg_engine.cu
}

using namespace llg;

namespace {

constexpr int kScratchRows = 1024;
constexpr int kScratchSlots = kRedSlots;  // [sum |a|^2, W_0 .. W_3]
constexpr int kThreadsNA = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kScratchRows * kScratchSlots];

std::mutex g_mu;
double* g_scratch[kMaxDevices] = {};

__device__ __forceinline__ double block_sum_na(double v, double* sh) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += sh[w];
    return r;
}

// Same per-thread accumulation as the engine's k_reduce_z; partial rows go to `partials`, the
// scratch array's device address.
template <class P>
__global__ void __launch_bounds__(kThreadsNA) k_reduce_z_scratch(const typename P::S* __restrict__ psi, uint64_t size,
                                                                 ZTerms z, double* __restrict__ partials) {
    __shared__ double sh[kThreadsNA / 32];
    typename P::Acc acc[kScratchSlots];
#pragma unroll
    for (int s = 0; s < kScratchSlots; ++s) acc[s] = P::acc_zero();
    const uint64_t step = (uint64_t)gridDim.x * kThreadsNA;
    for (uint64_t i = (uint64_t)blockIdx.x * kThreadsNA + threadIdx.x; i < size; i += step) {
        const auto a = P::load(psi[i]);
        acc[0] = P::acc_norm(acc[0], a);
        if (z.nterms > 0) {
            int cnt[kMaxZClasses] = {0, 0, 0, 0};
            for (int k = 0; k < z.nterms; ++k) {
                int par = (int)((i >> z.a[k]) & 1);
                if (z.b[k] >= 0) par ^= (int)((i >> z.b[k]) & 1);
                cnt[z.cls[k]] += par;
            }
#pragma unroll
            for (int c = 0; c < kMaxZClasses; ++c)
                if (c < z.nclass && cnt[c]) acc[1 + c] = P::acc_norm_w(acc[1 + c], a, (float)cnt[c]);
        }
    }
#pragma unroll
    for (int s = 0; s < kScratchSlots; ++s) {
        const double v = block_sum_na(P::acc_to_double(acc[s]), sh);
        if (threadIdx.x == 0) partials[(size_t)blockIdx.x * kScratchSlots + s] = v;
    }
}

// One warp: slot sums in a fixed order (deterministic), then the expectation on the device.
__global__ void k_finish_expect(const double* __restrict__ partials, int nblocks, ZTerms z, double* __restrict__ out) {
    __shared__ double slot[kScratchSlots];
    const int s = threadIdx.x;
    if (s < kScratchSlots) {
        double r = 0.0;
        for (int b = 0; b < nblocks; ++b) r += partials[(size_t)b * kScratchSlots + s];
        slot[s] = r;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double e = 0.0;
        for (int c = 0; c < z.nclass; ++c) {
            int cnt = 0;
            for (int k = 0; k < z.nterms; ++k) cnt += z.cls[k] == c;
            e += z.coef[c] * (cnt * slot[0] - 2.0 * slot[1 + c]);
        }
        out[0] = e;
        out[1] = slot[0];
    }
}

// Resolve this device's scratch address once (the device must be current).
int scratch_address(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(LLG_ECUDA, std::string("expect_zz_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return set_error(LLG_ERUNTIME, "expect_zz_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess || !p)
            return set_error(LLG_ECUDA, std::string("expect_zz_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_scratch[dev] = static_cast<double*>(p);
    }
    *out = g_scratch[dev];
    return LLG_OK;
}

// Device memory of the current device, or managed memory.
bool device_reachable(const void* p, int dev) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // the error this query itself raised (an unregistered host pointer)
        return false;
    }
    if (at.type == cudaMemoryTypeManaged) return true;
    return at.type == cudaMemoryTypeDevice && at.device == dev;
}

template <class P>
int launch(const void* d_amps, int n, const ZTerms& z, double* scratch, double* d_out, cudaStream_t s) {
    const uint64_t size = 1ULL << n;
    int sms = 1, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t want = (size + (uint64_t)kThreadsNA * 4 - 1) / ((uint64_t)kThreadsNA * 4);
    const uint64_t cap = (uint64_t)sms * 16 < (uint64_t)kScratchRows ? (uint64_t)sms * 16 : (uint64_t)kScratchRows;
    const unsigned grid = (unsigned)(want < 1 ? 1 : (want > cap ? cap : want));
    k_reduce_z_scratch<P><<<grid, kThreadsNA, 0, s>>>(static_cast<const typename P::S*>(d_amps), size, z, scratch);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_finish_expect<<<1, 32, 0, s>>>(scratch, (int)grid, z, d_out);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return set_error(LLG_ECUDA, std::string("expect_zz_noalloc: launch: ") + cudaGetErrorString(e));
    return LLG_OK;
}

}  // namespace

extern "C" int llg_expect_zz_noalloc(const void* d_amps, int n_qubits, int precision, int nterms, const int* a,
                                     const int* b, const double* coeff, double* d_out, void* stream) {
    if (!d_amps || !d_out || (nterms > 0 && (!a || !b || !coeff)))
        return set_error(LLG_EINVAL, "expect_zz_noalloc: NULL argument");
    if (n_qubits < 1 || n_qubits > 34)
        return set_error(LLG_EINVAL, "expect_zz_noalloc: n_qubits must be in [1, 34], got " + std::to_string(n_qubits));
    if (precision != LLG_F64 && precision != LLG_DF64 && precision != LLG_F32)
        return set_error(LLG_EINVAL, "expect_zz_noalloc: unknown precision");
    if (nterms < 0 || nterms > kMaxZTerms)
        return set_error(LLG_EINVAL, "expect_zz_noalloc: at most " + std::to_string(kMaxZTerms) + " terms, got " +
                                         std::to_string(nterms));
    ZTerms z;
    std::memset(&z, 0, sizeof(z));
    z.nterms = nterms;
    for (int k = 0; k < nterms; ++k) {
        if (a[k] < 0 || a[k] >= n_qubits || b[k] >= n_qubits || b[k] == a[k])
            return set_error(LLG_EINVAL, "expect_zz_noalloc: term " + std::to_string(k) + " has a bad qubit");
        if (!std::isfinite(coeff[k])) return set_error(LLG_EINVAL, "expect_zz_noalloc: non-finite coefficient");
        int c = -1;
        for (int j = 0; j < z.nclass; ++j)
            if (z.coef[j] == coeff[k]) c = j;
        if (c < 0) {
            if (z.nclass == kMaxZClasses)
                return set_error(LLG_EINVAL, "expect_zz_noalloc: at most " + std::to_string(kMaxZClasses) +
                                                 " distinct coefficients");
            c = z.nclass++;
            z.coef[c] = coeff[k];
        }
        z.a[k] = a[k];
        z.b[k] = b[k] < 0 ? -1 : b[k];
        z.cls[k] = c;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(LLG_ECUDA, std::string("expect_zz_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    e = cudaPeekAtLastError();
    if (e != cudaSuccess)
        return set_error(LLG_ECUDA, std::string("expect_zz_noalloc: a CUDA error is pending from earlier work: ") +
                                        cudaGetErrorString(e));
    if (!device_reachable(d_amps, dev) || !device_reachable(d_out, dev))
        return set_error(LLG_EINVAL, "expect_zz_noalloc: d_amps and d_out must be device memory of the current device "
                                     "(or managed memory)");
    double* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (precision) {
        case LLG_F64: return launch<PolF64>(d_amps, n_qubits, z, scratch, d_out, s);
        case LLG_F32: return launch<PolF32>(d_amps, n_qubits, z, scratch, d_out, s);
        default: return launch<PolDF64>(d_amps, n_qubits, z, scratch, d_out, s);
    }
}
